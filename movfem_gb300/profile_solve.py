"""Run one solve of a layered-earth model, for timing and for profiling the solver's
kernels (the vertex-patch preconditioner of the 36/54-DOF elements in particular).

  python -m movfem_gb300.profile_solve [--nodes-per-elem 20] [--cells 16] [--freqs 1]
                                       [--iters 20] [--mode 0] [--gpml]

Builds ``mesh.layered_blocks`` with ``cells`` x ``cells`` x ``cells*3/4`` earth cells
at 50 m (2 padding cells, 4 air cells), assembles, and runs the solver with an
iteration cap.  Prints one JSON line: sizes, iterations, residual, seconds.
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np

from . import api
from . import mesh as M


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--nodes-per-elem", type=int, default=20)
    ap.add_argument("--cells", type=int, default=16)
    ap.add_argument("--freqs", type=int, default=1)
    ap.add_argument("--iters", type=int, default=20)
    ap.add_argument("--mode", type=int, default=0)
    ap.add_argument("--gpml", action="store_true")
    a = ap.parse_args()
    m = M.layered_blocks(20261203, nodes_per_elem=a.nodes_per_elem, ncx=a.cells, ncy=a.cells,
                         ncz=max(2, a.cells * 3 // 4), d=50.0, nextd=2, n_air=4, dz_air=100.0, nfreq=a.freqs,
                         fmin=0.1, fmax=10.0, nrx=3, gpml_sch=0)
    m.dirichlet = 0 if a.gpml else 1
    p = api.MTProblem(m, device=0)
    w = 2 * math.pi * m.freqs
    p.assemble(w, sigma_f=np.stack([m.sigma_at(x) for x in w]))
    t0 = time.time()
    st = p.solve_device(tol=1e-10, mode=a.mode, max_iters=a.iters)
    dt = time.time() - t0
    print(json.dumps({"nodes_per_elem": a.nodes_per_elem, "nne": p.nne, "nnz": p.nnz, "freqs": a.freqs,
                      "inner_iters": st["inner_iters"], "rel_residual": st["rel_residual"], "seconds": dt}))


if __name__ == "__main__":
    main()
