"""Time the model mapping (nodal sigma / mu from an inner geomodel) on the GPU.

  python -m movfem_gb300.profile_map [--cells N] [--nz NZ] [--order 27] [--reps K]

Builds a grid of N x N x NZ core cells at 25 m (8 padding cells per side, 10 air
cells, Gaussian-sum topography up to +-300 m) and an inner geomodel of one point per
core cell with a 6-component sigma, then calls ``mvf_map_model`` ``reps`` times.
Prints one JSON line with the sizes and the kernels' device time per call.  Meant to
be run alone under ncu on a case smaller than the benchmark's.
"""
from __future__ import annotations

import argparse
import json
import math

import numpy as np

from . import api
from . import mesh as M


def grid_and_model(cells: int, nz: int, order: int = 27, seed: int = 20261205):
    rng = np.random.Generator(np.random.PCG64(seed))
    d = 25.0
    L = cells * d
    g = [(rng.uniform(0, L), rng.uniform(0, L), rng.uniform(-300, 300), rng.uniform(300, 1500)) for _ in range(5)]

    def topo(x, y):
        h = np.zeros_like(x, dtype=np.float64)
        for cx, cy, a, w in g:
            h = h + a * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * w * w))
        return np.clip(h, -300.0, 300.0)

    m = M.build_mesh(nodes_per_elem=order, ncx=cells, ncy=cells, ncz_earth=nz, dx=d, dy=d, dz=d, n_air=10,
                     dz_air=2 * d, nextd=8, sigma_fn=lambda x, y, dep: 0.01 + 0 * x, omega1=2 * math.pi * 1e-3,
                     topo_fn=topo, dirichlet=0, gpml_sch=1)
    gm = M.synthetic_geomodel(seed + 1, m, spacing=d, depth=nz * d, anisotropic=True, relief=0.0, topo_fn=topo)
    return m, gm


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=48)
    ap.add_argument("--nz", type=int, default=32)
    ap.add_argument("--order", type=int, default=27)
    ap.add_argument("--reps", type=int, default=1)
    a = ap.parse_args()
    m, gm = grid_and_model(a.cells, a.nz, a.order)
    w = 2 * math.pi * 1e-3
    secs = []
    for _ in range(a.reps):
        _, _, s = api.map_model(m, gm, w, device=0, timed=True)
        secs.append(s)
    print(json.dumps({"npt": int(m.npt), "model_points": int(gm.zm.size), "order": a.order,
                      "ms_per_call": [round(s * 1e3, 3) for s in secs],
                      "nodes_per_s": m.npt / min(secs)}))


if __name__ == "__main__":
    main()
