"""Regenerate tests/golden/oracle_small.npz: oracle outputs on small seeded models.

The reference itself cannot run here (Fortran + MUMPS, no compiler), so these
fixtures pin the oracle's own outputs against later changes; the numbering and slot
counts they hold were checked against the structural invariants in test_oracle.py, and
the model-mapping outputs against the pure-Python restatement in test_model_map.py.
Run:  python -m tests.golden.make_golden
"""
import math
import os

import numpy as np

import oracle
from tests import models


def compute():
    out = {}
    for mn in (8, 20, 27):
        m = models.box(mn)
        o = oracle.Oracle(m)
        gne, nne = o.numbering()
        nz, nnze = o.slot_map()
        ia, ja = o.coo_coords()
        K, M, b, _ = o.element(3, 2 * math.pi * 0.5)
        out[f"gne{mn}"] = gne
        out[f"ia{mn}"] = ia
        out[f"ja{mn}"] = ja
        out[f"K{mn}"] = K
        out[f"M{mn}"] = M
        out[f"b{mn}"] = b
        mg = models.box(mn, dirichlet=0, nextd=1, seed=2)
        og = oracle.Oracle(mg)
        K, M, b, _ = og.element(5, 2 * math.pi * 3.0, ifreq=1)
        out[f"gpmlK{mn}"] = K
        out[f"gpmlM{mn}"] = M
        out[f"gpmlb{mn}"] = b
    m = models.box(8, n=(4, 4, 3))
    o = oracle.Oracle(m)
    w = 2 * math.pi * 0.5
    x, A, rhs = o.solve_direct(w)
    Z = o.receivers(w, x)[2]
    out["Z8"] = Z
    out["rhs8"] = rhs
    # model mapping (innermodel_gqg): small grids with seeded geomodels
    from movfem_gb300 import mesh as M
    for mn, aniso in ((8, False), (20, True)):
        g = M.build_mesh(nodes_per_elem=mn, ncx=3, ncy=3, ncz_earth=2, dx=100.0, dy=120.0, dz=80.0, n_air=1,
                         dz_air=150.0, nextd=1, sigma_fn=lambda x, y, d: 0.01 + 0 * x, omega1=2 * math.pi * 0.1,
                         dirichlet=0, topo_fn=lambda x, y: 20.0 * np.sin(x / 90.0))
        gm = M.synthetic_geomodel(7, g, spacing=60.0, depth=200.0, relief=10.0, anisotropic=aniso,
                                  mu_tensor=aniso)
        s, u = oracle.map_model(g, gm, 2 * math.pi * 0.1)
        out[f"map_sigma{mn}"] = s
        out[f"map_mu{mn}"] = u
    return out


if __name__ == "__main__":
    path = os.path.join(os.path.dirname(__file__), "oracle_small.npz")
    np.savez_compressed(path, **compute())
    print("wrote", path, os.path.getsize(path), "bytes")
