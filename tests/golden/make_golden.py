"""Regenerate tests/golden/oracle_small.npz: oracle outputs on small seeded models.

The reference itself cannot run here (Fortran + MUMPS, no compiler), so these
fixtures pin the oracle's own outputs against later changes; the numbering and slot
counts they hold were checked against the structural invariants in test_oracle.py.
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
    return out


if __name__ == "__main__":
    path = os.path.join(os.path.dirname(__file__), "oracle_small.npz")
    np.savez_compressed(path, **compute())
    print("wrote", path, os.path.getsize(path), "bytes")
