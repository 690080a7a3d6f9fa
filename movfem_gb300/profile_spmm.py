"""Time the batched K/M SpMM of one model on the GPU (the roofline kernel).

  python -m movfem_gb300.profile_spmm [--cells N] [--freqs F] [--reps K]

Builds a linear-element Dirichlet model of N^3 earth cells (plus N/3 air layers),
assembles F frequencies (2F right-hand sides share K and M) and times ``reps``
launches of the FP32 SpMM with CUDA events on the library's stream.  Prints one JSON
line with the size, the per-launch time and the algorithmic bandwidth.  Meant to be
run alone under ncu to capture the SpMM on a model whose matrix exceeds L2.
"""
from __future__ import annotations

import argparse
import json
import math

import numpy as np

from . import api
from . import mesh as M


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=60)
    ap.add_argument("--freqs", type=int, default=1)
    ap.add_argument("--reps", type=int, default=5)
    a = ap.parse_args()
    m = M.plain_linear_block(ncells=a.cells, d=2000.0 / a.cells, n_air=max(2, a.cells // 3),
                             dz_air=6000.0 / a.cells, nrx=2)
    p = api.MTProblem(m, device=0)
    w = 2 * math.pi * np.logspace(-1, 2, a.freqs)
    p.assemble(w)
    r = p.profile_spmm(0, reps=a.reps)
    print(json.dumps({"cells": a.cells, "nne": p.nne, "nnz": p.nnz, "rhs": 2 * a.freqs,
                      "us_per_launch": r["seconds_per_launch"] * 1e6, "bytes_per_launch": r["bytes_per_launch"],
                      "GBps": r["bytes_per_launch"] / r["seconds_per_launch"] / 1e9,
                      "tuning": p.spmm_tuning()}))


if __name__ == "__main__":
    main()
