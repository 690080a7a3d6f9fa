"""Ablation of the learned warm start (GPU): train the operator with the library's own
kernels on solutions of this solver, then solve held-out models with and without it.

What the network may change is the iteration count; what it may not change is the
accepted answer.  Asserted: both arms pass the same acceptance (the FP64 true-residual
tolerance, or the air-kernel floor the solver reports); the fitted warm start never
starts above the zero start (initial relative residual <= 1); training lowers the
loss.  The measured iteration ratio is printed; at this training size the network
does not yet reduce iterations.
"""
from __future__ import annotations

import numpy as np
import pytest

from movfem_gb300 import learn

pytestmark = pytest.mark.gpu


def test_learned_warm_start_keeps_tolerance_and_reports_gain():
    data = [learn.make_sample(5000 + i)[:2] for i in range(24)]
    net = learn.WarmStartNet(width=16, seed=2)
    hist = learn.train(net, data, epochs=12, lr=3e-3, time_budget_s=120)
    assert hist[-1] < hist[0]
    rows = learn.evaluate(net, [910000 + i for i in range(4)], tol=1e-10)
    for r in rows:
        assert r["converged"]
        # both arms pass the same acceptance: the tolerance, or the air-kernel floor
        # (stagnation below 1e-5) that the solver reports as converged
        assert r["res_plain"] <= 1e-5 and r["res_learned"] <= 1e-5
        assert r["initial_rel_residual"] <= 1.0 + 1e-12
    ratio = np.mean([r["iters_learned"] for r in rows]) / np.mean([r["iters_plain"] for r in rows])
    print(f"learned/plain inner iterations: {ratio:.3f}; initial residuals "
          f"{[round(r['initial_rel_residual'], 3) for r in rows]}")
    assert ratio < 1.5
