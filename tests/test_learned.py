"""Learned warm start: the CPU reference network (finite differences), the host-side
feature / target / DOF mapping (CPU), and the library's BF16 forward and backward
kernels against the CPU reference (GPU)."""
from __future__ import annotations

import math

import numpy as np
import pytest

import oracle
from oracle import learned as ref
from movfem_gb300 import learn


def test_reference_gradient_matches_finite_differences():
    rng = np.random.Generator(np.random.PCG64(0))
    cin, width, cout, dil = 3, 4, 5, [1, 2]
    _, n = ref.layers(cin, width, cout, dil)
    p = rng.normal(size=n) * 0.3
    x = rng.normal(size=(4, 3, 5, cin))
    t = rng.normal(size=(4, 3, 5, cout))
    _, g = ref.loss_and_grad(p, x, t, cin, width, cout, dil, rounding=False)
    h = 1e-6
    idx = rng.choice(n, 60, replace=False)
    for i in idx:
        e = np.zeros(n)
        e[i] = h
        fd = (ref.loss_and_grad(p + e, x, t, cin, width, cout, dil, False)[0] -
              ref.loss_and_grad(p - e, x, t, cin, width, cout, dil, False)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-7 * max(1.0, np.abs(g).max())


def test_bf16_rounding_ties_to_even():
    v = np.array([1.0, 1.00390625, 1.005859375, 1.01171875, -3.14159], dtype=np.float32)
    assert list(ref.bf16(v)) == [1.0, 1.0, 1.0078125, 1.015625, -3.140625]


def test_targets_and_dof_mapping_round_trip():
    """Every cell carries the exact DOF values of its edges, so averaging them back onto
    the DOFs returns the (normalised) field exactly."""
    m = learn.random_block_model(7, ncx=5, ncz=4, n_air=2)
    gne, nne = oracle.Oracle(m).numbering()
    rng = np.random.Generator(np.random.PCG64(1))
    x = rng.normal(size=(2, nne)) + 1j * rng.normal(size=(2, nne))
    t, scale = learn.cell_targets(m, gne, x)
    assert t.shape == (m.nx, m.ny, m.nz, 4 * m.me)
    back = learn.dof_field(gne, nne, t.astype(np.float64))
    np.testing.assert_allclose(back * scale[:, None], x, rtol=1e-6, atol=1e-6 * np.abs(x).max())


def test_features_flag_air_and_depth():
    m = learn.random_block_model(3, ncx=4, ncz=3, n_air=2)
    f = float(m.freqs[0])
    F = learn.features(m, f)
    assert F.shape == (m.nx, m.ny, m.nz, learn.CIN)
    assert np.all(F[:, :, -2:, 1] == 1) and np.all(F[:, :, :-2, 1] == 0)
    assert np.all(F[:, :, :-2, 2] > 0) and np.all(F[:, :, -2:, 2] < 0)
    assert np.allclose(F[..., 3], math.log10(f) / 2)


@pytest.mark.gpu
def test_gpu_kernels_match_reference_forward_and_gradients():
    rng = np.random.Generator(np.random.PCG64(5))
    cin, width, cout, dil = learn.CIN, 8, 12, (1, 2)
    net = learn.WarmStartNet(me=cout // 4, width=width, dilations=dil, seed=3)
    p = net.params()
    x = rng.normal(size=(6, 5, 7, cin)).astype(np.float32)
    t = rng.normal(size=(6, 5, 7, cout)).astype(np.float32)
    out = net.forward(x)
    acts = ref.forward(p, x, cin, width, cout, list(dil))
    np.testing.assert_allclose(out, acts[-1], rtol=2e-3, atol=2e-3 * np.abs(acts[-1]).max())
    loss, g = net.gradients(x, t)
    rloss, rg = ref.loss_and_grad(p, x, t, cin, width, cout, list(dil))
    assert abs(loss - rloss) <= 1e-4 * rloss
    assert np.linalg.norm(g - rg) <= 1e-3 * np.linalg.norm(rg)
    # a training step moves the loss down on a fixed sample
    l0 = net.train_step(x, t, 1e-2)
    for _ in range(20):
        l1 = net.train_step(x, t, 1e-2)
    assert l1 < l0
