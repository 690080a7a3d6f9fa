"""CPU checks of the multilevel restatement (``oracle/multilevel.py``): the discrete
gradient of the 20/27-node spaces, and what limits the convergence of FGMRES with the
multilevel preconditioner on layered models with air.

Just above the earth's surface the quadratic interpolation of the nodal conductivity
(earth value at the surface nodes, 0 above) dips below zero: sigma(z) = sigma_e
zeta (zeta - 1) / 2 in the first air cells, down to -sigma_e / 8.  The true operator is
indefinite on the gradients there; the preconditioner's mass is made positive
semidefinite, which flips their sign.  An exact solve of those gradient modes with the
true operator (``surface_gradient=True``) removes the slow tail: these tests pin that
finding on a model where it shows within seconds.
"""
import math

import numpy as np
import pytest

import oracle
from oracle.multilevel import Multilevel, discrete_gradient
from movfem_gb300 import mesh as M
from tests import models


def _fgmres(A, prec, b, iters, restart=60):
    """Right-preconditioned GMRES; returns the relative residual after `iters` steps."""
    n = b.size
    x = np.zeros(n, complex)
    bn = np.linalg.norm(b)
    done = 0
    while done < iters:
        r = b - A @ x
        beta = np.linalg.norm(r)
        if beta / bn < 1e-13:
            break
        V = np.zeros((n, restart + 1), complex)
        Z = np.zeros((n, restart), complex)
        H = np.zeros((restart + 1, restart), complex)
        V[:, 0] = r / beta
        k = -1
        for k in range(min(restart, iters - done)):
            Z[:, k] = prec(V[:, k])
            w = A @ Z[:, k]
            for _ in range(2):
                for i in range(k + 1):
                    h = np.vdot(V[:, i], w)
                    H[i, k] += h
                    w -= h * V[:, i]
            H[k + 1, k] = np.linalg.norm(w)
            V[:, k + 1] = w / H[k + 1, k]
        e1 = np.zeros(k + 2, complex)
        e1[0] = beta
        y = np.linalg.lstsq(H[:k + 2, :k + 1], e1, rcond=None)[0]
        x = x + Z[:, :k + 1] @ y
        done += k + 1
    return np.linalg.norm(b - A @ x) / bn


@pytest.mark.parametrize("mn", [20, 27])
def test_discrete_gradient_is_in_the_curl_kernel(mn):
    m = models.box(mn, n=(3, 3, 2), seed=2)
    o = oracle.Oracle(m)
    gne, n = o.numbering()
    A, _ = o.matrix(2 * math.pi)
    K = A.real
    G = discrete_gradient(m, gne, n)
    assert G.nnz > 0
    assert abs(K @ G).max() <= 1e-12 * abs(K).max() * abs(G).max()


def test_surface_gradient_correction_removes_the_slow_tail():
    m = M.layered_blocks(20261203, nodes_per_elem=20, ncx=8, ncy=8, ncz=6, d=50.0, nextd=3, n_air=4,
                         dz_air=100.0, nfreq=1, fmin=1.0, fmax=1.0, nrx=4, gpml_sch=0)
    m.dirichlet = 1
    w = 2 * math.pi * 1.0
    ml = Multilevel(m, w, surface_gradient=True)
    b = ml.rhs[0]
    with_surface = _fgmres(ml.A_true, ml, b, 30)
    surface, ml.surface = ml.surface, None
    plain = _fgmres(ml.A_true, ml, b, 30)
    ml.surface = surface
    assert with_surface < 1e-8, with_surface
    assert plain > 1e-5, plain


@pytest.mark.parametrize("n,kl,ku,pivot", [(50, 3, 3, False), (400, 17, 17, True), (300, 5, 40, True),
                                            (1200, 90, 90, True)])
def test_band_lu_of_the_surface_correction(n, kl, ku, pivot):
    """The host band LU of mvf_surface.cu (partial pivoting, fill of kl extra rows)
    against a dense solve; indefinite matrices with small diagonals force row swaps."""
    from movfem_gb300 import api
    rng = np.random.Generator(np.random.PCG64(n + kl))
    a = rng.normal(size=(n, n))
    i, j = np.indices((n, n))
    a[(i - j > kl) | (j - i > ku)] = 0.0
    if not pivot:
        a[np.diag_indices(n)] += 2.0 * (kl + ku + 1)
    else:
        a[np.diag_indices(n)] *= 1e-3
    b = rng.normal(size=(n, 3))
    x = api.band_solve(a, b, kl, ku)
    ref = np.linalg.solve(a, b)
    assert np.abs(x - ref).max() <= 1e-8 * np.abs(ref).max()
