"""GPU parity tests: the CUDA library (through its C-ABI) against the oracle.

Integer outputs (DOF numbering, boundary flags, CSR pattern) must be bit-exact.
Element and global matrix values are FP64 on both sides: relative error <= 1e-10 of
the largest entry.  Solutions: relative FP64 residual <= 1e-10 and impedance
||Z - Z_oracle||_F / ||Z_oracle||_F <= 1e-6 per receiver against the oracle's direct
solve.
"""
import math

import numpy as np
import pytest

import oracle
from movfem_gb300 import api
from movfem_gb300 import mesh as M
from tests import models

pytestmark = pytest.mark.gpu

ORDERS = [8, 20, 27]


def _problem(m):
    return api.MTProblem(m)


@pytest.mark.parametrize("mn", ORDERS)
@pytest.mark.parametrize("dirichlet", [1, 0])
def test_numbering_bit_exact(mn, dirichlet):
    m = models.box(mn, n=(3, 4, 2), dirichlet=dirichlet, nextd=0 if dirichlet else 1)
    p = _problem(m)
    gne_ref, nne_ref = oracle.Oracle(m).numbering()
    gne = p.numbering()
    assert p.nne == nne_ref
    assert np.array_equal(gne, gne_ref)


@pytest.mark.parametrize("mn", ORDERS)
@pytest.mark.parametrize("dirichlet", [1, 0])
def test_pattern_equals_reference_coo(mn, dirichlet):
    m = models.box(mn, n=(3, 3, 3), dirichlet=dirichlet, nextd=0 if dirichlet else 1)
    p = _problem(m)
    p.assemble([2 * math.pi * 0.5])
    ia, ja, _ = p.export_coo(0)
    o = oracle.Oracle(m)
    ria, rja = o.coo_coords()
    low = ria >= rja
    ref = set(zip(ria[low].tolist(), rja[low].tolist()))
    got = list(zip(ia.tolist(), ja.tolist()))
    assert len(got) == len(ref) == p.nnz_lower
    assert set(got) == ref
    # row-major order
    assert all(np.diff(ia.astype(np.int64) * (p.nne + 1) + ja) > 0)
    assert p.nnz == 2 * p.nnz_lower - p.nne


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("mn", ORDERS)
@pytest.mark.parametrize("kind", ["dirichlet", "dirichlet-aniso", "topo", "gpml-fang", "gpml-zhou", "mu-tensor"])
def test_element_matrices(mn, kind):
    if kind == "topo":
        m = models.topo(mn)
    elif kind.startswith("gpml"):
        m = models.box(mn, n=(3, 3, 2), dirichlet=0, nextd=1, gpml_sch=0 if kind.endswith("fang") else 1, seed=3)
    elif kind == "mu-tensor":
        # mu != mu0: a full SPD permeability tensor per node exercises mu^-1 in the
        # curl-curl integrand and the curl source of the primary H field
        # (problem.f90:376-457, pe_modelcurl / pe_dmodel_pfield)
        m = models.box(mn, seed=9)
        rng = np.random.Generator(np.random.PCG64(12))
        mu0 = 4e-7 * math.pi
        rel = np.zeros((m.npt, 6))
        rel[:, [0, 3, 5]] = 1.0 + rng.uniform(0.0, 0.5, (m.npt, 3))
        rel[:, [1, 2, 4]] = rng.uniform(-0.05, 0.05, (m.npt, 3))
        m.mu = rel * mu0
    else:
        m = models.box(mn, aniso=kind.endswith("aniso"), seed=4)
    w = 2 * math.pi * np.array([0.5, 3.0])
    p = _problem(m)
    p.assemble(w, ifreq0=0)
    o = oracle.Oracle(m)
    ne = m.ne
    for f in range(2):
        K, Mm, b = p.element_matrices(0, ne, f)
        for e in range(ne):
            Kr, Mr, br, _ = o.element(e, w[f], ifreq=f)
            assert _rel(K[e], Kr) < 1e-10, (e, f)
            assert _rel(Mm[e], Mr) < 1e-10, (e, f)
            assert _rel(b[e], br) < 1e-10, (e, f)


@pytest.mark.parametrize("mn", ORDERS)
@pytest.mark.parametrize("dirichlet", [1, 0])
def test_assembled_system(mn, dirichlet):
    m = models.box(mn, n=(3, 3, 2), dirichlet=dirichlet, nextd=0 if dirichlet else 1, seed=5)
    w = 2 * math.pi * np.array([0.5, 3.0])
    p = _problem(m)
    p.assemble(w)
    o = oracle.Oracle(m)
    for f in range(2):
        ia, ja, a = p.export_coo(f)
        ra, rrhs = o.assemble(w[f], ifreq=f)
        ria, rja = o.coo_coords()
        low = ria >= rja
        order = np.lexsort((rja[low], ria[low]))
        ref = ra[low][order]
        assert np.array_equal(ia, ria[low][order]) and np.array_equal(ja, rja[low][order])
        assert _rel(a, ref) < 1e-10
        assert _rel(p.export_rhs(f), rrhs) < 1e-10


@pytest.mark.parametrize("mn", ORDERS)
def test_zero_drop(mn):
    """The export with exact zeros left out (find_zeros / rem_zeros) keeps the order of
    the full export and drops exactly its 0 + 0i entries; against the oracle's dropped set
    the two may differ only on entries that are cancellation noise (|a| <= 1e-14 max|a|),
    which two summation orders can round to zero or not."""
    m = models.box(mn, n=(3, 3, 2), seed=5)
    w = 2 * math.pi * 0.5
    p = _problem(m)
    p.assemble([w])
    ia, ja, a = p.export_coo(0)
    ka, kb, kv = p.export_coo(0, drop_zeros=True)
    zero = a == 0
    assert p.zeros_dropped == int(zero.sum()) and kv.size + p.zeros_dropped == a.size
    assert np.array_equal(ka, ia[~zero]) and np.array_equal(kb, ja[~zero]) and np.array_equal(kv, a[~zero])
    o = oracle.Oracle(m)
    ra, _ = o.assemble(w)
    ria, rja = o.coo_coords()
    low = ria >= rja
    order = np.lexsort((rja[low], ria[low]))
    ref = ra[low][order]
    _, _, _, nref = oracle.rem_zeros(ria[low][order], rja[low][order], ref)
    differ = zero != (ref == 0)
    assert np.all(np.abs(np.where(zero, ref, a)[differ]) <= 1e-14 * np.abs(ref).max())


@pytest.mark.parametrize("mn", ORDERS)
def test_spmv_matches_cpu_product(mn):
    m = models.box(mn, n=(3, 3, 2), seed=6)
    w = 2 * math.pi * 0.5
    p = _problem(m)
    p.assemble([w])
    A, _ = oracle.Oracle(m).matrix(w)
    rng = np.random.Generator(np.random.PCG64(7))
    x = rng.normal(size=(2, p.nne)) + 1j * rng.normal(size=(2, p.nne))
    y = p.spmv(0, x)
    ref = np.stack([A @ x[0], A @ x[1]])
    assert _rel(y, ref) < 1e-12


@pytest.mark.parametrize("mn", [8, 20])
def test_every_spmm_variant_matches_cpu_product(mn):
    """Each autotuner candidate, FP64 and FP32, every batch width it accepts, against
    the oracle's matrix: FP64 to 1e-12, FP32 (complex64 K, M and vectors) to 2e-6 of
    |A||x| row-wise."""
    m = models.box(mn, n=(3, 3, 2), seed=6)
    w = 2 * math.pi * 0.5
    p = _problem(m)
    p.assemble([w])
    A, _ = oracle.Oracle(m).matrix(w)
    absA = abs(A)
    rng = np.random.Generator(np.random.PCG64(8))
    for R in (1, 2, 4, 8, 16, 32):
        x = rng.normal(size=(p.nne, R)) + 1j * rng.normal(size=(p.nne, R))
        ref = A @ x
        scale = absA @ np.abs(x)
        for v in api.SPMM_VARIANTS:
            if (v == 1 and R > 4) or (v >= 2 and R > 16):
                continue
            y64 = p.spmm_variant(0, v, True, x)
            assert _rel(y64, ref) < 1e-12, (R, api.SPMM_VARIANTS[v])
            y32 = p.spmm_variant(0, v, False, x)
            assert np.max(np.abs(y32 - ref) / scale) < 2e-6, (R, api.SPMM_VARIANTS[v])
        if True:
            # the float-float operator (FP32 halves of K, M and x; about 44 bits), in
            # passes of 8 right-hand sides above R = 8
            yff = p.spmm_variant(0, 6, True, x)
            assert np.max(np.abs(yff - ref) / scale) < 1e-11, R
    assert p.spmm_tuning() == "" or "R=" in p.spmm_tuning()


def _c1_small():
    return M.plain_linear_block(ncells=8, d=250.0, n_air=4, dz_air=500.0, nrx=3)


@pytest.mark.parametrize("mode", [api.MODE_MIXED, api.MODE_FP64])
def test_solve_and_impedance_linear(mode):
    m = _c1_small()
    w = 2 * math.pi * 1.0
    o = oracle.Oracle(m)
    xd, A, rhs = o.solve_direct(w)
    Zd = o.receivers(w, xd)[2]
    p = _problem(m)
    p.assemble([w])
    x, st = p.solve(tol=1e-10, mode=mode, max_iters=4000)
    assert st["rel_residual"] <= 1e-10
    res = max(np.linalg.norm(rhs[k] - A @ x[0, k]) / np.linalg.norm(rhs[k]) for k in range(2))
    assert res <= 1e-9
    Z, rho, phi = p.impedance()
    err = np.linalg.norm(Z[0] - Zd, axis=1) / np.linalg.norm(Zd, axis=1)
    assert err.max() <= 1e-6


def test_impedance_kernel_matches_oracle_on_same_solution():
    # E, H, Z, rho, phi evaluated in FP64 on the GPU from the GPU solution and by the
    # oracle from the same solution vector
    m = _c1_small()
    w = 2 * math.pi * 1.0
    p = _problem(m)
    p.assemble([w])
    x, _ = p.solve(tol=1e-10)
    Z, rho, phi, E, H = p.impedance(with_fields=True)
    Er, Hr, Zr, rhor, phir = oracle.Oracle(m).receivers(w, x[0])
    assert _rel(E[0], Er) < 1e-11
    assert _rel(H[0], Hr) < 1e-11
    assert _rel(Z[0], Zr) < 1e-11
    assert np.allclose(rho[0], rhor, rtol=1e-11, atol=0)
    assert np.allclose(phi[0], phir, rtol=1e-11, atol=1e-12)


def test_multi_frequency_batch_matches_single():
    # three frequencies batched as six right-hand sides sharing K and M.  Away from the
    # grid-time frequency the right-hand side has a component in the air-gradient
    # kernel (update_sigma, geometry.f90:144-153), which bounds the residual from below:
    # the solver stops at that floor and the impedance still matches the direct solve.
    m = _c1_small()
    w = 2 * math.pi * np.array([0.1, 1.0, 10.0])
    sig = np.stack([m.sigma_at(x) for x in w])
    p = _problem(m)
    p.assemble(w, sigma_f=sig)
    xb, st = p.solve(tol=1e-10)
    assert st["rel_residual"] <= 1e-10 or (st["stagnated"] and st["rel_residual"] <= 1e-6)
    Z = p.impedance()[0]
    o = oracle.Oracle(m)
    for f in range(3):
        o.set_sigma(sig[f])
        xd, A, rhs = o.solve_direct(w[f], ifreq=f)
        assert _rel(p.export_rhs(f), rhs) < 1e-10
        Zd = o.receivers(w[f], xd)[2]
        err = np.linalg.norm(Z[f] - Zd, axis=1) / np.linalg.norm(Zd, axis=1)
        assert err.max() <= 1e-6


def test_errors_are_reported():
    m = _c1_small()
    m.mu[5] = 0.0
    with pytest.raises(api.MVFError) as e:
        _problem(m)
    assert e.value.code == api.E_SINGULAR
    m = _c1_small()
    p = _problem(m)
    with pytest.raises(api.MVFError) as e:
        p.solve()
    assert e.value.code == api.E_STATE or isinstance(e.value, api.MVFError)


def _primary_model(m, inimod):
    m.inimod = inimod
    if inimod == 2:
        m.h_sigma = 0.02
    else:
        m.l_sigma = np.array([0.05, 0.5, 0.01])
        m.l_dz = np.array([90.0, 150.0])
    return m


@pytest.mark.parametrize("mn", [8, 20])
@pytest.mark.parametrize("inimod", [2, 3])
def test_dirichlet_primary_models_assembly_and_receivers(mn, inimod):
    """Dirichlet half-space (2) and layered (3) boundary values: the lift of the
    prescribed boundary DOFs into b (local_vfem) and their use in the receivers'
    nodal E (get_er), against the oracle."""
    m = _primary_model(models.box(mn, n=(3, 3, 2), seed=9), inimod)
    w = 2 * math.pi * np.array([0.5, 3.0])
    p = _problem(m)
    p.assemble(w)
    o = oracle.Oracle(m)
    for f in range(2):
        _, rrhs = o.assemble(w[f], ifreq=f)
        assert np.abs(rrhs).max() > 0
        assert _rel(p.export_rhs(f), rrhs) < 1e-10
    x, _ = p.solve(tol=1e-10, raise_noconv=False)
    Z, rho, phi, E, H = p.impedance(with_fields=True)
    for f in range(2):
        Er, Hr, Zr, _, _ = o.receivers(w[f], x[f])
        assert _rel(E[f], Er) < 1e-11
        assert _rel(H[f], Hr) < 1e-11
        assert _rel(Z[f], Zr) < 1e-11


@pytest.mark.parametrize("mn", [8, 20])
@pytest.mark.parametrize("inimod", [1, 3])
def test_full_volume_node_fields(mn, inimod):
    """E, H, Z, rho, phi at every node (node_solution + z_rho_phi) from the GPU solution,
    against the oracle on the same solution vector."""
    m = models.box(mn, n=(3, 3, 2), seed=10)
    if inimod != 1:
        _primary_model(m, inimod)
    w = 2 * math.pi * np.array([0.5, 3.0])
    p = _problem(m)
    p.assemble(w)
    x, _ = p.solve(tol=1e-10, raise_noconv=False)
    E, H, Z, rho, phi = p.node_fields()
    o = oracle.Oracle(m)
    for f in range(2):
        Er, Hr, Zr, rr, pr = o.node_fields(w[f], x[f])
        assert _rel(E[f], Er) < 1e-11
        assert _rel(H[f], Hr) < 1e-11
        assert _rel(Z[f], Zr) < 1e-9
        np.testing.assert_allclose(rho[f], rr, rtol=1e-9, atol=0)
        # phase = atan(Im Z / Re Z): where Re Z is at rounding level relative to |Z| its
        # sign (and the phase's +-90) is noise on both sides
        solid = np.abs(Zr.real) > 1e-9 * np.abs(Zr)
        np.testing.assert_allclose(phi[f][solid], pr[solid], rtol=1e-9, atol=1e-9)
        np.testing.assert_allclose(np.abs(phi[f][~solid]), np.abs(pr[~solid]), rtol=1e-9, atol=1e-9)


def test_solve_many_matches_individual_solves():
    """Uneven models solved concurrently (mvf_solve_many) give the impedances of the
    same models solved one by one."""
    models_ = [M.plain_linear_block(ncells=n, d=2000.0 / n, n_air=max(2, n // 3), dz_air=6000.0 / n, nrx=3)
               for n in (6, 8, 10, 7)]
    w = 2 * math.pi * 1.0
    single, batch = [], []
    for m in models_:
        p = _problem(m)
        p.assemble([w])
        p.solve(tol=1e-10)
        single.append(p.impedance()[0])
        q = _problem(m)
        q.assemble([w])
        batch.append(q)
    stats = api.solve_many(batch, tol=1e-10, nthreads=3)
    for s, q, z in zip(stats, batch, single):
        assert s["rel_residual"] <= 1e-10
        zb = q.impedance()[0]
        assert _rel(zb, z) < 1e-7


def test_patch_preconditioner_float_float_matches_fp64():
    """The one-level vertex-patch preconditioner in float-float arithmetic on the FP32
    pipe follows the FP64 one: same iteration budget, residuals within 2x, impedances
    within 1e-5 of each other."""
    m = models.box(20, n=(4, 4, 3), seed=11)
    w = 2 * math.pi * np.array([0.5])
    out = {}
    for prec in (1, 2):
        p = _problem(m)
        p.set_preconditioner(1)
        p.set_solver(patch_precision=prec)
        p.assemble(w)
        st = p.solve_device(tol=1e-10, max_iters=120)
        assert p.patch_arithmetic() == prec
        out[prec] = (st["rel_residual"], p.impedance()[0])
    r64, z64 = out[1]
    rff, zff = out[2]
    assert rff <= 2.0 * r64 + 1e-12
    assert _rel(zff, z64) < 1e-5
