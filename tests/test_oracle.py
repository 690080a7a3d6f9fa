"""CPU tests of the oracle (known-answer tests; no GPU)."""
import math

import numpy as np
import pytest

import oracle
from movfem_gb300 import mesh as M
from tests import models


@pytest.mark.parametrize("mn", [8, 20, 27])
def test_shared_edges_identical(mn):
    # the reference's own self-check vf_check_sharing (v_fem.f90:556-863) on a box mesh
    o = oracle.Oracle(models.box(mn))
    assert o.check_sharing() < 1e-12


@pytest.mark.parametrize("mn", [8, 20, 27])
@pytest.mark.parametrize("dirichlet", [1, 0])
def test_slot_map_one_slot_per_entry(mn, dirichlet):
    m = models.box(mn, dirichlet=dirichlet, nextd=1 if not dirichlet else 0)
    o = oracle.Oracle(m)
    gne, nne = o.numbering()
    nz, nnze = o.slot_map()
    ia, ja = o.coo_coords()  # raises if a slot gets two coordinates
    pairs = set(zip(ia.tolist(), ja.tolist()))
    assert len(pairs) == nnze
    # the slots cover exactly the element couplings
    ref = set()
    for e in range(m.ne):
        g = gne[:, e]
        g = g[g > 0]
        for a in g:
            for b in g:
                ref.add((int(a), int(b)))
    assert pairs == ref
    assert nne == gne.max()


def test_linear_counts_match_plain_workload():
    m = M.plain_linear_block()
    gne, nne = oracle.Oracle(m).numbering()
    # 21x21x31 node grid: 39,270 edges, the 32,870 interior ones free
    assert nne == 32870
    assert (gne < 0).any() and set(np.unique(gne[gne < 0])) == {-1, -2, -3, -4, -5, -6}


def test_linear_cube_mass_matrix_exact():
    # unit-conductivity cube of side h: Nedelec mass entries h/9 * [4, 2, 1] for the
    # same edge / parallel edges sharing a face / opposite edges
    h = 100.0
    m = M.build_mesh(nodes_per_elem=8, ncx=1, ncy=1, ncz_earth=1, dx=h, dy=h, dz=h, n_air=1, dz_air=h, nextd=0,
                     sigma_fn=lambda x, y, d: 1.0 + 0 * x, omega1=1.0)
    o = oracle.Oracle(m)
    K, Mm, b, _ = o.element(0, 1.0)
    # edges 6,7,8,5 (dir 1) are the x-parallel edges: 5=(node4), 6=(8), 7=(3), 8=(7)
    i5, i6, i7, i8 = 4, 5, 6, 7
    assert Mm[i5, i5] == pytest.approx(4 * h / 9, rel=1e-7)
    assert Mm[i5, i6] == pytest.approx(2 * h / 9, rel=1e-7)   # nodes 4 and 8 share the x-z face
    assert Mm[i5, i7] == pytest.approx(2 * h / 9, rel=1e-7)   # nodes 4 and 3 share the x-y face
    assert Mm[i5, i8] == pytest.approx(1 * h / 9, rel=1e-7)   # diagonal
    assert np.allclose(K, K.T, rtol=0, atol=1e-12 * abs(K).max())
    assert np.allclose(Mm, Mm.T, rtol=0, atol=1e-12 * abs(Mm).max())


@pytest.mark.parametrize("mn", [8, 20, 27])
def test_curl_curl_null_space_dimension(mn):
    # exact sequence: the element curl-curl kernel is the gradient space of the
    # 8/20/27-node scalar element (dimension nodes - 1)
    m = models.box(mn, n=(1, 1, 1), n_air=1)
    K, Mm, b, _ = oracle.Oracle(m).element(0, 1.0)
    ev = np.linalg.eigvalsh(0.5 * (K + K.T))
    assert (np.abs(ev) < 1e-9 * np.abs(ev).max()).sum() == mn - 1
    assert np.linalg.eigvalsh(0.5 * (Mm + Mm.T)).min() > 0


def test_uniform_air_impedance():
    # no conductivity: the secondary field vanishes and Z at the surface comes from
    # the primary air field E = -i w b0 z (pol 1), with H = -(i/w) mu0^-1 curl E formed
    # from the nodal E as the reference does: Hy = -b0/mu0, so Zxy = +i w mu0 z_s
    m = models.box(8, n=(3, 3, 2))
    m.sigma[:] = 0.0
    m.sigma[:, [0, 3, 5]] = 1j * M.f32(M.EPS0 * 2 * math.pi * 0.5)
    o = oracle.Oracle(m)
    w = 2 * math.pi * 0.5
    x = np.zeros((2, o.numbering()[1]), dtype=np.complex128)
    E, H, Z, rho, phi = o.receivers(w, x)
    zs = m.ztop
    expect = 1j * w * 4 * math.pi * 1e-7 * zs
    assert np.allclose(Z[:, 1], expect, rtol=1e-6)
    assert np.allclose(Z[:, 2], -expect, rtol=1e-6)
    assert np.allclose(Z[:, 0], 0, atol=1e-12 * abs(expect))


def test_gpml_lag_flags():
    # element (ie,je,ke) is assembled with the zone flags of the element before it in
    # loop order (MoVFEM_3DMT.f90:200-206); the first element of the first frequency
    # has none, from the second frequency on it inherits the last element's flags
    m = models.box(8, n=(4, 4, 3), dirichlet=0, nextd=2)
    o = oracle.Oracle(m)
    _, _, _, fl0 = o.element(0, 1.0, ifreq=0)
    _, _, _, fl1 = o.element(0, 1.0, ifreq=1)
    assert list(fl0) == [0, 0, 0]
    assert list(fl1) == [1, 1, 1]
    # bottom element of the second column takes the top flag of the first column
    e = 1 * m.nz + 0
    _, _, _, fl = o.element(e, 1.0)
    assert fl[2] == 1
    o2 = oracle.Oracle(m, quirks=oracle.Q_ALL & ~oracle.Q_GPML_LAG)
    _, _, _, fl = o2.element(e, 1.0)
    assert fl[2] == 0


def test_golden_fixtures():
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "oracle_small.npz")
    g = np.load(path)
    from tests.golden.make_golden import compute
    cur = compute()
    for k in g.files:
        if g[k].dtype.kind in "iu" or k.startswith("map_"):  # integer work and the model mapping: bit-exact
            assert np.array_equal(g[k], cur[k]), k
        else:
            assert np.allclose(g[k], cur[k], rtol=1e-12, atol=1e-300), k


def test_rem_zeros_drops_exact_zeros_only():
    """find_zeros / rem_zeros (global_assembly.f90:123-150): 0 + 0i and -0.0 are dropped,
    tiny and purely imaginary values are kept, the order of the rest is unchanged."""
    a = np.array([1 + 1j, 0j, complex(-0.0, 0.0), 1e-300 + 0j, 0 + 2j, complex(0.0, -0.0), 3 + 0j])
    ia = np.arange(1, 8, dtype=np.int32)
    ja = ia[::-1].copy()
    ka, kb, kv, n = oracle.rem_zeros(ia, ja, a)
    assert n == 3
    assert list(ka) == [1, 4, 5, 7] and list(kb) == [7, 4, 3, 1]
    assert np.array_equal(kv, a[[0, 3, 4, 6]])
