"""Model mapping: nodal sigma / mu of the grid from the inner geomodel.

Reference: innermodel_gqg, min_dd_inner and assign_model (MoVFEM_3DMT/src/
geometry.f90:804-1085), called once by grid_3d (geometry.f90:106).  The C oracle
(``oracle.map_model``) restates them sequentially; here it is checked against a second,
pure-Python restatement written with the Fortran's 1-based loops, and the GPU kernel
(``mvf_map_model``) must match the oracle bit for bit on grids of all three element
orders, isotropic and full-tensor models, exact hits (points on grid nodes), distance
ties and duplicated points.
"""
import math

import numpy as np
import pytest

import oracle
from movfem_gb300 import mesh as M

EPS0 = 8.854187817e-12
MU0 = 4.0 * math.pi * 1.0e-7


def small_grid(order, nextd=2, topo=0.0, ncx=5, ncy=4, ncz=3):
    topo_fn = None
    if topo:
        def topo_fn(x, y):
            return topo * np.sin(x / 170.0) * np.cos(y / 230.0)
    return M.build_mesh(nodes_per_elem=order, ncx=ncx, ncy=ncy, ncz_earth=ncz, dx=100.0, dy=120.0, dz=80.0,
                        n_air=2, dz_air=150.0, nextd=nextd, sigma_fn=lambda x, y, d: 0.01 + 0 * x,
                        omega1=2 * math.pi * 0.1, dirichlet=0, topo_fn=topo_fn)


def python_map(m, gm, omega):
    """geometry.f90:804-1085 with the reference's 1-based loops (slow; small grids)."""
    o = m.nord - 1
    nord = o + 1
    nnx, nny, nnz = m.nnx, m.nny, m.nnz
    nyz = nny * nnz
    gnx, gny, gnz = m.nx + 1, m.ny + 1, m.nz + 1
    nextd = m.nextd
    nzl_top, nzl_air = m.nzl_top, m.nzl_air
    ieps = float(np.float32(EPS0 * omega))
    mx, my, mz = gm.zm.shape
    xm, ym, zm = list(gm.xm), list(gm.ym), list(gm.zm.reshape(-1))
    sig_in = gm.sigma.reshape(mx * my * mz, -1)
    isig = sig_in.shape[1]
    ijs = np.asarray(gm.ijsigma).reshape(-1, 2)
    sig = [[complex(-1.0, 0.0)] * 6 for _ in range(m.npt + 1)]  # 1-based
    mu = [[-1.0] * 6 for _ in range(m.npt + 1)]
    valued = [0] * (m.npt + 1)

    def assign(idd, p):  # assign_model; p 1-based
        if valued[idd]:
            return
        s = [0j] * 6
        if isig == 1:
            for c in (0, 3, 5):
                s[c] = complex(sig_in[p - 1, 0], 0.0) + complex(0.0, ieps)
        else:
            for c in range(isig):
                a, b = int(ijs[c, 0]), int(ijs[c, 1])
                s[(b if a == 1 else a + b) - 1] = complex(sig_in[p - 1, c], 0.0)
            for c in (0, 3, 5):
                s[c] = s[c] + complex(0.0, ieps)
        sig[idd] = s
        u = [0.0] * 6
        if gm.mu is None:
            for c in (0, 3, 5):
                u[c] = MU0 * 1.0
        elif gm.mu.reshape(mx * my * mz, -1).shape[1] == 1:
            for c in (0, 3, 5):
                u[c] = MU0 * gm.mu.reshape(-1)[p - 1]
        else:
            mu_in = gm.mu.reshape(mx * my * mz, -1)
            ijm = np.asarray(gm.ijmu).reshape(-1, 2)
            for c in range(mu_in.shape[1]):
                a, b = int(ijm[c, 0]), int(ijm[c, 1])
                u[(b if a == 1 else a + b) - 1] = MU0 * mu_in[p - 1, c]
        mu[idd] = u
        valued[idd] = 1

    for ie in range(nextd + 1, gnx - nextd - 1 + 1):
        for je in range(nextd + 1, gny - nextd - 1 + 1):
            for ke in range(nextd, gnz - nzl_top - nzl_air - 1 + 1):
                no = (ie - 1) * o * nyz + (je - 1) * o * nnz + (ke - 1) * o + 1
                for ii in range(1, nord + 1):
                    for jj in range(1, nord + 1):
                        for kk in range(1, nord + 1):
                            idd = no + (ii - 1) * nyz + (jj - 1) * nnz + (kk - 1)
                            x = m.xp[(ie - 1) * o + ii - 1]
                            y = m.yp[(je - 1) * o + jj - 1]
                            z = m.zp[idd - 1]
                            ddmin, best, hit = 1.0e20, -1, False
                            for im in range(1, mx + 1):
                                for jm in range(1, my + 1):
                                    for km in range(1, mz + 1):
                                        p = (im - 1) * my * mz + (jm - 1) * mz + km
                                        dd = math.sqrt((x - xm[im - 1]) ** 2 + (y - ym[jm - 1]) ** 2 +
                                                       (z - zm[p - 1]) ** 2)
                                        if dd <= 1.0e-5:
                                            assign(idd, p)
                                            hit = True
                                        elif dd < ddmin:
                                            ddmin, best = dd, p
                            if not hit:
                                assign(idd, best)
    E = nextd * o
    kmax = nnz - nzl_top * o - nzl_air * o

    def copy(idd, ip):
        if not valued[idd]:
            sig[idd] = list(sig[ip])
            mu[idd] = list(mu[ip])
            valued[idd] = 1

    for im in range(1, E + 1):
        for jm in range(E + 1, nny - E + 1):
            for km in range(E, kmax + 1):
                copy((im - 1) * nyz + (jm - 1) * nnz + km, E * nyz + (jm - 1) * nnz + km)
    for im in range(nnx - E + 1, nnx + 1):
        for jm in range(E + 1, nny - E + 1):
            for km in range(E, kmax + 1):
                copy((im - 1) * nyz + (jm - 1) * nnz + km, (nnx - E - 1) * nyz + (jm - 1) * nnz + km)
    for im in range(1, nnx + 1):
        for jm in range(1, E + 1):
            for km in range(E, kmax + 1):
                copy((im - 1) * nyz + (jm - 1) * nnz + km, (im - 1) * nyz + E * nnz + km)
    for im in range(1, nnx + 1):
        for jm in range(nny - E + 1, nny + 1):
            for km in range(E, kmax + 1):
                copy((im - 1) * nyz + (jm - 1) * nnz + km, (im - 1) * nyz + (nny - E - 1) * nnz + km)
    for im in range(1, nnx + 1):
        for jm in range(1, nny + 1):
            for km in range(1, E - 1 + 1):
                copy((im - 1) * nyz + (jm - 1) * nnz + km, (im - 1) * nyz + (jm - 1) * nnz + E)
    for im in range(1, nnx + 1):
        for jm in range(1, nny + 1):
            for km in range(kmax + 1, nnz + 1):
                idd = (im - 1) * nyz + (jm - 1) * nnz + km
                sig[idd] = [0j] * 6
                mu[idd] = [0.0] * 6
                for c in (0, 3, 5):
                    sig[idd][c] = complex(0.0, ieps)
                    mu[idd][c] = MU0
    for idd in range(2, m.npt + 1):  # node 1 would read before the array: left as it is
        for c in range(6):
            if sig[idd][c].real < 0:
                sig[idd][c] = sig[idd - 1][c]
            if mu[idd][c] < 0:
                mu[idd][c] = mu[idd - 1][c]
    return np.array(sig[1:], dtype=np.complex128), np.array(mu[1:])


CASES = [
    # (order, nextd, topo, model kwargs)
    (8, 2, 0.0, dict(spacing=90.0, depth=400.0)),
    (8, 1, 30.0, dict(spacing=70.0, depth=300.0, relief=25.0, anisotropic=True)),
    (20, 2, 0.0, dict(spacing=85.0, depth=350.0, anisotropic=True, mu_tensor=True)),
    (27, 2, 40.0, dict(spacing=60.0, depth=300.0, relief=10.0)),
    (20, 2, 0.0, dict(spacing=0.0, depth=0.0, on_nodes=True, node_stride=2)),
    (8, 2, 20.0, dict(spacing=80.0, depth=300.0, relief=15.0, mu_iso=True)),
]
IDS = ["linear-iso", "linear-aniso-topo-nextd1", "quadratic-aniso-mu-tensor", "lagrangian-iso-topo",
       "quadratic-points-on-nodes", "linear-iso-mu-topo"]


def _model(case, seed=3):
    order, nextd, topo, kw = case
    kw = dict(kw)
    mu_iso = kw.pop("mu_iso", False)
    m = small_grid(order, nextd=nextd, topo=topo)
    gm = M.synthetic_geomodel(seed, m, **kw)
    if mu_iso:  # in_imu = 1: one isotropic relative permeability per point
        rng = np.random.Generator(np.random.PCG64(seed))
        gm.mu = 1.0 + rng.uniform(0.0, 2.0, (gm.zm.size, 1))
        gm.ijmu = np.array([[1, 1]], dtype=np.int32)
    return m, gm


@pytest.mark.parametrize("case", CASES[:3] + CASES[4:], ids=IDS[:3] + IDS[4:])
def test_oracle_matches_python_restatement(case):
    m, gm = _model(case)
    w = 2 * math.pi * 0.1
    s_c, u_c = oracle.map_model(m, gm, w)
    s_p, u_p = python_map(m, gm, w)
    assert np.array_equal(s_c.view(np.float64), s_p.view(np.float64))
    assert np.array_equal(u_c, u_p)


def test_oracle_map_semantics():
    """Points on every node: each inner node takes its own point's value; the air is
    i*eps*omega (FP32-rounded) on the diagonal with mu0; the extension copies the
    last inner plane."""
    m = small_grid(8, nextd=2)
    gm = M.synthetic_geomodel(5, m, spacing=0.0, depth=0.0, on_nodes=True, node_stride=1)
    w = 2 * math.pi * 0.1
    s, u = oracle.map_model(m, gm, w)
    s = s.reshape(m.nnx, m.nny, m.nnz, 6)
    E = m.nextd
    ksurf = m.nnz - (m.nzl_top + m.nzl_air) - 1
    sig_pts = gm.sigma.reshape(gm.zm.shape)
    ieps = float(np.float32(EPS0 * w))
    inner = s[E:m.nnx - E, E:m.nny - E, E - 1:ksurf + 1, 0]
    assert np.array_equal(inner.real, sig_pts[:, :, E - 1:ksurf + 1])
    assert np.all(inner.imag == ieps)
    air = s[:, :, ksurf + 1:, :]
    assert np.all(air[..., [0, 3, 5]] == 1j * ieps) and np.all(air[..., [1, 2, 4]] == 0)
    assert np.all(u.reshape(m.nnx, m.nny, m.nnz, 6)[:, :, ksurf + 1:, [0, 3, 5]] == MU0)
    assert np.array_equal(s[0, E:m.nny - E, E - 1:ksurf + 1], s[E, E:m.nny - E, E - 1:ksurf + 1])
    assert np.array_equal(s[:, 0, E - 1:ksurf + 1], s[:, E, E - 1:ksurf + 1])
    assert np.array_equal(s[:, :, 0], s[:, :, E - 1])


def _ascending(v):
    return all(v[c] <= v[c + 1] for c in range(len(v) - 1))


def _close_run(v, d, t, T2):
    """close_run of mvf_model.cu: the run of sorted v (d = +1 ascending, -1 descending)
    whose rounded squared difference to t is <= T2, by two bisections."""
    n = len(v)
    lo, hi = 0, n
    while lo < hi:
        c = (lo + hi) >> 1
        past = v[c] >= t if d > 0 else v[c] <= t
        if past or (t - v[c]) * (t - v[c]) <= T2:
            hi = c
        else:
            lo = c + 1
    first = lo
    lo, hi = -1, n - 1
    while lo < hi:
        c = (lo + hi + 1) >> 1
        before = v[c] <= t if d > 0 else v[c] >= t
        if before or (t - v[c]) * (t - v[c]) <= T2:
            lo = c
        else:
            hi = c - 1
    return first, lo


def _pruned(x, y, z, xm, ym, zm):
    """The GPU kernel's scan (mvf_model.cu) in IEEE double: seed bound, sorted runs found
    by bisection, then the reference's comparisons on the points whose partial sums
    stay below T^2(1+1e-14)."""
    mx, my, mz = zm.shape
    xm, ym = [float(v) for v in xm], [float(v) for v in ym]
    zc = [[[float(v) for v in zm[a, b]] for b in range(my)] for a in range(mx)]
    xs, ys = _ascending(xm), _ascending(ym)
    zs = [[1 if _ascending(zc[a][b]) else -1 if _ascending(zc[a][b][::-1]) else 0 for b in range(my)]
          for a in range(mx)]
    ia = int(np.argmin(np.abs(x - np.array(xm))))
    ja = int(np.argmin(np.abs(y - np.array(ym))))
    cxy = (x - xm[ia]) * (x - xm[ia]) + (y - ym[ja]) * (y - ym[ja])
    col = zc[ia][ja]
    seed = 1e20
    for c in range(mz):
        dd = math.sqrt(cxy + (z - col[c]) * (z - col[c]))
        if dd < seed:
            seed = dd
    T = max(seed, 1e-5)
    T2 = T * T * (1.0 + 1e-14)
    xr = _close_run(xm, 1, x, T2) if xs else (0, mx - 1)
    yr = _close_run(ym, 1, y, T2) if ys else (0, my - 1)
    ddmin, best = 1e20, -1
    for a in range(xr[0], xr[1] + 1):
        cx = (x - xm[a]) * (x - xm[a])
        if cx > T2:
            continue
        for b in range(yr[0], yr[1] + 1):
            cxy = cx + (y - ym[b]) * (y - ym[b])
            if cxy > T2:
                continue
            col = zc[a][b]
            zr = _close_run(col, zs[a][b], z, T2) if zs[a][b] else (0, mz - 1)
            for c in range(zr[0], zr[1] + 1):
                s = cxy + (z - col[c]) * (z - col[c])
                if s > T2:
                    continue
                dd = math.sqrt(s)
                if dd <= 1e-5:
                    return (a * my + b) * mz + c
                if dd < ddmin:
                    ddmin, best = dd, (a * my + b) * mz + c
    return best


def _brute(x, y, z, xm, ym, zm):
    mx, my, mz = zm.shape
    ddmin, best = 1e20, -1
    for a in range(mx):
        for b in range(my):
            for c in range(mz):
                dd = math.sqrt((x - xm[a]) ** 2 + (y - ym[b]) ** 2 + (z - zm[a, b, c]) ** 2)
                if dd <= 1e-5:
                    return (a * my + b) * mz + c
                if dd < ddmin:
                    ddmin, best = dd, (a * my + b) * mz + c
    return best


def test_pruned_scan_picks_the_reference_point():
    """The kernel's pruning skips only points that can neither be within 1e-5 nor a new
    minimum: on lattices full of exact ties, duplicates, near-hits (just inside and
    outside 1e-5), sorted (both directions) and unsorted coordinates it returns the
    brute-force scan's point."""
    rng = np.random.Generator(np.random.PCG64(11))
    for trial in range(120):
        mx, my, mz = rng.integers(1, 7, 3)
        step = float(rng.choice([1.0, 0.5, 100.0, 1e-6]))
        xm = step * rng.integers(-3, 4, mx).astype(float)
        ym = step * rng.integers(-3, 4, my).astype(float)
        zm = step * rng.integers(-3, 4, (mx, my, mz)).astype(float)
        if trial % 3 == 1:
            xm += rng.uniform(-1, 1, mx) * step * 0.1
        if trial % 2 == 0:  # sorted coordinates (duplicates kept), columns either way
            xm, ym = np.sort(xm), np.sort(ym)
            zm = np.sort(zm, axis=2)
            if trial % 4 == 0:
                zm = zm[:, :, ::-1].copy()
        for _ in range(20):
            x, y, z = (step * rng.integers(-4, 5, 3)).astype(float) / 2.0
            if trial % 4 == 2:
                x += float(rng.choice([0.0, 9.9e-6, 1.01e-5, -1e-5]))
            assert _pruned(x, y, z, xm, ym, zm) == _brute(x, y, z, xm, ym, zm), (trial, x, y, z)


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=IDS)
def test_gpu_map_matches_oracle_bit_exact(case):
    from movfem_gb300 import api
    m, gm = _model(case)
    w = 2 * math.pi * 0.05
    s_o, u_o = oracle.map_model(m, gm, w)
    n0 = api.kernel_launches()
    s_g, u_g = api.map_model(m, gm, w)
    assert api.kernel_launches() > n0
    assert np.array_equal(s_g.view(np.float64), s_o.view(np.float64))
    assert np.array_equal(u_g, u_o)


@pytest.mark.gpu
def test_gpu_map_ties_and_duplicates():
    """Points at cell centres with no relief put several points at the same distance
    from a node, and every point is stored twice with different values: the first in
    point order must win, as in the reference's strict comparisons."""
    from movfem_gb300 import api
    m = small_grid(20, nextd=2)
    gm = M.synthetic_geomodel(9, m, spacing=100.0, depth=320.0, relief=0.0)
    mx, my, mz = gm.zm.shape
    zm2 = np.repeat(gm.zm, 2, axis=2)
    sig2 = np.repeat(gm.sigma.reshape(mx, my, mz, 1), 2, axis=2)
    sig2[:, :, 1::2] *= 3.0
    gm2 = M.GeoModel(xm=gm.xm, ym=gm.ym, zm=zm2, sigma=sig2.reshape(-1, 1), ijsigma=gm.ijsigma)
    w = 2 * math.pi * 1.0
    s_o, u_o = oracle.map_model(m, gm2, w)
    s_g, u_g = api.map_model(m, gm2, w)
    assert np.array_equal(s_g.view(np.float64), s_o.view(np.float64))
    assert np.array_equal(u_g, u_o)
    # no node took a duplicate (the tripled values)
    vals = set(np.round(gm.sigma.reshape(-1), 15))
    assert set(np.round(s_g[:, 0].real[s_g[:, 0].real > 0], 15)) <= vals


@pytest.mark.gpu
@pytest.mark.parametrize("layout", ["descending-columns", "unsorted"])
def test_gpu_map_sorted_and_unsorted_model_arrays(layout):
    """The kernel bisects sorted xm / ym / columns and scans unsorted ones in full; both
    must give the oracle's (brute-force) answer bit for bit."""
    from movfem_gb300 import api
    m = small_grid(20, nextd=2, topo=25.0)
    gm = M.synthetic_geomodel(13, m, spacing=70.0, depth=300.0, relief=20.0, anisotropic=True)
    rng = np.random.Generator(np.random.PCG64(17))
    if layout == "descending-columns":
        gm.zm = gm.zm[:, :, ::-1].copy()
    else:
        gm.xm = gm.xm[rng.permutation(gm.xm.size)]
        gm.ym = gm.ym[rng.permutation(gm.ym.size)]
        gm.zm = np.take_along_axis(gm.zm, rng.permuted(np.argsort(gm.zm, axis=2), axis=2), axis=2)
    w = 2 * math.pi * 0.3
    s_o, u_o = oracle.map_model(m, gm, w)
    s_g, u_g = api.map_model(m, gm, w)
    assert np.array_equal(s_g.view(np.float64), s_o.view(np.float64))
    assert np.array_equal(u_g, u_o)


@pytest.mark.gpu
def test_gpu_map_rejects_what_the_reference_cannot_map():
    from movfem_gb300 import api
    m = small_grid(8, nextd=2)
    gm = M.synthetic_geomodel(1, m, spacing=90.0, depth=300.0)
    bad = M.GeoModel(xm=gm.xm, ym=gm.ym, zm=gm.zm, sigma=np.zeros((gm.zm.size, 2)),
                     ijsigma=np.array([[1, 1], [4, 1]], dtype=np.int32))
    with pytest.raises(api.MVFError) as e:
        api.map_model(m, bad, 1.0)
    assert e.value.code == api.E_ARG and "ijsigma" in str(e.value)
    m0 = small_grid(8, nextd=2)
    m0.nextd = 0
    with pytest.raises(api.MVFError) as e:
        api.map_model(m0, gm, 1.0)
    assert e.value.code == api.E_ARG and "nextd" in str(e.value)


def test_map_model_rejects_bad_arguments_before_any_device_work():
    """mvf_map_model validates its arguments on the host before touching the GPU, so its
    refusals (and their messages, through mvf_last_error(NULL)) are checked here
    without one."""
    from movfem_gb300 import api
    m = small_grid(8, nextd=2)
    gm = M.synthetic_geomodel(1, m, spacing=90.0, depth=300.0)
    cases = []
    m0 = small_grid(8, nextd=2)
    m0.nextd = 0
    cases.append((m0, gm, "nextd"))
    m1 = small_grid(8, nextd=2)
    m1.nzl_top = m1.nzl_air = 0
    cases.append((m1, gm, "air"))
    m2 = small_grid(8, nextd=2)
    m2.nextd = 5  # nx = 9 elements: none left inside 2 x 5 extension cells
    cases.append((m2, gm, "inner elements"))
    bad_ij = M.GeoModel(xm=gm.xm, ym=gm.ym, zm=gm.zm, sigma=np.zeros((gm.zm.size, 2)),
                        ijsigma=np.array([[1, 1], [0, 2]], dtype=np.int32))
    cases.append((m, bad_ij, "ijsigma"))
    empty = M.GeoModel(xm=gm.xm[:0], ym=gm.ym, zm=gm.zm[:0], sigma=np.zeros((0, 1)),
                       ijsigma=np.array([[1, 1]], dtype=np.int32))
    cases.append((m, empty, "empty"))
    m3 = small_grid(8, nextd=2)
    m3.nodes_per_elem = 9
    cases.append((m3, gm, "nodes_per_elem"))
    for grid, model, word in cases:
        with pytest.raises(api.MVFError) as e:
            api.map_model(grid, model, 1.0)
        assert e.value.code == api.E_ARG, (word, e.value)
        assert word in str(e.value), (word, str(e.value))
