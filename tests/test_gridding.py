"""Gridding (grid_3d, geometry.f90:48-118): the native ``mvf_grid_3d`` against the CPU
restatement in ``oracle/gridding.py``, bit for bit, and both against the properties
the construction guarantees.  Host code only: these run without a GPU.

The reference's Fortran cannot be compiled on either machine, so these pin the native
code to the restatement; the restatement itself is checked by the defining properties
of the Shepard interpolant (it interpolates the data and reproduces quadratics) and of
the grid (padding widths 1.3 i d, layering, node order)."""
import math

import numpy as np
import pytest

import oracle
from oracle import gridding as G
from movfem_gb300 import api
from movfem_gb300 import mesh as M


def _case(mn, seed=1, n_if=2, npts=6, freq=100.0, sigma=1.0, d=100.0):
    """Receivers on a line, n_if interfaces of npts x npts jittered points (deepest
    first, the last one the topographic surface), a 4 x 4 x 3 inner model."""
    rng = np.random.Generator(np.random.PCG64(seed))
    rx = np.stack([np.linspace(0, 600, 7), np.full(7, 300.0), np.zeros(7)], 1)
    gx, gy = np.meshgrid(np.linspace(-100, 700, npts), np.linspace(-100, 700, npts), indexing="ij")
    ifs = []
    for l in range(n_if):
        z = -250.0 * (n_if - 1 - l) + 30 * np.sin(gx / 300 + l) * np.cos(gy / 250) + rng.normal(0, 3, gx.shape)
        ifs.append(np.stack([gx.ravel() + rng.uniform(-5, 5, gx.size), gy.ravel() + rng.uniform(-5, 5, gx.size),
                             z.ravel()], 1))
    xm = np.linspace(0, 600, 4)
    zm = np.broadcast_to(np.array([-400.0, -200.0, -50.0]), (4, 4, 3)).copy()
    return G.GridInput(d, d * 1.1, d * 0.9, 300.0, 500.0, mn, sigma, rx, ifs, xm, xm.copy(), zm,
                       np.array([freq, 10 * freq]))


def _native(g):
    return api.grid_3d(g.dx, g.dy, g.dz, g.high, g.depth, g.nodes_per_elem, g.sigma_bg, g.rx, g.interfaces, g.xm,
                       g.ym, g.zm, g.freqs)


def test_shepard_interpolates_and_reproduces_quadratics():
    """QSHEP2/QS2VAL: the interpolant passes through the data, and for quadratic data
    every nodal function is that quadratic, so the interpolant is too."""
    rng = np.random.Generator(np.random.PCG64(2))
    x, y = rng.uniform(0, 10, 60), rng.uniform(0, 10, 60)

    def q(x, y):
        return 1.5 + 0.3 * x - 0.2 * y + 0.05 * x * x - 0.02 * x * y + 0.04 * y * y

    s = G.qshep2(x, y, q(x, y), 13, 19, G.cells_per_side(60))
    assert all(G.qs2val(x[k], y[k], s) == q(x[k], y[k]) for k in range(60))
    pts = rng.uniform(2, 8, (100, 2))
    assert max(abs(G.qs2val(a, b, s) - q(a, b)) for a, b in pts) < 1e-12
    assert abs(s.a[7][1] - 0.05) < 1e-12 and abs(s.a[7][2] + 0.02) < 1e-12 and abs(s.a[7][3] - 0.04) < 1e-12


def test_cells_per_side_single_precision():
    assert G.cells_per_side(441) == 12 and G.cells_per_side(36) == 3 and G.cells_per_side(20) == 2


@pytest.mark.parametrize("mn", [8, 20, 27])
@pytest.mark.parametrize("n_if", [1, 2])
def test_native_matches_oracle(mn, n_if):
    g = _case(mn, n_if=n_if, seed=mn + n_if)
    o = G.grid_3d(g)
    info, xp, yp, zp, nzl = _native(g)
    assert (info["nextd"], info["nx"] + 1, info["ny"] + 1, info["nz"] + 1) == (o.nextd, o.nx, o.ny, o.nz)
    assert np.array_equal(nzl, o.nzl)
    assert (info["x0"], info["y0"], info["z0"], info["ztop"]) == (o.x0, o.y0, o.z0, o.ztop)
    assert np.array_equal(xp, o.xp) and np.array_equal(yp, o.yp) and np.array_equal(zp, o.zp)


# (frequency, conductivity, nd): ddx/depth >= 2.5; in [1.5, 2.5), where the reference
# leaves nd unset; <= 1/1.5; in (1/1.5, 1.5)
def _strip(n, width, seed):
    """n interface points in a narrow strip about y = 300: nearly collinear, so QSHEP2
    needs more equations (its label 7 path), the capped radius (label 9) and, for the
    narrowest, the damped linear fit (label 10)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    x = rng.uniform(-100, 700, n)
    return np.stack([x, 300 + rng.uniform(-width, width, n), 20 * np.sin(x / 150)], 1)


def _regular(n):
    """n x n points on a regular grid: equal distances everywhere (GETNP2's ties)."""
    gx, gy = np.meshgrid(np.linspace(-100, 700, n), np.linspace(-100, 700, n), indexing="ij")
    return np.stack([gx.ravel(), gy.ravel(), (40 * np.sin(gx / 200) * np.cos(gy / 170)).ravel()], 1)


@pytest.mark.parametrize("surface", ["strip-10-0", "strip-20-4", "strip-21-0.5-1", "strip-25-0.2-7",
                                     "strip-60-4-6", "regular-5", "regular-8"])
def test_every_shepard_branch_bit_exact(surface):
    """The native fit and the restatement agree bit for bit on inputs that take each
    branch of QSHEP2 (tie skipping, extra equations, radius cap, damped fit)."""
    kind, *a = surface.split("-")
    if kind == "regular":
        surf = _regular(int(a[0]))
    elif len(a) == 2:
        surf = _strip(30, float(a[0]), int(a[1]))
    else:
        surf = _strip(int(a[0]), float(a[1]), int(a[2]))
    g = _case(20)
    g.interfaces = [surf]
    o = G.grid_3d(g)
    info, xp, yp, zp, nzl = _native(g)
    assert np.array_equal(nzl, o.nzl)
    assert np.array_equal(xp, o.xp) and np.array_equal(yp, o.yp) and np.array_equal(zp, o.zp)


@pytest.mark.parametrize("freq,sigma,nd", [(100.0, 1.0, 1.5), (1.0, 1.0, 2.0), (0.05, 0.01, 2.0), (0.4, 1.0, 3.0)])
def test_padding_follows_the_skin_depth(freq, sigma, nd):
    """extension (geometry.f90:224-344): nextd is the first count >= 2 whose widths
    1.3 i min(d) sum past nd skin depths, and the padding grid lines step 1.3 i d outward."""
    g = _case(20, freq=freq, sigma=sigma)
    o = G.grid_3d(g)
    info = _native(g)[0]
    assert info["nd"] == nd
    depth = math.sqrt(2.0 / (G.MU_0 * sigma * 2.0 * G.PI * min(g.freqs)))
    assert info["skin_depth"] == o.info["skin_depth"] == depth
    assert info["nd"] == o.info["nd"]
    dmin, n = min(g.dx, g.dy, g.dz), info["nextd"]
    widths = lambda n: sum(1.3 * dmin * i for i in range(1, n + 1))
    assert widths(n) > info["nd"] * depth and (n == 2 or widths(n - 1) <= info["nd"] * depth)
    x = o.info["x"]
    steps = np.diff(x)
    assert np.allclose(steps[:n], [1.3 * i * g.dx for i in range(n, 0, -1)], rtol=1e-12)
    assert np.allclose(steps[-n:], [1.3 * i * g.dx for i in range(1, n + 1)], rtol=1e-12)
    assert np.allclose(steps[n:-n], g.dx, rtol=1e-9)


def test_grid_structure():
    """Node columns rise monotonically; the columns of the padding copy the core's edge
    columns (complete_grid); the layering sums to g_nz; coordinates are shifted by
    (x0, y0, z0) and the bottom of every column is z = 0."""
    g = _case(27, n_if=2)
    info, xp, yp, zp, nzl = _native(g)
    nnx, nny, nnz = info["nnx"], info["nny"], info["nnz"]
    assert info["nz"] == int(nzl.sum()) and nnz == info["nz"] * 2 + 1
    z = zp.reshape(nnx, nny, nnz)
    assert np.all(np.diff(z, axis=2) > 0) and np.all(z[:, :, 0] == 0.0)
    assert np.all(np.diff(xp) > 0) and np.all(np.diff(yp) > 0)
    e = info["nextd"] * 2
    assert np.array_equal(z[:e, e:nny - e], np.broadcast_to(z[e, e:nny - e], (e, nny - 2 * e, nnz)))
    assert np.array_equal(z[:, :e], np.broadcast_to(z[:, e:e + 1], (nnx, e, nnz)))
    # the top input interface: its mean height over the core matches the data's
    k_surf = 2 * int(nzl[:-2].sum())
    surf = z[e:nnx - e, e:nny - e, k_surf] + info["z0"]
    assert abs(surf.mean() - g.interfaces[-1][:, 2].mean()) < 30.0


def test_sample_sized_flat_model():
    """A flat surface of 21 x 21 points at 5 km, 42 receivers on two crossing lines,
    1990 m cells, 20 km of air and 50 km of earth, 0.01 S/m at 0.1 Hz, linear elements:
    the shape of the reference's sample input.  The surface and the bottom are flat, so
    every column is the same up to the rounding of the Shepard weights' sums, and the
    layers are 25 + 10 sub-layers thick."""
    gx, gy = np.meshgrid(np.linspace(0, 1e5, 21), np.linspace(0, 1e5, 21), indexing="ij")
    surf = np.stack([gx.ravel(), gy.ravel(), np.zeros(441)], 1)
    line = np.linspace(0, 1e5, 21)
    rx = np.concatenate([np.stack([line, np.full(21, 5e4), np.zeros(21)], 1),
                         np.stack([np.full(21, 5e4), line, np.zeros(21)], 1)])
    xm = np.linspace(0, 1e5, 21)
    zm = np.broadcast_to(np.linspace(-5e4, 0, 12), (21, 21, 12)).copy()
    info, xp, yp, zp, nzl = api.grid_3d(1990.0, 1990.0, 1990.0, 2e4, 5e4, 8, 0.01, rx, [surf], xm, xm, zm, [0.1])
    n = info["nextd"]
    assert list(nzl) == [n, 25, 10, n]
    z = zp.reshape(info["nnx"], info["nny"], info["nnz"])
    assert np.abs(z - z[0, 0]).max() < 1e-6
    assert abs(z[0, 0, n + 25] + info["z0"]) < 1e-6
    assert info["nx"] == int(1e5 / 1990) + 2 * n


def test_short_interface_is_an_error():
    g = _case(8)
    g.interfaces[0] = g.interfaces[0][:19]
    with pytest.raises(api.MVFError, match="fewer than 20 points"):
        _native(g)
    with pytest.raises(G.GridError):
        G.grid_3d(g)


@pytest.mark.gpu
@pytest.mark.parametrize("mn", [8, 20])
def test_grid_then_model_mapping_on_gpu(mn):
    """grid_3d's grid feeds the model mapping (innermodel_gqg, called at
    geometry.f90:103): the GPU mapping over the native grid matches the oracle's mapping
    over the same grid bit for bit, with the model points shifted like coord_transform
    shifts them (geometry.f90:367-411)."""
    g = _case(mn, n_if=2, seed=11)
    info, xp, yp, zp, nzl = _native(g)
    m = M.from_grid(info, xp, yp, zp)
    rng = np.random.Generator(np.random.PCG64(5))
    mx, my, mz = g.zm.shape
    gm = M.GeoModel(xm=g.xm - info["x0"], ym=g.ym - info["y0"], zm=g.zm - info["z0"],
                    sigma=rng.uniform(0.001, 1.0, (mx * my * mz, 1)), ijsigma=np.array([[1, 1]], dtype=np.int32))
    w = 2 * math.pi * g.freqs[0]
    s_o, u_o = oracle.map_model(m, gm, w)
    s_g, u_g = api.map_model(m, gm, w)
    assert np.array_equal(s_g.view(np.float64), s_o.view(np.float64))
    assert np.array_equal(u_g, u_o)
