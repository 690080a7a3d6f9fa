"""Synthetic MT models in the reference's mesh layout.

The reference builds its mesh in ``geometry.f90`` (``grid_3d``: extension zones,
``zblocks`` layering, ``gauss_grid`` node coordinates, ``assign_model`` nodal
conductivity).  Mesh generation is outside the accelerated path; this module emits
the same arrays that ``grid_3d`` leaves in the ``geometry`` module and that the
assembly reads:

* ``xp[nnx]``, ``yp[nny]``: tensor x/y node coordinates (``g_xp``, ``g_yp``),
* ``zp[npt]``: z of every node, node id ``(i*nny + j)*nnz + k`` (``g_zp``),
* ``sigma[npt, 6]`` complex128: packed (xx, xy, xz, yy, yz, zz) conductivity with
  ``i*eps*omega_1`` on the diagonal, FP32-rounded as ``cmplx()`` does in
  ``assign_model`` (geometry.f90:1037-1085) and in the air loop (geometry.f90:933-945),
* ``mu[npt, 6]``: packed permeability (``g_mu``),
* ``nextd`` (extension cells per side), ``nzl_top = g_nzl(g_nsf)`` and
  ``nzl_air = g_nzl(g_nsf-1)`` (geometry.f90:415-483).

Element order follows ``g_nordx`` (2 for 8-node, 3 for 20/27-node elements): quadratic
meshes carry mid-side and centre nodes in the node grid (geometry.f90:487-586).
Padding cells grow as ``1.3*i*d`` away from the core like ``extension``
(geometry.f90:224-344).  Seeds use numpy's PCG64.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

EPS0 = 8.854187817e-12
MU0 = 4.0 * math.pi * 1.0e-7
GROWTH = 1.3


def f32(x):
    return np.float64(np.float32(x))


@dataclasses.dataclass
class Mesh:
    nodes_per_elem: int
    nx: int
    ny: int
    nz: int
    xp: np.ndarray
    yp: np.ndarray
    zp: np.ndarray
    sigma: np.ndarray  # complex128 [npt, 6]
    mu: np.ndarray     # float64 [npt, 6]
    dirichlet: int = 1
    inimod: int = 1
    gpml_sch: int = 0
    a0: float = 1.0
    b0: float = 1.0
    nn: float = 2.0
    nextd: int = 0
    nzl_top: int = 0
    nzl_air: int = 0
    ztop: float = 0.0
    h_sigma: float = 0.01
    l_sigma: np.ndarray | None = None
    l_dz: np.ndarray | None = None
    quirks: int = 7
    rx: np.ndarray | None = None     # receivers [nrx, 2] (x, y)
    freqs: np.ndarray | None = None  # Hz
    name: str = ""

    @property
    def nord(self) -> int:
        return 2 if self.nodes_per_elem == 8 else 3

    @property
    def me(self) -> int:
        return {8: 12, 20: 36, 27: 54}[self.nodes_per_elem]

    @property
    def ne(self) -> int:
        return self.nx * self.ny * self.nz

    @property
    def nnx(self) -> int:
        return self.nx * (self.nord - 1) + 1

    @property
    def nny(self) -> int:
        return self.ny * (self.nord - 1) + 1

    @property
    def nnz(self) -> int:
        return self.nz * (self.nord - 1) + 1

    @property
    def npt(self) -> int:
        return self.nnx * self.nny * self.nnz

    def sigma_at(self, omega: float) -> np.ndarray:
        """Nodal sigma as the reference holds it at angular frequency ``omega``.

        ``update_sigma`` (geometry.f90:144-153) indexes ``g_sigma(i,j)`` with
        ``i`` up to g_npt on an array dimensioned (6, g_npt): in column-major memory it
        visits the linear entries 0 .. g_npt+29 and resets the imaginary part of each
        non-zero one to fp32(eps*omega).  Every other entry keeps its grid-time value.
        """
        s = self.sigma.reshape(-1).copy()
        n = min(self.npt + 30, s.size)
        head = s[:n]
        nz = head.imag != 0.0
        head[nz] = head.real[nz] + 1j * f32(EPS0 * omega)
        s[:n] = head
        return s.reshape(self.npt, 6)


@dataclasses.dataclass
class GeoModel:
    """Inner geomodel in the layout read_innermodel / read_geomodel leave it
    (read_input.f90:104-200): model point p = (im*my + jm)*mz + km at
    (xm[im], ym[jm], zm[p]) in the grid's coordinates; ``sigma[p, c]`` is component c,
    whose tensor index is ``ijsigma[c] = (i, j)`` (1-based, "SIGMAij"); ``mu`` likewise
    (relative permeability), or None for mu = mu0 (in_imu = 0)."""
    xm: np.ndarray          # [mx]
    ym: np.ndarray          # [my]
    zm: np.ndarray          # [mx, my, mz]
    sigma: np.ndarray       # [mx*my*mz, isigma]
    ijsigma: np.ndarray     # [isigma, 2]
    mu: np.ndarray | None = None    # [mx*my*mz, imu]
    ijmu: np.ndarray | None = None  # [imu, 2]

    @property
    def shape(self):
        return self.zm.shape

    def c_arrays(self) -> dict:
        """Contiguous arrays for the C-ABI: ij tables in the Fortran layout
        {i_1..i_n, j_1..j_n}."""
        mx, my, mz = self.zm.shape
        ij_s = np.asarray(self.ijsigma, dtype=np.int32).reshape(-1, 2)
        sig = np.ascontiguousarray(self.sigma, dtype=np.float64).reshape(mx * my * mz, ij_s.shape[0])
        ijs = np.ascontiguousarray(ij_s.T).reshape(-1)
        if self.mu is None:
            mu, ijm, imu = None, None, 0
        else:
            ij_m = np.asarray(self.ijmu, dtype=np.int32).reshape(-1, 2)
            mu = np.ascontiguousarray(self.mu, dtype=np.float64).reshape(mx * my * mz, ij_m.shape[0])
            imu = mu.shape[1]
            ijm = np.ascontiguousarray(ij_m.T).reshape(-1)
        return dict(mx=mx, my=my, mz=mz, xm=np.ascontiguousarray(self.xm, dtype=np.float64),
                    ym=np.ascontiguousarray(self.ym, dtype=np.float64),
                    zm=np.ascontiguousarray(self.zm, dtype=np.float64).reshape(-1), isigma=sig.shape[1],
                    ijsigma=ijs, sigma=sig, imu=imu, ijmu=ijm, mu=mu)


FULL_TENSOR = np.array([[1, 1], [1, 2], [1, 3], [2, 2], [2, 3], [3, 3]], dtype=np.int32)


def synthetic_geomodel(seed: int, mesh: "Mesh", *, spacing: float, depth: float, anisotropic: bool = False,
                       relief: float = 0.0, mu_tensor: bool = False, on_nodes: bool = False,
                       node_stride: int = 1, topo_fn=None) -> GeoModel:
    """A seeded inner geomodel over ``mesh``'s core: model points every ``spacing`` m in
    x and y over the inner elements and down to ``depth`` below the surface, z per
    column shifted by up to ``relief`` m; layered conductivity (log-uniform
    [1e-3, 1] S/m) with two blocks (log-uniform [1e-3, 10] S/m).  ``anisotropic``
    gives each point a full SPD tensor R diag(l) R^T (six components, off-diagonals of
    either sign); ``mu_tensor`` adds relative permeabilities near 1 as six components;
    ``on_nodes`` puts the points on every ``node_stride``-th grid node of the inner
    columns instead (exact hits, distance 0).  ``topo_fn(x, y)`` (the grid's surface
    relief) shifts each model column with the surface."""
    rng = np.random.Generator(np.random.PCG64(seed))
    o = mesh.nord - 1
    E = mesh.nextd * o
    x0, x1 = mesh.xp[E], mesh.xp[mesh.nnx - 1 - E]
    y0, y1 = mesh.yp[E], mesh.yp[mesh.nny - 1 - E]
    zs = mesh.ztop
    if on_nodes:
        # every node_stride-th grid node of the inner columns, from the bottom to the surface
        ksurf = mesh.nnz - (mesh.nzl_top + mesh.nzl_air) * o - 1
        ii = np.arange(E, mesh.nnx - E, node_stride)
        jj = np.arange(E, mesh.nny - E, node_stride)
        kk = np.arange(0, ksurf + 1, node_stride)
        xm, ym = mesh.xp[ii].copy(), mesh.yp[jj].copy()
        zm = mesh.zp.reshape(mesh.nnx, mesh.nny, mesh.nnz)[np.ix_(ii, jj, kk)].copy()
    else:
        xm = np.arange(x0 + 0.5 * spacing, x1, spacing)
        ym = np.arange(y0 + 0.5 * spacing, y1, spacing)
        nzm = max(2, int(depth // spacing))
        zline = zs - spacing * (0.5 + np.arange(nzm))[::-1]
        shift = relief * rng.uniform(-1, 1, (xm.size, ym.size, 1))
        zm = np.broadcast_to(zline[None, None, :] + shift, (xm.size, ym.size, nzm)).copy()
    mx, my, mz = zm.shape
    X, Y = np.meshgrid(xm, ym, indexing="ij")
    hs = np.zeros((mx, my, 1))
    if topo_fn is not None and not on_nodes:
        hs = topo_fn(X, Y)[..., None]
        zm = zm + hs
    X = np.broadcast_to(X[..., None], zm.shape)
    Y = np.broadcast_to(Y[..., None], zm.shape)
    d = (zs + hs) - zm
    lsig = 10.0 ** rng.uniform(-3, 0, 3)
    iface = np.sort(rng.uniform(0.1, 0.9, 2)) * max(depth, 1.0)
    s = lsig[np.searchsorted(iface, d)]
    for _ in range(2):
        c = rng.uniform([x0, y0, 0.0], [x1, y1, max(depth, 1.0)])
        h = rng.uniform(0.1, 0.3, 3) * np.array([x1 - x0, y1 - y0, max(depth, 1.0)])
        inside = (np.abs(X - c[0]) <= h[0]) & (np.abs(Y - c[1]) <= h[1]) & (np.abs(d - c[2]) <= h[2])
        s = np.where(inside, 10.0 ** rng.uniform(-3, 1), s)
    n = mx * my * mz
    if anisotropic:
        q, _ = np.linalg.qr(rng.normal(size=(n, 3, 3)))
        lam = s.reshape(n, 1) * 10.0 ** rng.uniform(-1, 1, (n, 3))
        T = np.einsum("nij,nj,nkj->nik", q, lam, q)
        sigma = np.stack([T[:, i - 1, j - 1] for i, j in FULL_TENSOR], axis=1)
        ijs = FULL_TENSOR.copy()
    else:
        sigma = s.reshape(n, 1).copy()
        ijs = np.array([[1, 1]], dtype=np.int32)
    mu = ijm = None
    if mu_tensor:
        mu = np.zeros((n, 6))
        mu[:, [0, 3, 5]] = 1.0 + rng.uniform(0, 0.5, (n, 3))
        mu[:, [1, 2, 4]] = rng.uniform(-0.05, 0.05, (n, 3))
        ijm = FULL_TENSOR.copy()
    return GeoModel(xm=xm, ym=ym, zm=zm, sigma=sigma, ijsigma=ijs, mu=mu, ijmu=ijm)


def from_grid(info: dict, xp: np.ndarray, yp: np.ndarray, zp: np.ndarray, **kw) -> Mesh:
    """The mesh of a grid built by :func:`movfem_gb300.api.grid_3d` (grid_3d's node
    coordinates, padding and layer counts), before the model mapping fills its nodal
    conductivity and permeability (zero here; :func:`movfem_gb300.api.map_model` gives
    them).  Keyword arguments set the boundary fields (dirichlet, gpml_sch, ...)."""
    npt = int(info["npt"])
    return Mesh(nodes_per_elem=int(info["nodes_per_elem"]), nx=int(info["nx"]), ny=int(info["ny"]),
                nz=int(info["nz"]), xp=xp, yp=yp, zp=zp, sigma=np.zeros((npt, 6), dtype=np.complex128),
                mu=np.zeros((npt, 6)), nextd=int(info["nextd"]), nzl_top=int(info["nzl_top"]),
                nzl_air=int(info["nzl_air"]), ztop=float(info["ztop"]), **kw)


def _padding(n: int, d: float) -> np.ndarray:
    return np.array([GROWTH * i * d for i in range(1, n + 1)])


def _axis(ncore: int, d: float, nextd: int, x0: float = 0.0) -> np.ndarray:
    """Cell edges: nextd growing cells, ncore cells of size d, nextd growing cells."""
    pad = _padding(nextd, d)
    left = x0 - np.cumsum(pad)[::-1] if nextd else np.array([])
    core = x0 + d * np.arange(ncore + 1)
    right = core[-1] + np.cumsum(pad) if nextd else np.array([])
    return np.concatenate([left, core, right])


def _refine(edges: np.ndarray, nord: int) -> np.ndarray:
    if nord == 2:
        return edges.copy()
    mids = 0.5 * (edges[:-1] + edges[1:])
    out = np.empty(2 * edges.size - 1)
    out[0::2] = edges
    out[1::2] = mids
    return out


def build_mesh(*, nodes_per_elem: int, ncx: int, ncy: int, ncz_earth: int, dx: float, dy: float,
               dz: float, n_air: int, dz_air: float, nextd: int, sigma_fn, omega1: float,
               topo_fn=None, dirichlet: int = 1, gpml_sch: int = 0, a0: float = 1.0, b0: float = 1.0,
               nn: float = 2.0, rx=None, freqs=None, name: str = "", full_tensor_fn=None) -> Mesh:
    """Build a mesh.  ``sigma_fn(x, y, depth)`` gives isotropic earth conductivity at
    node positions (depth below the local surface, metres); ``full_tensor_fn`` (if
    given) returns [..., 6] real packed tensors instead.  Air nodes get sigma = 0."""
    nord = 2 if nodes_per_elem == 8 else 3
    xe = _axis(ncx, dx, nextd)
    ye = _axis(ncy, dy, nextd)
    # z cells from the bottom: nextd growing cells, earth, air, nextd growing top cells
    zb = np.concatenate([-np.cumsum(_padding(nextd, dz))[::-1] if nextd else np.array([]),
                         dz * np.arange(ncz_earth + 1)])
    zsurf = zb[-1]
    za = zsurf + dz_air * np.arange(1, n_air + 1)
    ztop_edges = za[-1] + np.cumsum(_padding(nextd, dz_air)) if nextd else np.array([])
    ze = np.concatenate([zb, za, ztop_edges])
    nx, ny, nz = xe.size - 1, ye.size - 1, ze.size - 1
    xp, yp = _refine(xe, nord), _refine(ye, nord)
    zline = _refine(ze, nord)
    nnx, nny, nnz = xp.size, yp.size, zline.size
    X, Y, Z = np.meshgrid(xp, yp, zline, indexing="ij")
    k_surf = (nextd + ncz_earth) * (nord - 1)  # node index of the surface in a column
    if topo_fn is not None:
        # shift every node of the column by a height that fades to zero at the bottom
        # and top boundaries, keeping the surface node index fixed
        h = topo_fn(X[:, :, 0], Y[:, :, 0])[:, :, None]
        zb0, zt0 = zline[0], zline[-1]
        w = np.where(Z <= zsurf, (Z - zb0) / (zsurf - zb0), (zt0 - Z) / (zt0 - zsurf))
        Z = Z + h * w
    zp = Z.reshape(-1).copy()
    npt = zp.size
    kidx = np.broadcast_to(np.arange(nnz)[None, None, :], X.shape)
    surf_z = Z[:, :, k_surf][:, :, None]
    depth = surf_z - Z
    is_air = kidx > k_surf
    sig = np.zeros((nnx, nny, nnz, 6), dtype=np.complex128)
    ieps = 1j * f32(EPS0 * omega1)
    if full_tensor_fn is not None:
        t = full_tensor_fn(X, Y, np.maximum(depth, 0.0))
        sig[..., :] = t
    else:
        s = sigma_fn(X, Y, np.maximum(depth, 0.0))
        sig[..., 0] = s
        sig[..., 3] = s
        sig[..., 5] = s
    sig[is_air] = 0.0
    sig[..., 0] += ieps
    sig[..., 3] += ieps
    sig[..., 5] += ieps
    mu = np.zeros((nnx, nny, nnz, 6))
    mu[..., 0] = MU0
    mu[..., 3] = MU0
    mu[..., 5] = MU0
    m = Mesh(nodes_per_elem=nodes_per_elem, nx=nx, ny=ny, nz=nz, xp=xp, yp=yp, zp=zp,
             sigma=sig.reshape(npt, 6), mu=mu.reshape(npt, 6), dirichlet=dirichlet,
             gpml_sch=gpml_sch, a0=a0, b0=b0, nn=nn, nextd=nextd, nzl_top=nextd, nzl_air=n_air,
             ztop=zsurf, name=name)
    m.rx = np.asarray(rx, dtype=np.float64) if rx is not None else None
    m.freqs = np.asarray(freqs, dtype=np.float64) if freqs is not None else None
    return m


def rx_grid(n: int, lo: float, hi: float) -> np.ndarray:
    """n x n receivers strictly inside [lo, hi) so each falls in one element column."""
    c = lo + (hi - lo) * (np.arange(n) + 0.5) / n
    gx, gy = np.meshgrid(c, c, indexing="ij")
    return np.stack([gx.ravel(), gy.ravel()], axis=1)


# ------------------------------------------------------------------ workloads
def plain_linear_block(ncells: int = 20, d: float = 100.0, n_air: int = 10, dz_air: float = 200.0,
                       nrx: int = 11) -> Mesh:
    """Linear 8-node elements, ncells^3 earth cells at d m + n_air air cells of dz_air m,
    Dirichlet zero-secondary boundaries; half-space 0.01 S/m with a 1 S/m block of
    6x6x4 cells centred 300 m deep; 1 Hz; nrx x nrx surface receivers."""
    L = ncells * d
    cx = 0.5 * L
    bx = 3 * d * ncells / 20.0
    top, bot = 100.0 * ncells / 20.0, 500.0 * ncells / 20.0

    def sigma_fn(x, y, depth):
        inside = (np.abs(x - cx) <= bx + 1e-9) & (np.abs(y - cx) <= bx + 1e-9) & \
                 (depth >= top - 1e-9) & (depth <= bot + 1e-9)
        return np.where(inside, 1.0, 0.01)

    f = np.array([1.0])
    return build_mesh(nodes_per_elem=8, ncx=ncells, ncy=ncells, ncz_earth=ncells, dx=d, dy=d, dz=d,
                      n_air=n_air, dz_air=dz_air, nextd=0, sigma_fn=sigma_fn,
                      omega1=2 * math.pi * f[0], dirichlet=1, rx=rx_grid(nrx, 0.0, L), freqs=f,
                      name=f"linear-{ncells}x{ncells}x{ncells + n_air}-dirichlet")


def layered_blocks(seed: int, *, nodes_per_elem: int = 20, ncx: int = 40, ncy: int = 40, ncz: int = 30,
                   d: float = 50.0, nextd: int = 8, n_air: int = 10, dz_air: float = 100.0,
                   nfreq: int = 8, fmin: float = 1e-3, fmax: float = 100.0, nrx: int = 11,
                   gpml_sch: int = 0, nlayer: int = 4, nblock: int = 3) -> Mesh:
    """Layered earth (nlayer layers, sigma log-uniform [1e-3, 1] S/m, thicknesses
    uniform [100, 800] m) with nblock seeded blocks of 4-10 cells per side (sigma
    log-uniform [1e-3, 10]); GPML boundaries; nfreq frequencies log-spaced."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lsig = 10.0 ** rng.uniform(-3, 0, nlayer)
    thick = rng.uniform(100, 800, nlayer - 1)
    iface = np.cumsum(thick)
    blocks = []
    for _ in range(nblock):
        size = rng.integers(4, 11, 3)
        lo = [rng.integers(0, max(1, n - s)) for n, s in zip((ncx, ncy, ncz), size)]
        blocks.append((np.array(lo) * d, (np.array(lo) + size) * d, 10.0 ** rng.uniform(-3, 1)))

    def sigma_fn(x, y, depth):
        s = lsig[np.searchsorted(iface, depth, side="left").clip(0, nlayer - 1)]
        for lo, hi, sv in blocks:
            inside = (x >= lo[0]) & (x <= hi[0]) & (y >= lo[1]) & (y <= hi[1]) & \
                     (depth >= lo[2]) & (depth <= hi[2])
            s = np.where(inside, sv, s)
        return s

    f = np.logspace(np.log10(fmin), np.log10(fmax), nfreq)
    return build_mesh(nodes_per_elem=nodes_per_elem, ncx=ncx, ncy=ncy, ncz_earth=ncz, dx=d, dy=d, dz=d,
                      n_air=n_air, dz_air=dz_air, nextd=nextd, sigma_fn=sigma_fn,
                      omega1=2 * math.pi * f[0], dirichlet=0, gpml_sch=gpml_sch, a0=1.0, b0=1.0, nn=2.0,
                      rx=rx_grid(nrx, 0.0, ncx * d), freqs=f,
                      name=f"order{nodes_per_elem}-{ncx}x{ncy}x{ncz}-gpml{gpml_sch}")
