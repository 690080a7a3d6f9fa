"""CPU restatement of the library's multilevel preconditioner -- TEST INFRASTRUCTURE ONLY.

The reference factorises every system with MUMPS (``zmumps`` job=6,
MoVFEM_3DMT.f90:113-115) and has no preconditioner; this module restates, in numpy and
scipy, the one the GPU library uses for its 36/54-DOF systems (``mvf_mg.cu``), so that a
test can compare one preconditioner cycle computed both ways on the same input:

* level 0: K + i w Mp, where Mp is the mass matrix of the interpolated conductivity
  shifted positive semidefinite at every Gauss point (optional) plus a floor
  conductivity (the oracle's ``orc_set_pmass`` switch), plus tau diag(K) (optional);
  FGMRES keeps the true A = K + i w M;
* level 1: the 12-edge space on the same cells, prolongation from the exact local
  combination of the 36/54-DOF element's edge functions (:func:`p_local`), operator
  P^T A P;
* levels 2, ...: cells merged in pairs per axis, the 12-edge prolongation of box cells
  (:func:`h_prolongation`), operator P^T A P, until at most 96 DOFs remain;
* every level but the coarsest: multiplicative vertex-patch Schwarz, colours 0..7
  before and 7..0 after the coarse correction; the coarsest: a dense solve.

Only ``tests/`` use this module.
"""
from __future__ import annotations

import copy
import math

import numpy as np
import scipy.sparse as sp

from . import Oracle

# reference coordinates of the element nodes (n_fem.f90:112-134) and the edge DOF ->
# (node, direction) tables (v_fem.f90:488-506), 1-based
NR = np.array([
    [1, 1, -1, -1, 1, 1, -1, -1, 1, 0, -1, 0, 1, 0, -1, 0, 1, 1, -1, -1, 1, 0, -1, 0, 0, 0, 0],
    [-1, 1, 1, -1, -1, 1, 1, -1, 0, 1, 0, -1, 0, 1, 0, -1, -1, 1, 1, -1, 0, 1, 0, -1, 0, 0, 0],
    [-1, -1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, -1, 1, 0]])
EDGES = {
    8: ([4, 4, 8, 3, 4, 8, 3, 7, 1, 1, 5, 2], [3, 2, 2, 3, 1, 1, 1, 1, 3, 2, 2, 3]),
    20: ([4, 8, 4, 3, 8, 7, 3, 7, 4, 1, 8, 5, 3, 2, 7, 6, 1, 5, 1, 2, 5, 6, 2, 6, 12, 20, 12, 16, 10, 17, 11, 20, 11,
          15, 19, 9],
         [3, 3, 2, 2, 2, 2, 3, 3, 1, 1, 1, 1, 1, 1, 1, 1, 3, 3, 2, 2, 2, 2, 3, 3, 3, 2, 2, 2, 3, 2, 3, 1, 1, 1, 1, 3]),
    27: ([4, 8, 4, 20, 8, 11, 15, 3, 19, 7, 3, 7, 4, 20, 8, 11, 15, 3, 19, 7, 12, 16, 12, 10, 16, 14, 10, 14, 1, 17, 5,
          9, 13, 2, 18, 6, 1, 5, 1, 17, 5, 9, 13, 2, 18, 6, 2, 6, 25, 26, 24, 22, 23, 21],
         [3, 3, 2, 2, 2, 3, 3, 2, 2, 2, 3, 3, 1, 1, 1, 1, 1, 1, 1, 1, 3, 3, 2, 2, 2, 2, 3, 3, 1, 1, 1, 1, 1, 1, 1, 1,
          3, 3, 2, 2, 2, 3, 3, 2, 2, 2, 3, 3, 3, 3, 2, 2, 1, 1]),
}
COARSEST = 96


def edge_factor(mn, i, d, t):
    """Scalar factor L of the edge basis of node i (0-based), direction d at points t
    [n, 3] (v_fem.f90:78-179 for the three element orders)."""
    a = NR[:, i]
    f = np.ones((t.shape[0], 3))
    if mn == 8:
        for k in range(3):
            if k != d:
                f[:, k] = 0.5 * (1 + a[k] * t[:, k])
        return f.prod(1)
    if mn == 20:
        if i < 8:
            s = a[0] * t[:, 0] + a[1] * t[:, 1] + a[2] * t[:, 2] - 1
            p = np.ones(t.shape[0])
            for k in range(3):
                if k != d:
                    p = p * (1 + a[k] * t[:, k])
            return p * s * 0.125
        for k in range(3):
            n = a[k]
            if n == 0:
                f[:, k] = 1 - t[:, k] ** 2
            elif k == d:
                f[:, k] = 1
            else:
                f[:, k] = 1 + n * t[:, k]
        f[:, 0] *= 0.5
        return f.prod(1)
    for k in range(3):
        n = a[k]
        if k == d:
            f[:, k] = 0.5 * (1 + n * t[:, k])
        else:
            f[:, k] = (1 - t[:, k] ** 2) if n == 0 else 0.5 * n * t[:, k] * (1 + n * t[:, k])
    return f.prod(1)


def nodal_fn(mn, i, t):
    """Shape function of node i (0-based) of the 20- or 27-node element at points t [n, 3]
    (the serendipity and Lagrange families of n_fem.f90:138-317)."""
    a = NR[:, i]
    if mn == 20:
        if i < 8:
            p = np.prod([1 + a[k] * t[:, k] for k in range(3)], axis=0)
            return p * (a[0] * t[:, 0] + a[1] * t[:, 1] + a[2] * t[:, 2] - 2) / 8
        return 0.25 * np.prod([(1 - t[:, k] ** 2) if a[k] == 0 else (1 + a[k] * t[:, k]) for k in range(3)], axis=0)
    return np.prod([(1 - t[:, k] ** 2) if a[k] == 0 else 0.5 * a[k] * t[:, k] * (1 + a[k] * t[:, k])
                    for k in range(3)], axis=0)


def grad_local(mn):
    """[me, mn]: the gradient of node function n as a combination of the element's edge
    functions, sum_i G[i, n] * edge fn i (exact: the edge space contains the gradients of
    the nodal space; the coefficients are multiples of 1/8)."""
    t = np.random.default_rng(1).uniform(-1, 1, (400, 3))
    en, ed = EDGES[mn]
    G = np.zeros((len(en), mn))
    h = 1e-5
    for n in range(mn):
        for d in range(3):
            tp, tm = t.copy(), t.copy()
            tp[:, d] += h
            tm[:, d] -= h
            target = (nodal_fn(mn, n, tp) - nodal_fn(mn, n, tm)) / (2 * h)
            idx = [i for i in range(len(en)) if ed[i] - 1 == d]
            B = np.stack([edge_factor(mn, en[i] - 1, d, t) for i in idx], 1)
            G[idx, n] = np.round(np.linalg.lstsq(B, target, rcond=None)[0] * 8) / 8
    return G


def node_ids(m):
    """[mn, ne]: global grid node (i*nny + j)*nnz + k of every element's local nodes."""
    o = m.nord - 1
    ie, je, ke = [v.ravel() for v in np.meshgrid(np.arange(m.nx), np.arange(m.ny), np.arange(m.nz), indexing="ij")]
    out = np.zeros((m.nodes_per_elem, ie.size), dtype=np.int64)
    for l in range(m.nodes_per_elem):
        a, b, c = NR[:, l] + 1
        out[l] = ((o * ie + a) * m.nny + o * je + b) * m.nnz + o * ke + c
    return out


def discrete_gradient(m, gne, n):
    """[n, npt] sparse: edge-DOF coefficients of the gradient of every grid node's
    function (20/27-node meshes); nodes on the outer boundary are left out, since with
    the Dirichlet boundary their gradients lose the boundary edges."""
    G = _csr_from_local(grad_local(m.nodes_per_elem), gne, node_ids(m) + 1, n, m.npt)
    i, j, k = np.meshgrid(np.arange(m.nnx), np.arange(m.nny), np.arange(m.nnz), indexing="ij")
    inner = ((i > 0) & (i < m.nnx - 1) & (j > 0) & (j < m.nny - 1) & (k > 0) & (k < m.nnz - 1)).ravel()
    return (G @ sp.diags(inner.astype(float))).tocsr()


def p_local(mn):
    """[me, 12]: 12-edge basis function j = sum_i P[i, j] * (mn-node element's edge fn i)."""
    t = np.random.default_rng(0).uniform(-1, 1, (400, 3))
    qn, qd = EDGES[mn]
    ln, ld = EDGES[8]
    P = np.zeros((len(qn), 12))
    for j in range(12):
        d = ld[j] - 1
        idx = [i for i in range(len(qn)) if qd[i] - 1 == d]
        B = np.stack([edge_factor(mn, qn[i] - 1, d, t) for i in idx], 1)
        c = np.linalg.lstsq(B, edge_factor(8, ln[j] - 1, d, t), rcond=None)[0]
        P[idx, j] = np.round(c * 8) / 8
    return P


def _csr_from_local(loc, rows, cols, nrow, ncol):
    """Global sparse map from identical local blocks loc [nr, nc] with row ids rows
    [nr, ne] and column ids cols [nc, ne] (1-based, <= 0 skipped); repeated entries
    keep the first."""
    r, c, v = [], [], []
    for a in range(loc.shape[0]):
        for b in range(loc.shape[1]):
            if loc[a, b] == 0:
                continue
            ok = (rows[a] > 0) & (cols[b] > 0)
            r.append(rows[a][ok] - 1); c.append(cols[b][ok] - 1); v.append(np.full(ok.sum(), loc[a, b]))
    r, c, v = np.concatenate(r), np.concatenate(c), np.concatenate(v)
    _, u = np.unique(r.astype(np.int64) * ncol + c, return_index=True)
    return sp.csr_matrix((v[u], (r[u], c[u])), shape=(nrow, ncol))


def linear_twin(m):
    """The 8-node mesh over the same cells (the corner nodes of m's grid)."""
    l = copy.copy(m)
    l.nodes_per_elem = 8
    o = m.nord - 1
    s = (m.nnx, m.nny, m.nnz)
    l.xp, l.yp = m.xp[::o].copy(), m.yp[::o].copy()
    l.zp = m.zp.reshape(s)[::o, ::o, ::o].reshape(-1).copy()
    l.sigma = m.sigma.reshape(s + (6,))[::o, ::o, ::o].reshape(-1, 6).copy()
    l.mu = m.mu.reshape(s + (6,))[::o, ::o, ::o].reshape(-1, 6).copy()
    return l


def merge_axis(n):
    return np.array([min(2 * i, n) for i in range((n + 1) // 2 + 1)])


def merged(l):
    """8-node mesh whose cells are l's cells merged in pairs per axis (a last odd cell
    stays single)."""
    c = copy.copy(l)
    ix, iy, iz = merge_axis(l.nx), merge_axis(l.ny), merge_axis(l.nz)
    c.nx, c.ny, c.nz = ix.size - 1, iy.size - 1, iz.size - 1
    s = (l.nx + 1, l.ny + 1, l.nz + 1)
    c.xp, c.yp = l.xp[ix].copy(), l.yp[iy].copy()
    c.zp = l.zp.reshape(s)[np.ix_(ix, iy, iz)].reshape(-1).copy()
    c.sigma = l.sigma.reshape(s + (6,))[np.ix_(ix, iy, iz)].reshape(-1, 6).copy()
    c.mu = l.mu.reshape(s + (6,))[np.ix_(ix, iy, iz)].reshape(-1, 6).copy()
    c._maps = (ix, iy, iz)
    return c


def h_prolongation(f, c, gf, nf, gc, nc):
    """12-edge functions of c's merged box cells expressed on f's cells: the fine
    coefficient is the merged cell's edge factor at the fine edge times the length ratio
    along the edge."""
    ln, ld = EDGES[8]
    ix, iy, iz = c._maps
    z1 = f.zp.reshape(f.nx + 1, f.ny + 1, f.nz + 1)[0, 0, :]
    coords, cmaps = [f.xp, f.yp, z1], [ix, iy, iz]
    ie, je, ke = (a.ravel() for a in np.meshgrid(np.arange(f.nx), np.arange(f.ny), np.arange(f.nz), indexing="ij"))
    fidx, cidx = [ie, je, ke], [ie // 2, je // 2, ke // 2]
    ce = (cidx[0] * c.ny + cidx[1]) * c.nz + cidx[2]
    r, cc, v = [], [], []
    for jf in range(12):
        nd, d = ln[jf] - 1, ld[jf] - 1
        a = NR[:, nd]
        cref = {}
        for ax in range(3):
            if ax != d:
                X = coords[ax][fidx[ax] + (a[ax] + 1) // 2]
                X0 = coords[ax][cmaps[ax][cidx[ax]]]
                X1 = coords[ax][cmaps[ax][cidx[ax] + 1]]
                cref[ax] = -1 + 2 * (X - X0) / (X1 - X0)
        ratio = (coords[d][fidx[d] + 1] - coords[d][fidx[d]]) / (
            coords[d][cmaps[d][cidx[d] + 1]] - coords[d][cmaps[d][cidx[d]]])
        for jc in range(12):
            if ld[jc] - 1 != d:
                continue
            ac = NR[:, ln[jc] - 1]
            val = ratio.copy()
            for ax in range(3):
                if ax != d:
                    val = val * 0.5 * (1 + ac[ax] * cref[ax])
            rows, cols = gf[jf], gc[jc][ce]
            ok = (rows > 0) & (cols > 0) & (np.abs(val) > 1e-14)
            r.append(rows[ok] - 1); cc.append(cols[ok] - 1); v.append(val[ok])
    r, cc, v = np.concatenate(r), np.concatenate(cc), np.concatenate(v)
    _, u = np.unique(r.astype(np.int64) * nc + cc, return_index=True)
    return sp.csr_matrix((v[u], (r[u], cc[u])), shape=(nf, nc))


def vertex_patches(m, gne, n):
    """{vertex: [DOFs]}: a DOF is in the patch of vertex v when every element holding it
    lies in the 2x2x2 block of elements around v."""
    lo = np.full((n, 3), 1 << 30)
    hi = np.full((n, 3), -1)
    idx = np.stack([a.ravel() for a in np.meshgrid(np.arange(m.nx), np.arange(m.ny), np.arange(m.nz),
                                                   indexing="ij")], 1)
    for j in range(gne.shape[0]):
        ok = gne[j] > 0
        g = gne[j][ok] - 1
        for a in range(3):
            np.minimum.at(lo[:, a], g, idx[ok, a])
            np.maximum.at(hi[:, a], g, idx[ok, a])
    P = {}
    for g in range(n):
        for vi in range(hi[g, 0], lo[g, 0] + 2):
            for vj in range(hi[g, 1], lo[g, 1] + 2):
                for vk in range(hi[g, 2], lo[g, 2] + 2):
                    P.setdefault((vi, vj, vk), []).append(g)
    return P


def _colour_inverses(A, patches, nfine):
    """Per vertex-parity colour the block-diagonal sum of R_v^T A_v^-1 R_v."""
    A = A.tocsr()
    out = []
    for col in range(8):
        r, c, v = [], [], []
        for (vi, vj, vk), d in patches.items():
            if (vi & 1, vj & 1, vk & 1) != (col & 1, (col >> 1) & 1, (col >> 2) & 1):
                continue
            d = np.array(d)
            inv = np.linalg.inv(A[d][:, d].toarray())
            r.append(np.repeat(d, d.size)); c.append(np.tile(d, d.size)); v.append(inv.ravel())
        if r:
            out.append(sp.csr_matrix((np.concatenate(v), (np.concatenate(r), np.concatenate(c))),
                                     shape=(nfine, nfine)))
    return out


class Multilevel:
    """The preconditioner of one frequency w (angular; FP32-rounded as the assembly
    does when the mesh keeps the FP32-constant quirk) for mesh m (20/27 nodes)."""

    def __init__(self, m, omega, floor=1e-8, tau=0.0, semidefinite=True, surface_gradient=False):
        from . import lib
        w = float(np.float32(omega)) if (m.quirks & 2) else float(omega)
        o = Oracle(m)
        o.set_sigma(m.sigma_at(omega))
        A, self.rhs = o.matrix(omega)
        self.A_true = A.tocsr()
        lib().orc_set_pmass(1 if semidefinite else 2, float(floor))
        try:
            A0 = Oracle(m, sigma=m.sigma_at(omega)).matrix(omega)[0].tocsr()
        finally:
            lib().orc_set_pmass(0, 0.0)
        if tau > 0:
            A0 = (A0 + 1j * w * tau * sp.diags(self.A_true.real.diagonal())).tocsr()
        gq, nq = o.numbering()
        self.A = [A0]
        self.P = []
        self.B = [_colour_inverses(A0, vertex_patches(m, gq, nq), nq)]
        lm = linear_twin(m)
        gl, nl = Oracle(lm).numbering()
        P = _csr_from_local(p_local(m.nodes_per_elem), gq, gl, nq, nl)
        cur, g, n = lm, gl, nl
        while True:
            self.P.append(P)
            self.A.append((P.T @ self.A[-1] @ P).tocsr())
            if n <= COARSEST or max(cur.nx, cur.ny, cur.nz) <= 1:
                break
            cm = merged(cur)
            gc, nc = Oracle(cm).numbering()
            if nc <= 0:
                break
            self.B.append(_colour_inverses(self.A[-1], vertex_patches(cur, g, n), n))
            P = h_prolongation(cur, cm, g, n, gc, nc)
            cur, g, n = cm, gc, nc
        self.coarse = np.linalg.inv(self.A[-1].toarray())
        self.sizes = [a.shape[0] for a in self.A]
        self.surface = None
        if surface_gradient:
            self.surface = self._surface_gradient(m, gq, nq, surface_gradient == "negative")

    def _surface_gradient(self, m, gq, nq, negative=False):
        """Gradient-space correction on the node layers around the earth's surface (and,
        with ``negative``, on the nodes of every element whose interpolated conductivity
        turns negative), with the true operator.  Just above the surface the quadratic interpolation of the nodal
        conductivity (earth value at the surface nodes, 0 above) dips below zero, to
        -sigma/8 at mid-height of the first air cells, so the true A is indefinite on the
        gradients there while the preconditioner's mass is positive: those modes are solved
        exactly here, G_s (G_s^T A G_s)^-1 G_s^T, G_s the gradients of the grid nodes from
        one node layer below the surface to the top of the first air cells."""
        import scipy.sparse.linalg as spla
        o = m.nord - 1
        ksurf = o * (m.nz - m.nzl_air - m.nzl_top)
        kk = np.arange(m.npt) % m.nnz
        G = discrete_gradient(m, gq, nq)
        sel = (kk >= ksurf - 1) & (kk <= ksurf + o)
        if negative:
            # also the nodes of every element whose interpolated conductivity turns
            # negative at one of its 27 Gauss points (block and layer edges inside the earth)
            g = np.array([-math.sqrt(0.6), 0.0, math.sqrt(0.6)])
            gp = np.array([[a, b, c] for a in g for b in g for c in g])
            Nv = np.stack([nodal_fn(m.nodes_per_elem, i, gp) for i in range(m.nodes_per_elem)], 0)
            ids = node_ids(m)
            sg = Nv.T @ m.sigma[:, 0].real[ids]
            sel[ids[:, sg.min(0) < 0].ravel()] = True
        cols = np.nonzero(sel)[0]
        Gs = G[:, cols].tocsr()
        used = np.nonzero(np.asarray(abs(Gs).sum(axis=0)).ravel() > 0)[0]
        Gs = Gs[:, used].tocsr()
        lu = spla.splu((Gs.T @ self.A_true @ Gs).tocsc())
        return Gs, lu

    def _cycle(self, l, b):
        if l == len(self.A) - 1:
            return self.coarse @ b
        A, B = self.A[l], self.B[l]
        x = np.zeros_like(b)
        for Bc in B:
            x = x + Bc @ (b - A @ x)
        x = x + self.P[l] @ self._cycle(l + 1, self.P[l].T @ (b - A @ x))
        for Bc in B[::-1]:
            x = x + Bc @ (b - A @ x)
        return x

    def _apply(self, r):
        z = self._cycle(0, r)
        if self.surface is not None:
            Gs, lu = self.surface
            z = z + Gs @ lu.solve(Gs.T @ (r - self.A_true @ z))
        return z

    def __call__(self, r):
        r = np.asarray(r, dtype=np.complex128)
        if r.ndim == 1:
            return self._apply(r)
        return np.stack([self._apply(r[:, q]) for q in range(r.shape[1])], 1)
