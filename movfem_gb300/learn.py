"""Learned warm start for the Krylov solve.  No counterpart in the reference.

A small dilated 3-D convolutional operator (``mvf_net_*`` in the CUDA library: BF16
weights and activations, FP32 accumulation, trained with the library's own forward
and backward kernels and Adam) maps a description of the model on its cell grid to
the secondary field on every cell's edges.  The field is averaged onto the global
edge DOFs, and the amplitude of each polarisation is fitted exactly: x0 = a x^,
with a = (A x^)^H b / ||A x^||^2, which minimises ||b - a A x^||.  So the warm
start never leaves a larger residual than x0 = 0.  The FP64 refinement loop then
starts from b - A x0 and stops at the same true-residual tolerance.  The network
changes iteration counts, never the accepted answer.

Input channels per cell (all O(1)):
  0. (log10 sigma + 2) / 2, with sigma the mean of the diagonal conductivity at the
     cell's corner nodes (1e-6 S/m in the air);
  1. air flag;
  2. depth of the cell centre / 1 km (negative in the air);
  3. log10(f) / 2;
  4. log10(skin depth / cell size) / 2.
Output channels per cell: (pol * me + edge) * 2 + (re, im) of the solution,
normalised per polarisation to unit RMS over the DOFs.

Training data: seeded linear-element Dirichlet models of the family below, solved by
this library's FGMRES to a true residual of 1e-10.
"""
from __future__ import annotations

import ctypes
import math
import time

import numpy as np

from . import api
from . import mesh as M

CIN = 5


class WarmStartNet:
    """The operator on the GPU (owns an ``mvf_net``)."""

    def __init__(self, me: int = 12, width: int = 32, dilations=(1, 2, 4, 1), seed: int = 1, device: int = 0):
        self.L = api.load()
        self.me, self.width, self.dilations = me, width, tuple(dilations)
        self.cout = 4 * me
        d = (ctypes.c_int32 * len(dilations))(*dilations)
        h = ctypes.c_void_p()
        rc = self.L.mvf_net_create(ctypes.byref(h), CIN, width, self.cout, len(dilations), d, seed, device)
        self.h = h
        if rc != 0:
            msg = self.L.mvf_net_last_error(h).decode() if h.value else "bad arguments"
            raise api.MVFError(rc, msg)
        self.nparams = int(self.L.mvf_net_num_params(h))

    def _chk(self, rc):
        if rc != 0:
            raise api.MVFError(rc, self.L.mvf_net_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.L.mvf_net_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        p = np.empty(self.nparams, dtype=np.float32)
        self._chk(self.L.mvf_net_get_params(self.h, p.ctypes.data))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.nparams
        self._chk(self.L.mvf_net_set_params(self.h, p.ctypes.data))

    def forward(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float32)
        X, Y, Z, _ = x.shape
        out = np.empty((X, Y, Z, self.cout), dtype=np.float32)
        self._chk(self.L.mvf_net_forward(self.h, X, Y, Z, x.ctypes.data, out.ctypes.data))
        return out

    def gradients(self, x, target):
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(target, dtype=np.float32)
        X, Y, Z, _ = x.shape
        loss = ctypes.c_float()
        g = np.empty(self.nparams, dtype=np.float32)
        self._chk(self.L.mvf_net_gradients(self.h, X, Y, Z, x.ctypes.data, t.ctypes.data, ctypes.byref(loss),
                                           g.ctypes.data))
        return float(loss.value), g

    def train_step(self, x, target, lr: float) -> float:
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(target, dtype=np.float32)
        X, Y, Z, _ = x.shape
        loss = ctypes.c_float()
        self._chk(self.L.mvf_net_train_step(self.h, X, Y, Z, x.ctypes.data, t.ctypes.data, lr, ctypes.byref(loss)))
        return float(loss.value)


# ------------------------------------------------------------------ model family
def random_block_model(seed: int, ncx: int = 16, ncz: int = 12, d: float = 100.0, n_air: int = 6,
                       dz_air: float = 200.0, fmin: float = 0.1, fmax: float = 100.0) -> M.Mesh:
    """Linear-element Dirichlet model: half-space (sigma log-uniform [1e-3, 1] S/m)
    with 2-6 blocks of 2-6 cells per side (sigma log-uniform [1e-4, 10] S/m) and one
    frequency log-uniform in [fmin, fmax] Hz."""
    rng = np.random.Generator(np.random.PCG64(seed))
    bg = 10.0 ** rng.uniform(-3, 0)
    blocks = []
    for _ in range(int(rng.integers(2, 7))):
        size = np.minimum(rng.integers(2, 7, 3), [ncx, ncx, ncz])
        lo = [int(rng.integers(0, n - s + 1)) for n, s in zip((ncx, ncx, ncz), size)]
        blocks.append((np.array(lo) * d, (np.array(lo) + size) * d, 10.0 ** rng.uniform(-4, 1)))
    f = 10.0 ** rng.uniform(math.log10(fmin), math.log10(fmax))

    def sigma_fn(x, y, depth):
        s = np.full(np.broadcast(x, y, depth).shape, bg)
        for lo, hi, sv in blocks:
            inside = (x >= lo[0]) & (x <= hi[0]) & (y >= lo[1]) & (y <= hi[1]) & \
                     (depth >= lo[2]) & (depth <= hi[2])
            s = np.where(inside, sv, s)
        return s

    L = ncx * d
    return M.build_mesh(nodes_per_elem=8, ncx=ncx, ncy=ncx, ncz_earth=ncz, dx=d, dy=d, dz=d, n_air=n_air,
                        dz_air=dz_air, nextd=0, sigma_fn=sigma_fn, omega1=2 * math.pi * f, dirichlet=1,
                        rx=M.rx_grid(5, 0.0, L), freqs=np.array([f]), name=f"blocks-{seed}")


# ------------------------------------------------------------------ features / targets
def features(m: M.Mesh, f: float) -> np.ndarray:
    """Input grid [nx, ny, nz, CIN] float32 for frequency f (Hz)."""
    s = 2 if m.nodes_per_elem != 8 else 1  # corner-node stride in the node grid
    sig = np.real(m.sigma[:, 0] + m.sigma[:, 3] + m.sigma[:, 5]).reshape(m.nnx, m.nny, m.nnz) / 3.0
    zc = m.zp.reshape(m.nnx, m.nny, m.nnz)
    corner = sig[::s, ::s, ::s]
    zcn = zc[::s, ::s, ::s]
    cs = np.zeros((m.nx, m.ny, m.nz))
    zs = np.zeros((m.nx, m.ny, m.nz))
    for a in (0, 1):
        for b in (0, 1):
            for c in (0, 1):
                cs += corner[a:a + m.nx, b:b + m.ny, c:c + m.nz]
                zs += zcn[a:a + m.nx, b:b + m.ny, c:c + m.nz]
    cs /= 8.0
    zs /= 8.0
    air = zs > m.ztop
    cs = np.where(air | (cs <= 0.0), 1e-6, cs)
    dx = np.diff(np.asarray(m.xp))[::s][:m.nx].mean()
    skin = 503.0 / np.sqrt(cs * f)
    out = np.empty((m.nx, m.ny, m.nz, CIN), dtype=np.float32)
    out[..., 0] = (np.log10(cs) + 2.0) / 2.0
    out[..., 1] = air
    out[..., 2] = (m.ztop - zs) / 1000.0
    out[..., 3] = math.log10(f) / 2.0
    out[..., 4] = np.log10(skin / dx) / 2.0
    return out


def cell_targets(m: M.Mesh, gne: np.ndarray, x: np.ndarray):
    """Solution x [2, nne] -> per-cell target [nx, ny, nz, 4 me] (unit RMS per
    polarisation) and the two scales."""
    me = gne.shape[0]
    scale = np.sqrt(np.mean(np.abs(x) ** 2, axis=1))
    xn = x / np.where(scale > 0, scale, 1.0)[:, None]
    g = gne.T  # [ne, me]
    vals = np.where(g[None] > 0, xn[:, np.clip(g - 1, 0, None)], 0.0)  # [2, ne, me]
    t = np.empty((m.ne, 2, me, 2), dtype=np.float32)
    t[..., 0] = vals.real.transpose(1, 0, 2)
    t[..., 1] = vals.imag.transpose(1, 0, 2)
    return t.reshape(m.nx, m.ny, m.nz, 4 * me), scale


def dof_field(gne: np.ndarray, nne: int, out: np.ndarray) -> np.ndarray:
    """Network output [nx, ny, nz, 4 me] -> DOF field [2, nne] (mean over the cells
    sharing each DOF)."""
    me = gne.shape[0]
    g = gne.T.reshape(-1)
    o = out.reshape(-1, 2, me, 2)
    keep = g > 0
    idx = g[keep] - 1
    cnt = np.bincount(idx, minlength=nne).astype(np.float64)
    x = np.empty((2, nne), dtype=np.complex128)
    for p in range(2):
        v = (o[:, p, :, 0] + 1j * o[:, p, :, 1]).reshape(-1)[keep]
        x[p] = (np.bincount(idx, weights=v.real, minlength=nne) + 1j * np.bincount(idx, weights=v.imag, minlength=nne))
        x[p] /= np.maximum(cnt, 1.0)
    return x


def fitted_guess(p: api.MTProblem, xhat: np.ndarray, rhs: np.ndarray) -> np.ndarray:
    """Per polarisation, the multiple a x^ that minimises ||b - a A x^|| (FP64 SpMV)."""
    y = p.spmv(0, xhat)
    x0 = np.empty_like(xhat)
    for k in range(2):
        den = np.vdot(y[k], y[k])
        x0[k] = xhat[k] * (np.vdot(y[k], rhs[k]) / den if abs(den) > 0 else 0.0)
    return x0


# ------------------------------------------------------------------ pipeline
def make_sample(seed: int, tol: float = 1e-10):
    m = random_block_model(seed)
    f = float(m.freqs[0])
    p = api.MTProblem(m, device=0)
    p.assemble([2 * math.pi * f])
    x, st = p.solve(None, tol=tol, mode=api.MODE_MIXED, max_iters=5000, raise_noconv=False)
    gne = p.numbering()
    t, _ = cell_targets(m, gne, x[0])
    return features(m, f), t, st


def train(net: WarmStartNet, data, epochs: int = 30, lr: float = 2e-3, seed: int = 0, time_budget_s: float = 600.0):
    rng = np.random.Generator(np.random.PCG64(seed))
    t0 = time.time()
    hist = []
    for ep in range(epochs):
        order = rng.permutation(len(data))
        lr_e = lr * 0.5 * (1 + math.cos(math.pi * ep / epochs))
        losses = [net.train_step(data[i][0], data[i][1], lr_e) for i in order]
        hist.append(float(np.mean(losses)))
        if time.time() - t0 > time_budget_s:
            break
    return hist


def evaluate(net: WarmStartNet, seeds, tol: float = 1e-10, mode: int = api.MODE_MIXED):
    """Per held-out model: inner iterations and true residual without and with the
    learned warm start, and the warm start's initial relative residual."""
    rows = []
    for s in seeds:
        m = random_block_model(s)
        f = float(m.freqs[0])
        p = api.MTProblem(m, device=0)
        p.assemble([2 * math.pi * f])
        rhs = np.stack([p.export_rhs(0)])[0]
        x, st0 = p.solve(None, tol=tol, mode=mode, max_iters=5000, raise_noconv=False)
        gne = p.numbering()
        xhat = dof_field(gne, p.nne, net.forward(features(m, f)))
        x0 = fitted_guess(p, xhat, rhs)
        r0 = max(np.linalg.norm(rhs[k] - p.spmv(0, x0)[k]) / np.linalg.norm(rhs[k]) for k in range(2))
        e0 = max(np.linalg.norm(x0[k] - x[0, k]) / np.linalg.norm(x[0, k]) for k in range(2))
        p.set_guess(x0[None])
        st1 = p.solve_device(tol=tol, mode=mode, max_iters=5000)
        rows.append({"seed": s, "iters_plain": st0["inner_iters"], "iters_learned": st1["inner_iters"],
                     "res_plain": st0["rel_residual"], "res_learned": st1["rel_residual"],
                     "converged": bool(st0["converged"] and st1["converged"]), "initial_rel_residual": r0,
                     "initial_rel_error": e0})
        p.close()
    return rows


def main():
    import argparse
    import json
    ap = argparse.ArgumentParser(description="train the learned warm start and report the ablation")
    ap.add_argument("--train", type=int, default=96)
    ap.add_argument("--test", type=int, default=16)
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--width", type=int, default=32)
    ap.add_argument("--save", default="")
    a = ap.parse_args()
    t0 = time.time()
    data = [make_sample(1000 + i)[:2] for i in range(a.train)]
    t1 = time.time()
    net = WarmStartNet(width=a.width)
    hist = train(net, data, epochs=a.epochs, lr=a.lr)
    t2 = time.time()
    rows = evaluate(net, [900000 + i for i in range(a.test)])
    ip = np.mean([r["iters_plain"] for r in rows])
    il = np.mean([r["iters_learned"] for r in rows])
    print(json.dumps({"train_models": a.train, "data_s": t1 - t0, "train_s": t2 - t1, "loss_first": hist[0],
                      "loss_last": hist[-1], "epochs": len(hist), "mean_iters_plain": ip, "mean_iters_learned": il,
                      "iteration_ratio": il / ip, "all_converged": all(r["converged"] for r in rows),
                      "mean_initial_rel_residual": float(np.mean([r["initial_rel_residual"] for r in rows])),
                      "mean_initial_rel_error": float(np.mean([r["initial_rel_error"] for r in rows])),
                      "rows": rows}))
    if a.save:
        np.save(a.save, net.params())


if __name__ == "__main__":
    main()
