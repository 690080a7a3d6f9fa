"""Small seeded models used by the parity tests (sizes the oracle handles in seconds)."""
import math

import numpy as np

from movfem_gb300 import mesh as M


def box(nodes_per_elem, n=(3, 3, 2), d=(100.0, 80.0, 60.0), n_air=2, dirichlet=1, aniso=False, seed=0, nextd=0,
        gpml_sch=0):
    rng = np.random.Generator(np.random.PCG64(seed))
    blk = rng.uniform(0.2, 2.0)

    def sigma_fn(x, y, depth):
        return np.where(depth > 0.4 * n[2] * d[2], blk, 0.05) + 0 * x

    def full(x, y, depth):
        # random SPD tensor per node: R diag(l) R^T
        sh = x.shape
        lam = 10.0 ** rng.uniform(-3, 0, sh + (3,))
        a = rng.normal(size=sh + (3, 3))
        q, _ = np.linalg.qr(a)
        t = np.einsum("...ij,...j,...kj->...ik", q, lam, q)
        return np.stack([t[..., 0, 0], t[..., 0, 1], t[..., 0, 2], t[..., 1, 1], t[..., 1, 2], t[..., 2, 2]], -1)

    m = M.build_mesh(nodes_per_elem=nodes_per_elem, ncx=n[0], ncy=n[1], ncz_earth=n[2], dx=d[0], dy=d[1], dz=d[2],
                     n_air=n_air, dz_air=2 * d[2], nextd=nextd, sigma_fn=sigma_fn, omega1=2 * math.pi * 0.5,
                     dirichlet=dirichlet, gpml_sch=gpml_sch, full_tensor_fn=full if aniso else None,
                     rx=M.rx_grid(2, 0.0, n[0] * d[0]), freqs=np.array([0.5, 3.0]))
    return m


def topo(nodes_per_elem, n=(3, 3, 2), dirichlet=1, seed=1, nextd=0):
    rng = np.random.Generator(np.random.PCG64(seed))
    c = rng.uniform(0, 200, 2)

    def h(x, y):
        return 40.0 * np.exp(-((x - c[0]) ** 2 + (y - c[1]) ** 2) / (2 * 120.0 ** 2))

    m = M.build_mesh(nodes_per_elem=nodes_per_elem, ncx=n[0], ncy=n[1], ncz_earth=n[2], dx=100.0, dy=90.0, dz=70.0,
                     n_air=2, dz_air=140.0, nextd=nextd, sigma_fn=lambda x, y, d: 0.02 + 0 * x,
                     omega1=2 * math.pi, dirichlet=dirichlet, topo_fn=h, rx=M.rx_grid(2, 0.0, n[0] * 100.0),
                     freqs=np.array([1.0]))
    return m
