"""CPU oracle for the MoVFEM_3DMT hot path -- TEST INFRASTRUCTURE ONLY.

A plain-C restatement of the reference's Fortran assembly, numbering and
post-processing (see ``movfem_oracle.h`` for the file:line map), wrapped with ctypes,
plus an FP64 direct solve with SciPy's SuperLU standing in for MUMPS 4.10 (the
reference's third-party solver; it is not vendored and not installed here).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
use this package, and only to compare against.  The product library never loads it.

Parity pin: the reference (Fortran + MUMPS) cannot be compiled on either machine, so
no reference outputs exist; "parity unpinned" against the reference itself.  The
oracle is pinned by known-answer tests and committed fixtures under tests/golden.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB = os.path.join(_BUILD, "libmovfem_oracle.so")
_lock = threading.Lock()
_lib = None

Q_LIN_DZETA, Q_FP32_CONST, Q_GPML_LAG, Q_ALL = 1, 2, 4, 7


def build(force: bool = False) -> str:
    src = os.path.join(_HERE, "movfem_oracle.c")
    os.makedirs(_BUILD, exist_ok=True)
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(src):
        tmp = _LIB + f".{os.getpid()}.tmp"
        subprocess.check_call(["gcc", "-O2", "-std=c99", "-ffp-contract=off", "-fPIC", "-shared", "-o", tmp, src, "-lm"])
        os.replace(tmp, _LIB)
    return _LIB


class _Mesh(ctypes.Structure):
    _fields_ = [
        ("nodes_per_elem", ctypes.c_int32), ("nx", ctypes.c_int32), ("ny", ctypes.c_int32),
        ("nz", ctypes.c_int32), ("xp", ctypes.c_void_p), ("yp", ctypes.c_void_p), ("zp", ctypes.c_void_p),
        ("sigma", ctypes.c_void_p), ("mu", ctypes.c_void_p), ("dirichlet", ctypes.c_int32),
        ("inimod", ctypes.c_int32), ("gpml_sch", ctypes.c_int32), ("a0", ctypes.c_double),
        ("b0", ctypes.c_double), ("nn", ctypes.c_double), ("nextd", ctypes.c_int32),
        ("nzl_top", ctypes.c_int32), ("nzl_air", ctypes.c_int32), ("ztop", ctypes.c_double),
        ("h_sigma", ctypes.c_double), ("nlayers", ctypes.c_int32), ("l_sigma", ctypes.c_void_p),
        ("l_dz", ctypes.c_void_p), ("quirks", ctypes.c_int32),
    ]


def lib():
    global _lib
    with _lock:
        if _lib is None:
            L = ctypes.CDLL(build())
            P, I32, I64, D = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
            L.orc_numbering.restype = I32
            L.orc_numbering.argtypes = [P, P]
            L.orc_slot_map.restype = I64
            L.orc_slot_map.argtypes = [P, P, P]
            L.orc_coo_coords.restype = ctypes.c_int
            L.orc_coo_coords.argtypes = [P, P, P, I64, P, P]
            L.orc_element.restype = ctypes.c_int
            L.orc_element.argtypes = [P, I64, D, I32, P, P, P, P]
            L.orc_assemble.restype = ctypes.c_int
            L.orc_assemble.argtypes = [P, P, P, I64, I32, D, I32, P, P]
            L.orc_receivers.restype = ctypes.c_int
            L.orc_receivers.argtypes = [P, P, I32, D, P, I32, P, P, P, P, P, P, P]
            L.orc_node_fields.restype = ctypes.c_int
            L.orc_node_fields.argtypes = [P, P, I32, D, P, P, P, P, P, P]
            L.orc_check_sharing.restype = D
            L.orc_check_sharing.argtypes = [P]
            L.orc_set_pmass.restype = None
            L.orc_set_pmass.argtypes = [ctypes.c_int, D]
            L.orc_map_model.restype = ctypes.c_int
            L.orc_map_model.argtypes = [P, P, D, P, P]
            _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data if a is not None else None


class _Model(ctypes.Structure):
    _fields_ = [
        ("mx", ctypes.c_int32), ("my", ctypes.c_int32), ("mz", ctypes.c_int32), ("xm", ctypes.c_void_p),
        ("ym", ctypes.c_void_p), ("zm", ctypes.c_void_p), ("isigma", ctypes.c_int32), ("ijsigma", ctypes.c_void_p),
        ("sigma", ctypes.c_void_p), ("imu", ctypes.c_int32), ("ijmu", ctypes.c_void_p), ("mu", ctypes.c_void_p),
    ]


def map_model(mesh, model, omega):
    """Nodal sigma [npt, 6] complex and mu [npt, 6] of ``mesh``'s grid from the inner
    geomodel ``model`` (a ``movfem_gb300.mesh.GeoModel``), restating innermodel_gqg /
    min_dd_inner / assign_model (geometry.f90:804-1085) sequentially."""
    a = model.c_arrays()
    dummy = np.zeros(1)
    o = Oracle.__new__(Oracle)
    o.mesh, o.quirks = mesh, mesh.quirks
    o.xp = np.ascontiguousarray(mesh.xp, dtype=np.float64)
    o.yp = np.ascontiguousarray(mesh.yp, dtype=np.float64)
    o.zp = np.ascontiguousarray(mesh.zp, dtype=np.float64)
    o.sigma, o.mu, o.l_sigma, o.l_dz = dummy, dummy, None, None
    md = _Model(a["mx"], a["my"], a["mz"], _ptr(a["xm"]), _ptr(a["ym"]), _ptr(a["zm"]), a["isigma"],
                _ptr(a["ijsigma"]), _ptr(a["sigma"]), a["imu"], _ptr(a["ijmu"]), _ptr(a["mu"]))
    sigma = np.empty((mesh.npt, 6), dtype=np.complex128)
    mu = np.empty((mesh.npt, 6))
    rc = lib().orc_map_model(o._s(), ctypes.byref(md), float(omega), _ptr(sigma), _ptr(mu))
    if rc != 0:
        raise RuntimeError(f"oracle model mapping failed rc={rc}")
    return sigma, mu


def rem_zeros(ia, ja, a):
    """find_zeros + rem_zeros (global_assembly.f90:123-150) as MoVFEM_3DMT.f90 applies them
    before the MUMPS call (MoVFEM_3DMT.f90:85-97): the entries whose complex value equals
    0 + 0i (so -0.0 too) are left out, the others keep their order.  Returns
    (ia, ja, a, number dropped)."""
    keep = a != 0
    return ia[keep], ja[keep], a[keep], int(a.size - keep.sum())


class Oracle:
    """Oracle bound to one mesh (keeps the numpy buffers alive)."""

    def __init__(self, mesh, sigma=None, quirks=None):
        self.mesh = mesh
        self.xp = np.ascontiguousarray(mesh.xp, dtype=np.float64)
        self.yp = np.ascontiguousarray(mesh.yp, dtype=np.float64)
        self.zp = np.ascontiguousarray(mesh.zp, dtype=np.float64)
        self.set_sigma(mesh.sigma if sigma is None else sigma)
        self.mu = np.ascontiguousarray(mesh.mu, dtype=np.float64)
        self.l_sigma = None if mesh.l_sigma is None else np.ascontiguousarray(mesh.l_sigma, dtype=np.float64)
        self.l_dz = None if mesh.l_dz is None else np.ascontiguousarray(mesh.l_dz, dtype=np.float64)
        self.quirks = mesh.quirks if quirks is None else quirks
        self._gne = None
        self._nz = None

    def set_sigma(self, sigma):
        self.sigma = np.ascontiguousarray(sigma, dtype=np.complex128)
        self._struct = None

    def _s(self):
        m = self.mesh
        s = _Mesh(m.nodes_per_elem, m.nx, m.ny, m.nz, _ptr(self.xp), _ptr(self.yp), _ptr(self.zp),
                  _ptr(self.sigma), _ptr(self.mu), m.dirichlet, m.inimod, m.gpml_sch, m.a0, m.b0, m.nn,
                  m.nextd, m.nzl_top, m.nzl_air, m.ztop, m.h_sigma,
                  0 if self.l_sigma is None else self.l_sigma.size, _ptr(self.l_sigma), _ptr(self.l_dz),
                  self.quirks)
        self._struct = s
        return ctypes.byref(s)

    def numbering(self):
        """gne in the reference's layout gne(ne, me) (column-major) -> returned as
        [me, ne] int32 and nne."""
        if self._gne is None:
            m = self.mesh
            gne = np.zeros((m.me, m.ne), dtype=np.int32)
            nne = lib().orc_numbering(self._s(), _ptr(gne))
            if nne < 0:
                raise RuntimeError("oracle numbering failed")
            self._gne, self.nne = gne, int(nne)
        return self._gne, self.nne

    def slot_map(self):
        if self._nz is None:
            m = self.mesh
            gne, _ = self.numbering()
            nz = np.empty(m.ne * m.me * m.me, dtype=np.int32)
            nnze = lib().orc_slot_map(self._s(), _ptr(gne), _ptr(nz))
            if nnze < 0:
                raise RuntimeError("oracle slot map failed")
            self._nz, self.nnze = nz, int(nnze)
        return self._nz, self.nnze

    def coo_coords(self):
        gne, _ = self.numbering()
        nz, nnze = self.slot_map()
        ia = np.empty(nnze, dtype=np.int32)
        ja = np.empty(nnze, dtype=np.int32)
        if lib().orc_coo_coords(self._s(), _ptr(gne), _ptr(nz), nnze, _ptr(ia), _ptr(ja)) != 0:
            raise RuntimeError("slot with two coordinates")
        return ia, ja

    def element(self, e, omega, ifreq=0):
        me = self.mesh.me
        K = np.empty((me, me))
        M = np.empty((me, me))
        b = np.empty((me, 2), dtype=np.complex128)
        pml = np.zeros(3, dtype=np.int32)
        rc = lib().orc_element(self._s(), int(e), float(omega), int(ifreq), _ptr(K), _ptr(M), _ptr(b), _ptr(pml))
        if rc != 0:
            raise RuntimeError(f"oracle element failed rc={rc}")
        return K, M, b, pml

    def assemble(self, omega, ifreq=0):
        """Pre-sort COO values a[nnze] and RHS[2, nne] (pol-major)."""
        gne, nne = self.numbering()
        nz, nnze = self.slot_map()
        a = np.empty(nnze, dtype=np.complex128)
        rhs = np.empty(2 * nne, dtype=np.complex128)
        rc = lib().orc_assemble(self._s(), _ptr(gne), _ptr(nz), nnze, nne, float(omega), int(ifreq), _ptr(a),
                                _ptr(rhs))
        if rc != 0:
            raise RuntimeError(f"oracle assembly failed rc={rc}")
        return a, rhs.reshape(2, nne)

    def matrix(self, omega, ifreq=0):
        """Full symmetric complex CSR (scipy) and RHS [2, nne]."""
        import scipy.sparse as sp
        ia, ja = self.coo_coords()
        a, rhs = self.assemble(omega, ifreq)
        n = self.nne
        low = sp.coo_matrix((a, (ia - 1, ja - 1)), shape=(n, n)).tocsr()
        diag = sp.diags(low.diagonal())
        full = (low + low.T - diag).tocsr()
        full.sort_indices()
        return full, rhs

    def solve_direct(self, omega, ifreq=0):
        """FP64 direct solve (SuperLU standing in for MUMPS), both polarisations."""
        import scipy.sparse.linalg as spla
        A, rhs = self.matrix(omega, ifreq)
        lu = spla.splu(A.tocsc())
        x = np.stack([lu.solve(rhs[0]), lu.solve(rhs[1])])
        return x, A, rhs

    def receivers(self, omega, x, rx=None):
        """E, H [nrx, 2, 3], Z [nrx, 4], rho [nrx, 4], phi [nrx, 4] at receivers."""
        gne, nne = self.numbering()
        rx = self.mesh.rx if rx is None else np.asarray(rx, dtype=np.float64)
        xr = np.ascontiguousarray(rx[:, 0])
        yr = np.ascontiguousarray(rx[:, 1])
        nrx = xr.size
        xs = np.ascontiguousarray(np.asarray(x, dtype=np.complex128).reshape(-1))
        E = np.empty((nrx, 2, 3), dtype=np.complex128)
        H = np.empty((nrx, 2, 3), dtype=np.complex128)
        Z = np.empty((nrx, 4), dtype=np.complex128)
        rho = np.empty((nrx, 4))
        phi = np.empty((nrx, 4))
        rc = lib().orc_receivers(self._s(), _ptr(gne), nne, float(omega), _ptr(xs), nrx, _ptr(xr), _ptr(yr),
                                 _ptr(E), _ptr(H), _ptr(Z), _ptr(rho), _ptr(phi))
        if rc != 0:
            raise RuntimeError(f"oracle receivers failed rc={rc}")
        return E, H, Z, rho, phi

    def node_fields(self, omega, x):
        """E, H [npt, 2, 3], Z [npt, 4], rho [npt, 4], phi [npt, 4] at every node."""
        gne, nne = self.numbering()
        npt = self.mesh.npt
        xs = np.ascontiguousarray(np.asarray(x, dtype=np.complex128).reshape(-1))
        E = np.empty((npt, 2, 3), dtype=np.complex128)
        H = np.empty((npt, 2, 3), dtype=np.complex128)
        Z = np.empty((npt, 4), dtype=np.complex128)
        rho = np.empty((npt, 4))
        phi = np.empty((npt, 4))
        rc = lib().orc_node_fields(self._s(), _ptr(gne), nne, float(omega), _ptr(xs), _ptr(E), _ptr(H), _ptr(Z),
                                   _ptr(rho), _ptr(phi))
        if rc != 0:
            raise RuntimeError(f"oracle node fields failed rc={rc}")
        return E, H, Z, rho, phi

    def check_sharing(self):
        return lib().orc_check_sharing(self._s())
