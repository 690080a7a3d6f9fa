"""Host-side mirror of the reference's hot-path call sites over the C-ABI.

The reference's Fortran driver (MoVFEM_3DMT/src/MoVFEM_3DMT.f90) calls, per frequency,
``global_vfem`` (:82) to assemble, ``zmumps`` with job=6 (:113-115) to solve both
polarisations, and ``node_solution`` + ``write_receiver_data`` (:123-127) for E, H, Z,
rho and phi.  :class:`MTProblem` exposes the same steps on the GPU library
(``include/movfem_gpu.h``): :meth:`assemble` (all frequencies at once),
:meth:`solve` (replaces zmumps), :meth:`impedance` (receiver Z / rho / phi), plus the
parity hooks :meth:`numbering`, :meth:`export_coo`, :meth:`export_rhs`,
:meth:`element_matrices` and :meth:`spmv`.

Errors: every C-ABI status other than 0 raises :class:`MVFError` carrying the
library's message (the reference prints and ``stop``s).  There is no CPU fallback:
constructing a problem without the CUDA library or a GPU raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

MVF_OK, E_ARG, E_CUDA, E_SINGULAR, E_NOCONV, E_STATE, E_RECEIVER, E_NOMEM, E_UNSUPPORTED = 0, -1, -2, -3, -4, -5, -6, -7, -8
MODE_MIXED, MODE_FP64 = 0, 1


class MVFError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"movfem_gpu error {code}: {msg}")
        self.code = code


class _Mesh(ctypes.Structure):
    _fields_ = [
        ("nodes_per_elem", ctypes.c_int32), ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("xp", ctypes.c_void_p), ("yp", ctypes.c_void_p), ("zp", ctypes.c_void_p), ("sigma", ctypes.c_void_p),
        ("mu", ctypes.c_void_p), ("dirichlet", ctypes.c_int32), ("inimod", ctypes.c_int32),
        ("gpml_sch", ctypes.c_int32), ("a0", ctypes.c_double), ("b0", ctypes.c_double), ("nn", ctypes.c_double),
        ("nextd", ctypes.c_int32), ("nzl_top", ctypes.c_int32), ("nzl_air", ctypes.c_int32),
        ("ztop", ctypes.c_double), ("quirks", ctypes.c_int32), ("h_sigma", ctypes.c_double),
        ("nlayers", ctypes.c_int32), ("l_sigma", ctypes.c_void_p), ("l_dz", ctypes.c_void_p),
    ]


class Stats(ctypes.Structure):
    _fields_ = [("outer_iters", ctypes.c_int32), ("inner_iters", ctypes.c_int32), ("rel_residual", ctypes.c_double),
                ("seconds", ctypes.c_double), ("bytes_moved", ctypes.c_int64), ("stagnated", ctypes.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


EXPORTS = ["mvf_create", "mvf_destroy", "mvf_last_error", "mvf_sizes", "mvf_numbering", "mvf_set_sigma",
           "mvf_assemble", "mvf_export_coo", "mvf_export_coo_nz", "mvf_export_rhs", "mvf_element_matrices", "mvf_solve",
           "mvf_impedance", "mvf_spmv", "mvf_profile_spmm", "mvf_kernel_launches", "mvf_spmv_noalloc",
           "mvf_spmm_tuning", "mvf_spmm_variant", "mvf_set_guess", "mvf_net_create", "mvf_net_destroy",
           "mvf_net_last_error", "mvf_net_num_params", "mvf_net_get_params", "mvf_net_set_params", "mvf_net_forward",
           "mvf_net_gradients", "mvf_net_train_step", "mvf_node_fields", "mvf_solve_many", "mvf_profile_patch",
           "mvf_set_solver", "mvf_patch_arithmetic", "mvf_map_model", "mvf_set_preconditioner", "mvf_mg_levels", "mvf_mg_apply_once", "mvf_profile_mg", "mvf_set_batching", "mvf_set_surface_correction", "mvf_band_solve",
           "mvf_grid_3d", "mvf_grid_get_info", "mvf_grid_export", "mvf_grid_destroy"]
_NOT_STATUS = ("mvf_destroy", "mvf_last_error", "mvf_create", "mvf_kernel_launches", "mvf_spmm_tuning",
               "mvf_net_destroy", "mvf_net_last_error", "mvf_net_num_params", "mvf_patch_arithmetic",
               "mvf_grid_destroy")
SPMM_VARIANTS = {0: "chunked", 1: "direct", 2: "vec/G=4", 3: "vec/G=8", 4: "vec/G=16", 5: "vec/G=32"}


def kernel_launches() -> int:
    """Kernels launched by the library in this process so far."""
    return int(load().mvf_kernel_launches())

_lib = None


def library_path(build: bool = True) -> str:
    return _build.build() if build else _build.LIB


def load(build: bool = True):
    """Load libmovfem_gpu.so (building it first if stale)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path(build)
    if not os.path.exists(path):
        raise RuntimeError(f"CUDA library missing: {path}")
    L = ctypes.CDLL(path)
    P, I32, I64, D = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_double
    L.mvf_create.argtypes = [ctypes.POINTER(P), P, I32]
    L.mvf_create.restype = ctypes.c_int
    L.mvf_destroy.argtypes = [P]
    L.mvf_destroy.restype = None
    L.mvf_last_error.argtypes = [P]
    L.mvf_last_error.restype = ctypes.c_char_p
    L.mvf_sizes.argtypes = [P, P, P, P, P, P]
    L.mvf_numbering.argtypes = [P, P]
    L.mvf_set_sigma.argtypes = [P, P]
    L.mvf_assemble.argtypes = [P, I32, P, P, I32]
    L.mvf_export_coo.argtypes = [P, I32, P, P, P, P]
    L.mvf_export_coo_nz.argtypes = [P, I32, P, P, P, P, P]
    L.mvf_export_rhs.argtypes = [P, I32, P]
    L.mvf_element_matrices.argtypes = [P, I64, I64, I32, P, P, P]
    L.mvf_solve.argtypes = [P, P, D, I32, I32, P]
    L.mvf_impedance.argtypes = [P, I32, P, P, P, P, P, P, P]
    L.mvf_spmv.argtypes = [P, I32, P, P]
    L.mvf_profile_spmm.argtypes = [P, I32, I32, P, P]
    L.mvf_spmv_noalloc.argtypes = [P, I32, P, P]
    L.mvf_kernel_launches.argtypes = []
    L.mvf_kernel_launches.restype = I64
    L.mvf_spmm_variant.argtypes = [P, I32, I32, I32, I32, P, P]
    L.mvf_set_guess.argtypes = [P, P]
    L.mvf_node_fields.argtypes = [P, P, P, P, P, P]
    L.mvf_solve_many.argtypes = [P, I32, D, I32, I32, P, I32]
    L.mvf_profile_patch.argtypes = [P, I32, I32, P, P]
    L.mvf_set_solver.argtypes = [P, I32, I32, I32]
    L.mvf_set_preconditioner.argtypes = [P, I32, ctypes.c_double, ctypes.c_double]
    L.mvf_mg_levels.argtypes = [P, P, P, I32]
    L.mvf_mg_apply_once.argtypes = [P, I32, I32, P, P]
    L.mvf_profile_mg.argtypes = [P, I32, P, P]
    L.mvf_set_batching.argtypes = [P, I32]
    L.mvf_set_surface_correction.argtypes = [P, I32]
    L.mvf_band_solve.argtypes = [I64, I32, I32, P, P, I32]
    L.mvf_patch_arithmetic.argtypes = [P]
    L.mvf_patch_arithmetic.restype = I32
    L.mvf_net_create.argtypes = [ctypes.POINTER(P), I32, I32, I32, I32, P, ctypes.c_uint64, I32]
    L.mvf_net_destroy.argtypes = [P]
    L.mvf_net_destroy.restype = None
    L.mvf_net_last_error.argtypes = [P]
    L.mvf_net_last_error.restype = ctypes.c_char_p
    L.mvf_net_num_params.argtypes = [P]
    L.mvf_net_num_params.restype = I64
    L.mvf_net_get_params.argtypes = [P, P]
    L.mvf_net_set_params.argtypes = [P, P]
    L.mvf_net_forward.argtypes = [P, I32, I32, I32, P, P]
    L.mvf_net_gradients.argtypes = [P, I32, I32, I32, P, P, P, P]
    L.mvf_net_train_step.argtypes = [P, I32, I32, I32, P, P, ctypes.c_float, P]
    L.mvf_spmm_tuning.argtypes = [P]
    L.mvf_spmm_tuning.restype = ctypes.c_char_p
    L.mvf_map_model.argtypes = [P, P, D, P, P, P, I32]
    L.mvf_grid_3d.argtypes = [P, ctypes.POINTER(P)]
    L.mvf_grid_get_info.argtypes = [P, P]
    L.mvf_grid_export.argtypes = [P, P, P, P, P]
    L.mvf_grid_destroy.argtypes = [P]
    L.mvf_grid_destroy.restype = None
    for n in EXPORTS:
        if n not in _NOT_STATUS:
            getattr(L, n).restype = ctypes.c_int
    _lib = L
    return L


def _p(a):
    return None if a is None else a.ctypes.data


class _GridIn(ctypes.Structure):
    _fields_ = [
        ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double), ("high", ctypes.c_double),
        ("depth", ctypes.c_double), ("nodes_per_elem", ctypes.c_int32), ("sigma_bg", ctypes.c_double),
        ("nsr", ctypes.c_int32), ("rx", ctypes.c_void_p), ("nsf0", ctypes.c_int32), ("nsp", ctypes.c_void_p),
        ("pts", ctypes.c_void_p), ("mx", ctypes.c_int32), ("my", ctypes.c_int32), ("mz", ctypes.c_int32),
        ("xm", ctypes.c_void_p), ("ym", ctypes.c_void_p), ("zm", ctypes.c_void_p), ("nf", ctypes.c_int32),
        ("freqs", ctypes.c_void_p),
    ]


class GridInfo(ctypes.Structure):
    _fields_ = [
        ("nodes_per_elem", ctypes.c_int32), ("nextd", ctypes.c_int32), ("nsf", ctypes.c_int32),
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32), ("nnx", ctypes.c_int64),
        ("nny", ctypes.c_int64), ("nnz", ctypes.c_int64), ("npt", ctypes.c_int64), ("nzl_top", ctypes.c_int32),
        ("nzl_air", ctypes.c_int32), ("x0", ctypes.c_double), ("y0", ctypes.c_double), ("z0", ctypes.c_double),
        ("ztop", ctypes.c_double), ("skin_depth", ctypes.c_double), ("nd", ctypes.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def band_solve(a, b, kl: int, ku: int):
    """Test hook: the surface correction's band LU (``mvf_band_solve``) on the band
    [-kl, ku] of the dense matrix ``a`` [n, n], for ``b`` [n] or [n, nrhs]."""
    L = load()
    n = a.shape[0]
    af = np.asfortranarray(a, dtype=np.float64)
    bb = np.ascontiguousarray(np.asarray(b, dtype=np.float64).reshape(n, -1).T)
    rc = L.mvf_band_solve(n, kl, ku, af.ctypes.data, bb.ctypes.data, bb.shape[0])
    if rc != 0:
        raise MVFError(rc, "band solve failed")
    return bb.T.reshape(np.shape(b))


def grid_3d(dx, dy, dz, high, depth, nodes_per_elem, sigma_bg, rx, interfaces, xm, ym, zm, freqs):
    """Node grid of the model domain (``mvf_grid_3d``: grid_3d, geometry.f90:48-118, on
    the host in native code).  ``rx`` [nsr, 3]; ``interfaces``: one [n, 3] array of
    points per input interface, deepest first (read_top_interfaces order,
    read_input.f90:72-101); ``xm`` [mx], ``ym`` [my], ``zm`` [mx, my, mz] the inner
    model's coordinates; ``freqs`` in Hz.  Returns ``(info, xp, yp, zp, nzl)``: ``info``
    a dict of :class:`GridInfo` (the grid coordinates are the input's minus
    ``(x0, y0, z0)``), ``zp`` of node ``(i*nny + j)*nnz + k``."""
    L = load()
    rxa = np.ascontiguousarray(rx, dtype=np.float64).reshape(-1, 3)
    ifs = [np.ascontiguousarray(p, dtype=np.float64).reshape(-1, 3) for p in interfaces]
    nsp = np.array([p.shape[0] for p in ifs], dtype=np.int32)
    pts = np.ascontiguousarray(np.concatenate(ifs, axis=0))
    xma = np.ascontiguousarray(xm, dtype=np.float64)
    yma = np.ascontiguousarray(ym, dtype=np.float64)
    zma = np.ascontiguousarray(zm, dtype=np.float64)
    fa = np.ascontiguousarray(np.atleast_1d(freqs), dtype=np.float64)
    gi = _GridIn(float(dx), float(dy), float(dz), float(high), float(depth), int(nodes_per_elem), float(sigma_bg),
                 rxa.shape[0], _p(rxa), len(ifs), _p(nsp), _p(pts), xma.size, yma.size, zma.size // (xma.size * yma.size),
                 _p(xma), _p(yma), _p(zma), fa.size, _p(fa))
    h = ctypes.c_void_p()
    rc = L.mvf_grid_3d(ctypes.byref(gi), ctypes.byref(h))
    if rc != 0:
        raise MVFError(rc, L.mvf_last_error(None).decode())
    try:
        info = GridInfo()
        L.mvf_grid_get_info(h, ctypes.byref(info))
        xp = np.empty(info.nnx)
        yp = np.empty(info.nny)
        zp = np.empty(info.npt)
        nzl = np.empty(info.nsf, dtype=np.int32)
        L.mvf_grid_export(h, _p(xp), _p(yp), _p(zp), _p(nzl))
    finally:
        L.mvf_grid_destroy(h)
    return info.as_dict(), xp, yp, zp, nzl


class _Model(ctypes.Structure):
    _fields_ = [
        ("mx", ctypes.c_int32), ("my", ctypes.c_int32), ("mz", ctypes.c_int32), ("xm", ctypes.c_void_p),
        ("ym", ctypes.c_void_p), ("zm", ctypes.c_void_p), ("isigma", ctypes.c_int32), ("ijsigma", ctypes.c_void_p),
        ("sigma", ctypes.c_void_p), ("imu", ctypes.c_int32), ("ijmu", ctypes.c_void_p), ("mu", ctypes.c_void_p),
    ]


def map_model(mesh, model, omega: float, device: int = -1, timed: bool = False):
    """Nodal conductivity and permeability of ``mesh``'s grid from the inner geomodel
    ``model`` (:class:`movfem_gb300.mesh.GeoModel`) on the GPU (``mvf_map_model``,
    replacing innermodel_gqg / min_dd_inner / assign_model, geometry.f90:804-1085,
    which grid_3d calls at geometry.f90:106).  ``omega`` is the grid-time angular
    frequency 2*pi*f_1.  Returns sigma [npt, 6] complex128 and mu [npt, 6] (plus the
    kernels' device seconds when ``timed``)."""
    L = load()
    xp = np.ascontiguousarray(mesh.xp, dtype=np.float64)
    yp = np.ascontiguousarray(mesh.yp, dtype=np.float64)
    zp = np.ascontiguousarray(mesh.zp, dtype=np.float64)
    g = _Mesh(mesh.nodes_per_elem, mesh.nx, mesh.ny, mesh.nz, _p(xp), _p(yp), _p(zp), None, None,
              mesh.dirichlet, mesh.inimod, mesh.gpml_sch, mesh.a0, mesh.b0, mesh.nn, mesh.nextd, mesh.nzl_top,
              mesh.nzl_air, mesh.ztop, mesh.quirks, mesh.h_sigma, 0, None, None)
    a = model.c_arrays()
    md = _Model(a["mx"], a["my"], a["mz"], _p(a["xm"]), _p(a["ym"]), _p(a["zm"]), a["isigma"], _p(a["ijsigma"]),
                _p(a["sigma"]), a["imu"], _p(a["ijmu"]), _p(a["mu"]))
    sigma = np.empty((mesh.npt, 6), dtype=np.complex128)
    mu = np.empty((mesh.npt, 6))
    sec = ctypes.c_double(0.0)
    rc = L.mvf_map_model(ctypes.byref(g), ctypes.byref(md), float(omega), _p(sigma), _p(mu), ctypes.byref(sec),
                         device)
    if rc != 0:
        raise MVFError(rc, L.mvf_last_error(None).decode())
    return (sigma, mu, sec.value) if timed else (sigma, mu)


def solve_many(problems, tol: float = 1e-10, mode: int = 0, max_iters: int = 5000, nthreads: int = 8):
    """Solve the assembled systems of several :class:`MTProblem` concurrently
    (``mvf_solve_many``); solutions stay on the device.  Returns per-problem
    statistics with a ``converged`` flag."""
    L = load()
    n = len(problems)
    hs = (ctypes.c_void_p * n)(*[p.h for p in problems])
    st = (Stats * n)()
    rc = L.mvf_solve_many(hs, n, tol, mode, max_iters, st, nthreads)
    if rc not in (0, E_NOCONV):
        raise MVFError(rc, " / ".join(L.mvf_last_error(p.h).decode() for p in problems))
    out = []
    for i, p in enumerate(problems):
        d = st[i].as_dict()
        d["converged"] = d["rel_residual"] <= tol or bool(d["stagnated"])
        out.append(d)
    return out


class MTProblem:
    """One model on the GPU (the reference's module state after ``initialize_vfem``)."""

    def __init__(self, mesh, device: int = -1):
        self.L = load()
        self.mesh = mesh
        xp = np.ascontiguousarray(mesh.xp, dtype=np.float64)
        yp = np.ascontiguousarray(mesh.yp, dtype=np.float64)
        zp = np.ascontiguousarray(mesh.zp, dtype=np.float64)
        sg = np.ascontiguousarray(mesh.sigma, dtype=np.complex128)
        mu = np.ascontiguousarray(mesh.mu, dtype=np.float64)
        ls = None if mesh.l_sigma is None else np.ascontiguousarray(mesh.l_sigma, dtype=np.float64)
        ld = None if mesh.l_dz is None else np.ascontiguousarray(mesh.l_dz, dtype=np.float64)
        m = _Mesh(mesh.nodes_per_elem, mesh.nx, mesh.ny, mesh.nz, _p(xp), _p(yp), _p(zp), _p(sg), _p(mu),
                  mesh.dirichlet, mesh.inimod, mesh.gpml_sch, mesh.a0, mesh.b0, mesh.nn, mesh.nextd, mesh.nzl_top,
                  mesh.nzl_air, mesh.ztop, mesh.quirks, mesh.h_sigma, 0 if ls is None else ls.size, _p(ls), _p(ld))
        h = ctypes.c_void_p()
        rc = self.L.mvf_create(ctypes.byref(h), ctypes.byref(m), device)
        self.h = h
        if rc != 0:
            msg = self.L.mvf_last_error(h).decode()
            self.L.mvf_destroy(h)
            self.h = None
            raise MVFError(rc, msg)
        nne = ctypes.c_int32()
        nnz = ctypes.c_int64()
        nlo = ctypes.c_int64()
        me = ctypes.c_int32()
        ne = ctypes.c_int64()
        self._chk(self.L.mvf_sizes(h, ctypes.byref(nne), ctypes.byref(nnz), ctypes.byref(nlo), ctypes.byref(me),
                                   ctypes.byref(ne)))
        self.nne, self.nnz, self.nnz_lower, self.me, self.ne = nne.value, nnz.value, nlo.value, me.value, ne.value
        self.omega = None

    def _chk(self, rc):
        if rc != 0:
            raise MVFError(rc, self.L.mvf_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.L.mvf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def numbering(self):
        gne = np.empty((self.me, self.ne), dtype=np.int32)
        self._chk(self.L.mvf_numbering(self.h, _p(gne)))
        return gne

    def set_sigma(self, sigma):
        s = np.ascontiguousarray(sigma, dtype=np.complex128)
        self._chk(self.L.mvf_set_sigma(self.h, _p(s)))

    def assemble(self, omega, sigma_f=None, ifreq0: int = 0):
        om = np.ascontiguousarray(np.atleast_1d(omega), dtype=np.float64)
        sf = None if sigma_f is None else np.ascontiguousarray(sigma_f, dtype=np.complex128)
        self._chk(self.L.mvf_assemble(self.h, om.size, _p(om), _p(sf), ifreq0))
        self.omega = om

    def export_coo(self, f: int = 0, drop_zeros: bool = False):
        """Lower-triangle COO (1-based, row-major) of frequency ``f``.  ``drop_zeros``
        leaves out the exact-zero entries as ``find_zeros``/``rem_zeros`` do
        (global_assembly.f90:123-150) and records how many in ``self.zeros_dropped``."""
        n = ctypes.c_int64()
        z = ctypes.c_int64()
        if drop_zeros:
            call = lambda *a: self.L.mvf_export_coo_nz(self.h, f, *a, ctypes.byref(n), ctypes.byref(z))
        else:
            call = lambda *a: self.L.mvf_export_coo(self.h, f, *a, ctypes.byref(n))
        self._chk(call(None, None, None))
        ia = np.empty(n.value, dtype=np.int32)
        ja = np.empty(n.value, dtype=np.int32)
        a = np.empty(n.value, dtype=np.complex128)
        self._chk(call(_p(ia), _p(ja), _p(a)))
        if drop_zeros:
            self.zeros_dropped = z.value
        return ia, ja, a

    def export_rhs(self, f: int = 0):
        b = np.empty((2, self.nne), dtype=np.complex128)
        self._chk(self.L.mvf_export_rhs(self.h, f, _p(b)))
        return b

    def element_matrices(self, e0: int, count: int, f: int = 0):
        K = np.empty((count, self.me, self.me))
        M = np.empty((count, self.me, self.me))
        b = np.empty((count, self.me, 2), dtype=np.complex128)
        self._chk(self.L.mvf_element_matrices(self.h, e0, count, f, _p(K), _p(M), _p(b)))
        return K, M, b

    def solve(self, rhs=None, tol: float = 1e-10, mode: int = MODE_MIXED, max_iters: int = 5000,
              raise_noconv: bool = True):
        """Solve every assembled frequency and both polarisations.  Returns the
        solutions [nfreq, 2, nne] and the solver statistics."""
        if self.omega is None:
            self._chk(self.L.mvf_solve(self.h, None, tol, mode, max_iters, None))
        nf = self.omega.size
        if rhs is None:
            buf = np.stack([self.export_rhs(f) for f in range(nf)])
        else:
            buf = np.ascontiguousarray(rhs, dtype=np.complex128).reshape(nf, 2, self.nne).copy()
        st = Stats()
        rc = self.L.mvf_solve(self.h, _p(buf), tol, mode, max_iters, ctypes.byref(st))
        if not (rc == E_NOCONV and not raise_noconv):
            self._chk(rc)
        d = st.as_dict()
        d["converged"] = rc == 0
        return buf, d

    def solve_device(self, tol: float = 1e-10, mode: int = MODE_MIXED, max_iters: int = 5000):
        """Solve with the assembled right-hand sides; the solutions stay on the device
        (read them through :meth:`impedance`).  Returns the statistics."""
        st = Stats()
        rc = self.L.mvf_solve(self.h, None, tol, mode, max_iters, ctypes.byref(st))
        if rc not in (0, E_NOCONV):
            self._chk(rc)
        d = st.as_dict()
        d["converged"] = rc == 0
        return d

    def profile_spmm(self, f: int = 0, reps: int = 20):
        s = ctypes.c_double()
        b = ctypes.c_int64()
        self._chk(self.L.mvf_profile_spmm(self.h, f, reps, ctypes.byref(s), ctypes.byref(b)))
        return {"seconds_per_launch": s.value, "bytes_per_launch": b.value}

    def set_solver(self, restart: int = 0, mixed_passes: int = 0, patch_precision: int = 0):
        """FGMRES restart length, mixed-mode Gram-Schmidt passes and the patch
        preconditioner's arithmetic (1 FP64, 2 float-float); 0 keeps a setting."""
        self._chk(self.L.mvf_set_solver(self.h, restart, mixed_passes, patch_precision))

    def set_preconditioner(self, kind: int = 0, floor: float = 0.0, tau: float = -1.0):
        """36/54-DOF preconditioner: 0 multilevel (default), 1 one-level vertex patches;
        floor > 0 sets the multilevel operator's floor conductivity (S/m), tau >= 0 its
        shift tau diag(K).  Call before :meth:`assemble`."""
        self._chk(self.L.mvf_set_preconditioner(self.h, kind, floor, tau))

    def set_batching(self, per_frequency: bool):
        """Mixed mode: one batch per frequency (True) or all frequencies at once (False)."""
        self._chk(self.L.mvf_set_batching(self.h, int(per_frequency)))

    def set_surface_correction(self, on: bool = True):
        """After each multilevel cycle, solve the gradient modes of the layers around the
        earth's surface exactly with the true operator (``mvf_set_surface_correction``)."""
        self._chk(self.L.mvf_set_surface_correction(self.h, int(on)))

    def mg_levels(self):
        """Free DOFs of each level of the multilevel preconditioner (empty if unused)."""
        n = ctypes.c_int32()
        d = np.zeros(32, dtype=np.int32)
        self._chk(self.L.mvf_mg_levels(self.h, ctypes.byref(n), _p(d), 32))
        return d[:n.value].tolist()

    def mg_apply_once(self, f: int, r: np.ndarray) -> np.ndarray:
        """One multilevel preconditioner cycle for frequency f on r [n] or [n, R]."""
        r2 = np.ascontiguousarray(np.asarray(r, dtype=np.complex128).reshape(self.nne, -1))
        z = np.empty_like(r2)
        self._chk(self.L.mvf_mg_apply_once(self.h, f, r2.shape[1], _p(r2), _p(z)))
        return z.reshape(np.asarray(r).shape)

    def profile_mg(self, reps: int = 3):
        """Seconds and algorithmic bytes of one level-0 smoothing sweep (all frequencies)."""
        s = ctypes.c_double()
        b = ctypes.c_int64()
        self._chk(self.L.mvf_profile_mg(self.h, reps, ctypes.byref(s), ctypes.byref(b)))
        return {"seconds_per_sweep": s.value, "bytes_per_sweep": b.value}

    def patch_arithmetic(self) -> int:
        """0 no patches, 1 FP64, 2 float-float (as set up by the last inversion)."""
        return int(self.L.mvf_patch_arithmetic(self.h))

    def profile_patch(self, f: int = 0, reps: int = 5):
        """Seconds and algorithmic bytes of one vertex-patch preconditioner application."""
        s = ctypes.c_double()
        b = ctypes.c_int64()
        self._chk(self.L.mvf_profile_patch(self.h, f, reps, ctypes.byref(s), ctypes.byref(b)))
        return {"seconds_per_apply": s.value, "bytes_per_apply": b.value}

    def spmm_variant(self, f: int, variant: int, fp64: bool, x: np.ndarray) -> np.ndarray:
        """y = A_f x with one SpMM candidate; x: [nne, R] complex, R a power of two."""
        x = np.ascontiguousarray(x, dtype=np.complex128)
        y = np.empty_like(x)
        self._chk(self.L.mvf_spmm_variant(self.h, f, variant, int(fp64), x.shape[1], _p(x), _p(y)))
        return y

    def node_fields(self):
        """E, H [nfreq, npt, 2, 3], Z [nfreq, npt, 4], rho, phi [nfreq, npt, 4] at every
        node of the mesh (node_solution + z_rho_phi)."""
        nf, npt = self.omega.size, self.mesh.npt
        E = np.empty((nf, npt, 2, 3), dtype=np.complex128)
        H = np.empty((nf, npt, 2, 3), dtype=np.complex128)
        Z = np.empty((nf, npt, 4), dtype=np.complex128)
        rho = np.empty((nf, npt, 4))
        phi = np.empty((nf, npt, 4))
        self._chk(self.L.mvf_node_fields(self.h, _p(E), _p(H), _p(Z), _p(rho), _p(phi)))
        return E, H, Z, rho, phi

    def set_guess(self, x0: np.ndarray | None):
        """Initial guess [nfreq, 2, nne] complex for the following solves (None drops it)."""
        if x0 is None:
            self._chk(self.L.mvf_set_guess(self.h, None))
            return
        x0 = np.ascontiguousarray(x0, dtype=np.complex128)
        if x0.shape != (self.omega.size, 2, self.nne):
            raise ValueError(f"guess must be [{self.omega.size}, 2, {self.nne}]")
        self._chk(self.L.mvf_set_guess(self.h, _p(x0)))

    def spmm_tuning(self) -> str:
        """The SpMM variants the autotuner picked on this context so far."""
        return self.L.mvf_spmm_tuning(self.h).decode()

    def impedance(self, rx=None, with_fields: bool = False):
        rx = self.mesh.rx if rx is None else np.asarray(rx, dtype=np.float64)
        xr = np.ascontiguousarray(rx[:, 0])
        yr = np.ascontiguousarray(rx[:, 1])
        nf, nrx = self.omega.size, xr.size
        Z = np.empty((nf, nrx, 4), dtype=np.complex128)
        rho = np.empty((nf, nrx, 4))
        phi = np.empty((nf, nrx, 4))
        E = np.empty((nf, nrx, 2, 3), dtype=np.complex128) if with_fields else None
        H = np.empty((nf, nrx, 2, 3), dtype=np.complex128) if with_fields else None
        self._chk(self.L.mvf_impedance(self.h, nrx, _p(xr), _p(yr), _p(Z), _p(rho), _p(phi), _p(E), _p(H)))
        return (Z, rho, phi, E, H) if with_fields else (Z, rho, phi)

    def spmv_noalloc(self, f: int, x_dev_ptr: int, y_dev_ptr: int):
        """y = A_f x on device buffers ([2][nne] complex128) without any allocation
        by the library; see mvf_spmv_noalloc in include/movfem_gpu.h."""
        self._chk(self.L.mvf_spmv_noalloc(self.h, f, ctypes.c_void_p(x_dev_ptr), ctypes.c_void_p(y_dev_ptr)))

    def spmv(self, f: int, x):
        xx = np.ascontiguousarray(x, dtype=np.complex128).reshape(2, self.nne)
        y = np.empty_like(xx)
        self._chk(self.L.mvf_spmv(self.h, f, _p(xx), _p(y)))
        return y
