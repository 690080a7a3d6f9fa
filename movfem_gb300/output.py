"""Output writers in the reference's layouts.

SOLUTION.OUT: ``write_solution`` (solution.f90:71-205), whole-volume case
(``inner == 0``), fed by :meth:`movfem_gb300.api.MTProblem.node_fields`.
RECEIVER.OUT: ``write_receiver_data`` (receiver_data.f90:25-67), fed by
:meth:`movfem_gb300.api.MTProblem.impedance` with ``with_fields=True``.
SURFACE.OUT: ``write_surface_data`` (receiver_data.f90:69-109) on the surface nodes
that ``sur_data`` selects, fed by ``node_fields``.

SOLUTION.OUT, per frequency:
  * a list-directed header line ``vector-fem solution: <nf>``;
  * a '(24A15)' title line and one '(24es20.5)' record per node: Re/Im of E_x, E_y,
    E_z, then B_x, B_y, B_z (the reference prints H with the label B and unit factor 1),
    first polarisation then second;
  * a '(8A15)' title and one '(8es20.5)' record per node: Re/Im of Zxx, Zxy, Zyx, Zyy;
  * a '(8A15)' title and one '(8f20.5)' record per node: rho_a then phase.

Fortran edit descriptors are reproduced as follows: Aw right-justifies in w columns;
esw.d prints a one-digit mantissa, d decimals and a signed exponent of at least two
digits in w columns; fw.d prints d decimals in w columns.  List-directed output is
compiler-specific; the header follows gfortran's (a leading blank, the string, an
integer in 12 columns).
"""
from __future__ import annotations

import numpy as np

_TITLE_E = ["Re[Ex_(1)]", "Im[Ex_(1)]", "Re[Ey_(1)]", "Im[Ey_(1)]", "Re[Ez_(1)]", "Im[Ez_(1)]", "Re[Bx_(1)]",
            "Im[Bx_(1)]", "Re[By_(1)]", "Im[By_(1)]", "Re[Bz_(1)]", "Im[Bz_(1)]", "Re[Ex_(2)]", "Im[Ex_(2)]",
            "Re[Ey_(2)]", "Im[Ey_(2)]", "Re[Ez_(2)]", "Im[Ez_(2)]", "Re[Bx_(2)]", "Im[Bx_(2)]", "Re[By_(2)]",
            "Im[By_(2)]", "Re[Bz_(2)]", "Im[Bz_(2)]"]
_TITLE_Z = ["Re(Zxx)", "Im(Zxx)", "Re(Zxy)", "Im(Zxy)", "Re(Zyx)", "Im(Zyx)", "Re(Zyy)", "Im(Zyy)"]
_TITLE_R = ["App_RHO_xx", "App_RHO_xy", "App_RHO_yx", "App_RHO_yy", "App_PHI_xx", "App_PHI_xy", "App_PHI_yx",
            "App_PHI_yy"]


def es(v: float, w: int = 20, d: int = 5) -> str:
    """Fortran ``esw.d``."""
    s = f"{v:.{d}E}"
    mant, exp = s.split("E")
    e = int(exp)
    body = f"{mant}E{e:+03d}" if abs(e) < 100 else f"{mant}{e:+04d}"
    return body.rjust(w) if len(body) <= w else "*" * w


def fw(v: float, w: int = 20, d: int = 5) -> str:
    """Fortran ``fw.d``."""
    s = f"{v:.{d}f}"
    return s.rjust(w) if len(s) <= w else "*" * w


def solution_block(nf: int, E: np.ndarray, H: np.ndarray, Z: np.ndarray, rho: np.ndarray, phi: np.ndarray) -> str:
    """One frequency's block.  E, H: [npt, 2, 3] complex; Z: [npt, 4]; rho, phi:
    [npt, 4]."""
    out = [f" vector-fem solution: {nf:12d}", "".join(t.rjust(15) for t in _TITLE_E)]
    for ip in range(E.shape[0]):
        vals = []
        for p in range(2):
            for a in range(3):
                vals += [E[ip, p, a].real, E[ip, p, a].imag]
            for a in range(3):
                vals += [H[ip, p, a].real, H[ip, p, a].imag]
        out.append("".join(es(v) for v in vals))
    out.append("".join(t.rjust(15) for t in _TITLE_Z))
    for ip in range(Z.shape[0]):
        out.append("".join(es(v) for i in range(4) for v in (Z[ip, i].real, Z[ip, i].imag)))
    out.append("".join(t.rjust(15) for t in _TITLE_R))
    for ip in range(rho.shape[0]):
        out.append("".join(fw(v) for v in list(rho[ip]) + list(phi[ip])))
    return "\n".join(out) + "\n"


def _ld(*vals) -> str:
    """A list-directed record.  Its exact spacing is compiler-specific: integers in 12
    columns and reals with 17 significant digits in 25 columns (gfortran's widths for
    default integers and REAL(8)), after one leading blank."""
    parts = []
    for v in vals:
        if isinstance(v, (int, np.integer)):
            parts.append(f"{int(v):12d}")
        elif isinstance(v, str):
            parts.append(v)
        else:
            parts.append(f"{float(v):25.16E}")
    return " " + "".join(parts)


def receiver_block(nf: int, rx: np.ndarray, E, H, Z, rho, phi) -> str:
    """One frequency's RECEIVER.OUT block (after the coordinate header): rx [nrx, 2]
    (x, y); E, H [nrx, 2, 3] complex; Z [nrx, 4]; rho, phi [nrx, 4]."""
    out = [f"{nf:5d} " + "".join(t.rjust(15) for t in ["x", "y"] + _TITLE_E)]
    for i in range(rx.shape[0]):
        vals = [rx[i, 0], rx[i, 1]]
        for p in range(2):
            for a in range(3):
                vals += [E[i, p, a].real, E[i, p, a].imag]
            for a in range(3):
                vals += [H[i, p, a].real, H[i, p, a].imag]
        out.append("".join(es(v) for v in vals))
    out.append(f"{nf:5d} " + "".join(t.rjust(15) for t in ["x", "y"] + _TITLE_Z))
    for i in range(rx.shape[0]):
        out.append("".join(es(v) for v in [rx[i, 0], rx[i, 1]] + [w for k in range(4) for w in (Z[i, k].real,
                                                                                               Z[i, k].imag)]))
    out.append(f"{nf:5d} " + "".join(t.rjust(15) for t in ["x", "y"] + _TITLE_R))
    for i in range(rx.shape[0]):
        out.append("".join(fw(v) for v in [rx[i, 0], rx[i, 1]] + list(rho[i]) + list(phi[i])))
    return "\n".join(out) + "\n"


def write_receivers(path: str, rx: np.ndarray, rz: np.ndarray, E, H, Z, rho, phi) -> None:
    """RECEIVER.OUT for every frequency (leading axis of E, H, Z, rho, phi); rx [nrx, 2],
    rz [nrx] the receivers' heights."""
    nf = E.shape[0]
    with open(path, "w") as fh:
        fh.write(_ld("----------------rx coords-----------------------") + "\n")
        fh.write(_ld(rx.shape[0], 2, nf) + "\n")
        for i in range(rx.shape[0]):
            fh.write(_ld(rx[i, 0], rx[i, 1], rz[i]) + "\n")
        for f in range(nf):
            fh.write(receiver_block(f + 1, rx, E[f], H[f], Z[f], rho[f], phi[f]))


def write_solution(path: str, E, H, Z, rho, phi) -> None:
    """All frequencies (leading axis of every array) into one SOLUTION.OUT."""
    with open(path, "w") as fh:
        for f in range(E.shape[0]):
            fh.write(solution_block(f + 1, E[f], H[f], Z[f], rho[f], phi[f]))


def surface_nodes(m) -> np.ndarray:
    """Node ids of the inner-grid surface in sur_data's order (receiver_data.f90:135-168):
    j outer, i inner, over the nodes inside the extension cells, at the node layer
    below the top padding and air layers."""
    s = m.nord - 1
    i1, i2 = m.nextd * s, m.nnx - 1 - m.nextd * s
    j1, j2 = m.nextd * s, m.nny - 1 - m.nextd * s
    k = m.nnz - 1 - (m.nzl_top + m.nzl_air) * s
    return np.array([(i * m.nny + j) * m.nnz + k for j in range(j1, j2 + 1) for i in range(i1, i2 + 1)],
                    dtype=np.int64)


def write_surface(path: str, m, E, H, Z, rho, phi) -> None:
    """SURFACE.OUT (write_surface_data, receiver_data.f90:69-109) from the full-volume
    fields of :meth:`movfem_gb300.api.MTProblem.node_fields` (leading axis: frequency)."""
    ids = surface_nodes(m)
    s = m.nord - 1
    xs = np.asarray(m.xp)[m.nextd * s: m.nnx - m.nextd * s]
    ys = np.asarray(m.yp)[m.nextd * s: m.nny - m.nextd * s]
    nf = E.shape[0]
    with open(path, "w") as fh:
        fh.write(_ld("-----------------surface coords----------------") + "\n")
        fh.write(_ld(xs.size, ys.size, ids.size, 2, nf) + "\n")
        fh.write(_ld(*xs) + "\n")
        fh.write(_ld(*ys) + "\n")
        fh.write(_ld(*np.asarray(m.zp)[ids]) + "\n")
        for f in range(nf):
            out = [f"{f + 1:5d} " + "".join(t.rjust(15) for t in _TITLE_E)]
            for n in ids:
                vals = []
                for p in range(2):
                    for a in range(3):
                        vals += [E[f, n, p, a].real, E[f, n, p, a].imag]
                    for a in range(3):
                        vals += [H[f, n, p, a].real, H[f, n, p, a].imag]
                out.append("".join(es(v) for v in vals))
            out.append(f"{f + 1:5d} " + "".join(t.rjust(15) for t in _TITLE_Z))
            for n in ids:
                out.append("".join(es(v) for i in range(4) for v in (Z[f, n, i].real, Z[f, n, i].imag)))
            out.append(f"{f + 1:5d} " + "".join(t.rjust(15) for t in _TITLE_R))
            for n in ids:
                out.append("".join(fw(v) for v in list(rho[f, n]) + list(phi[f, n])))
            fh.write("\n".join(out) + "\n")
