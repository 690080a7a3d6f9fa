"""SOLUTION.OUT writer: the layout of the reference's ``write_solution``
(solution.f90:71-205) for the whole-volume case (``inner == 0``), fed by
:meth:`movfem_gb300.api.MTProblem.node_fields`.

Per frequency block:
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


def write_solution(path: str, E, H, Z, rho, phi) -> None:
    """All frequencies (leading axis of every array) into one SOLUTION.OUT."""
    with open(path, "w") as fh:
        for f in range(E.shape[0]):
            fh.write(solution_block(f + 1, E[f], H[f], Z[f], rho[f], phi[f]))
