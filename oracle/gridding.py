"""CPU restatement of the reference's gridding (``grid_3d``, geometry.f90:48-118) and of
the modified quadratic Shepard interpolation it calls (ACM TOMS algorithm 660, Renka
1988: ``QSHEP2`` / ``QS2VAL`` with ``STORE2``, ``GETNP2``, ``SETUP2``, ``GIVENS``,
``ROTATE``; the reference carries a Fortran 90 version in toms660.f90).

TEST INFRASTRUCTURE ONLY: the oracle the tests compare ``movfem_gb300``'s native
gridding (``mvf_grid_3d``) against.  Nothing in the product imports it.

The loops follow the Fortran statement by statement, 1-based (index 0 of every array is
unused), so that each node is written in the same order and the last write wins as it
does there.  Two things differ, neither changing a value:

* ``zblocks`` and ``gauss_grid`` refit both interfaces of a layer with QSHEP2 at every
  (x, y) cell (geometry.f90:459-460, 549-550).  QSHEP2 is a pure function of its
  inputs, so the fits are made once per (interface, nq, nw) here.
* the bottom layer of ``gauss_grid`` interpolates a zero surface (``zt1 = 0``,
  geometry.f90:536-542); that fit is a fit of zeros and evaluates to exactly 0.

Inputs that the reference turns into reads of unset memory raise ``GridError`` instead:
an interface with fewer than 20 points (QSHEP2 then returns ier = 1 before fitting,
toms660.f90:921-932) and any other nonzero ier.  In ``extension`` the ratio
``ddx/depth`` in [1.5, 2.5) matches none of the three branches and leaves ``nd`` unset
(geometry.f90:246-252); ``nd = 2`` is used there, the value of the middle branch.

Parity is unpinned: the reference needs a Fortran compiler, which neither machine has.
The restatement is checked by properties (QS2VAL interpolates the data, reproduces
quadratics, the grid's layering sums up) and against ``mvf_grid_3d``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

PI = 3.1415926535897932384626433
MU_0 = 4.0 * PI * 1.0e-7


class GridError(ValueError):
    pass


# ---------------------------------------------------------------- TOMS 660 (QSHEP2D)

@dataclass
class Shepard:
    """A QSHEP2 fit: nodes (1-based), the cell grid of STORE2, radii and coefficients."""
    n: int
    x: list
    y: list
    f: list
    nr: int
    lcell: list
    lnext: list
    xmin: float
    ymin: float
    dx: float
    dy: float
    rmax: float
    rsq: list
    a: list  # a[k] = [_, a1..a5]


def store2(x, y, n, nr):
    """Cell grid of the nodes (toms660.f90:1579-1745, STORE2): nr x nr cells over the bounding box,
    lcell[i][j] = first node of the cell, lnext[k] = next node (k itself at the end);
    nodes are entered from n down to 1."""
    if n < 2 or nr < 1:
        raise GridError("STORE2: ier = 1")
    xmin = min(x[1:n + 1])
    xmax = max(x[1:n + 1])
    ymin = min(y[1:n + 1])
    ymax = max(y[1:n + 1])
    dx = (xmax - xmin) / float(nr)
    dy = (ymax - ymin) / float(nr)
    if dx == 0.0 or dy == 0.0:
        raise GridError("STORE2: ier = 2 (nodes on a line)")
    lcell = [[0] * (nr + 1) for _ in range(nr + 1)]
    lnext = [0] * (n + 1)
    for k in range(n, 0, -1):
        i = min(int((x[k] - xmin) / dx) + 1, nr)
        j = min(int((y[k] - ymin) / dy) + 1, nr)
        l = lcell[i][j]
        lnext[k] = l if l != 0 else k
        lcell[i][j] = k
    return lcell, lnext, xmin, ymin, dx, dy


def getnp2(px, py, x, y, nr, lcell, lnext, xmin, ymin, dx, dy):
    """Nearest unmarked node to (px, py) by rings of cells (toms660.f90:4-288, GETNP2); marks it
    (lnext negated).  The ring search stops once the ring covers [imin, imax] on the
    right and [jmin, jmax]: the left test of this version compares i1 with itself
    (toms660.f90:267) and is always true.  Ties keep the node met first."""
    first = True
    imin, imax, jmin, jmax = 1, nr, 1, nr
    delx = px - xmin
    dely = py - ymin
    i0 = min(max(int(delx / dx) + 1, 1), nr)
    j0 = min(max(int(dely / dy) + 1, 1), nr)
    i1 = i2 = i0
    j1 = j2 = j0
    lmin, rsmin = 0, 0.0
    while True:
        for j in range(j1, j2 + 1):
            if jmax < j:
                break
            if j < jmin:
                continue
            for i in range(i1, i2 + 1):
                if imax < i:
                    break
                if i < imin:
                    continue
                if j != j1 and j != j2 and i != i1 and i != i2:
                    continue
                l = lcell[i][j]
                if l > 0:
                    while True:
                        ln = lnext[l]
                        if ln >= 0:
                            ddx = x[l] - px
                            ddy = y[l] - py
                            rsq = ddx * ddx + ddy * ddy
                            if first:
                                lmin, rsmin = l, rsq
                                r = math.sqrt(rsmin)
                                imin = max(int((delx - r) / dx) + 1, 1)
                                imax = min(int((delx + r) / dx) + 1, nr)
                                jmin = max(int((dely - r) / dy) + 1, 1)
                                jmax = min(int((dely + r) / dy) + 1, nr)
                                first = False
                            elif rsq < rsmin:
                                lmin, rsmin = l, rsq
                        if abs(ln) != l:
                            l = abs(ln)
                        else:
                            break
        if imax <= i2 and j1 <= jmin and jmax <= j2:
            break
        i1 -= 1
        i2 += 1
        j1 -= 1
        j2 += 1
    if first:
        return 0, 0.0
    lnext[lmin] = -lnext[lmin]
    return lmin, rsmin


def givens(a, b):
    """Givens rotation zeroing b against a (toms660.f90:289-395, GIVENS): returns the new a (r),
    the new b (the reconstruction code), c and s."""
    if abs(b) < abs(a):
        u = 2.0 * a
        v = b / u
        r = math.sqrt(0.25 + v * v) * u
        c = a / r
        s = 2.0 * v * c
        return r, s, c, s
    if b != 0.0:
        u = 2.0 * b
        v = a / u
        a = math.sqrt(0.25 + v * v) * u
        s = b / a
        c = 2.0 * v * s
        return a, (1.0 / c if c != 0.0 else 1.0), c, s
    return a, b, 1.0, 0.0


def rotate(n, c, s, B, col_x, col_y, r0):
    """Apply the rotation to entries r0 .. r0+n-1 of columns col_x, col_y of B
    (toms660.f90:1426-1483, ROTATE)."""
    if n <= 0 or (c == 1.0 and s == 0.0):
        return
    for r in range(r0, r0 + n):
        xi = B[r][col_x]
        yi = B[r][col_y]
        B[r][col_x] = c * xi + s * yi
        B[r][col_y] = -(s * xi) + c * yi


def setup2(xk, yk, fk, xi, yi, fi, s1, s2, r, B, col):
    """One weighted least-squares row of node k's quadratic (toms660.f90:1484-1578, SETUP2)."""
    dx = xi - xk
    dy = yi - yk
    d = math.sqrt(dx * dx + dy * dy)
    if d <= 0.0 or r <= d:
        for q in range(1, 7):
            B[q][col] = 0.0
        return
    w = (r - d) / r / d
    B[1][col] = dx * dx * w / s2
    B[2][col] = dx * dy * w / s2
    B[3][col] = dy * dy * w / s2
    B[4][col] = dx * w / s1
    B[5][col] = dy * w / s1
    B[6][col] = (fi - fk) * w


def qshep2(xs, ys, fs, nq, nw, nr) -> Shepard:
    """Fit of the nodal quadratics and radii (toms660.f90:679-1208, QSHEP2): xs, ys, fs 0-based."""
    DTOL, RTOL, SF = 0.01, 1.0e-05, 1.0
    n = len(xs)
    x = [0.0] + [float(v) for v in xs]
    y = [0.0] + [float(v) for v in ys]
    f = [0.0] + [float(v) for v in fs]
    nqwmax = max(nq, nw)
    lmax = min(40, n - 1)
    if nq < 5 or nw < 1 or lmax < nqwmax or nr < 1:
        raise GridError(f"QSHEP2: ier = 1 (n = {n}, nq = {nq}, nw = {nw}, nr = {nr})")
    lcell, lnext, xmn, ymn, ddx, ddy = store2(x, y, n, nr)
    rsq = [0.0] * (n + 1)
    a = [[0.0] * 6 for _ in range(n + 1)]
    B = [[0.0] * 7 for _ in range(7)]
    rsmx = 0.0
    for k in range(1, n + 1):
        xk, yk, fk = x[k], y[k], f[k]
        lnext[k] = -lnext[k]
        rs = sum2 = rws = rq = 0.0
        lnp = 0
        npts = [0] * 41
        neq, avsq = 0, 0.0
        # nearest nodes until both nq and nw are exceeded (labels 1, 3, 4)
        while True:
            sum2 += rs
            if lnp == lmax:
                if rws == 0.0:
                    rws = 1.1 * rs
                if rq == 0.0:
                    neq = lmax
                    rq = math.sqrt(1.1 * rs)
                    avsq = sum2 / float(neq)
                break
            lnp += 1
            rsold = rs
            np_, rs = getnp2(xk, yk, x, y, nr, lcell, lnext, xmn, ymn, ddx, ddy)
            if rs == 0.0:
                raise GridError("QSHEP2: ier = 2 (duplicate nodes)")
            npts[lnp] = np_
            if (rs - rsold) / rs < RTOL:
                continue
            if rws == 0.0 and nw < lnp:
                rws = rs
            if rq == 0.0 and nq < lnp:
                neq = lnp - 1
                rq = math.sqrt(rs)
                avsq = sum2 / float(neq)
            if nqwmax < lnp:
                break
        rsq[k] = rws
        rsmx = max(rsmx, rws)
        av = math.sqrt(avsq)
        i = 0
        # rows of the least-squares system by Givens rotations (labels 5, 7, 9, 10)
        while True:
            i += 1
            np_ = npts[i]
            irow = min(i, 6)
            setup2(xk, yk, fk, x[np_], y[np_], f[np_], av, avsq, rq, B, irow)
            if i == 1:
                continue
            for j in range(1, irow):
                B[j][j], B[j][irow], c, s = givens(B[j][j], B[j][irow])
                rotate(6 - j, c, s, B, j, irow, j + 1)
            if i < neq:
                continue
            dmin = min(abs(B[1][1]), abs(B[2][2]), abs(B[3][3]), abs(B[4][4]), abs(B[5][5]))
            if DTOL <= dmin * rq:
                break
            if neq == lmax:
                # regularise toward a linear fit (label 10)
                for ii in range(1, 4):
                    B[ii][6] = SF
                    for q in range(ii + 1, 7):
                        B[q][6] = 0.0
                    for j in range(ii, 6):
                        B[j][j], B[j][6], c, s = givens(B[j][j], B[j][6])
                        rotate(6 - j, c, s, B, j, 6, j + 1)
                dmin = min(abs(B[1][1]), abs(B[2][2]), abs(B[3][3]), abs(B[4][4]), abs(B[5][5]))
                if dmin * rq < DTOL:
                    raise GridError("QSHEP2: ier = 3 (ill-conditioned fit)")
                break
            # one more equation (label 7)
            while True:
                rsold = rs
                neq += 1
                if neq == lmax:
                    rq = math.sqrt(1.1 * rs)
                    break
                if neq != lnp:
                    np_ = npts[neq + 1]
                    ex = x[np_] - xk
                    ey = y[np_] - yk
                    rs = ex * ex + ey * ey
                    if (rs - rsold) / rs < RTOL:
                        continue
                    rq = math.sqrt(rs)
                    break
                lnp += 1
                np_, rs = getnp2(xk, yk, x, y, nr, lcell, lnext, xmn, ymn, ddx, ddy)
                if np_ == 0:
                    raise GridError("QSHEP2: ier = 2")
                npts[lnp] = np_
                if (rs - rsold) / rs < RTOL:
                    continue
                rq = math.sqrt(rs)
                break
        # back substitution (label 13)
        for ii in range(5, 0, -1):
            t = 0.0
            for j in range(ii + 1, 6):
                t = t + B[j][ii] * a[k][j]
            a[k][ii] = (B[6][ii] - t) / B[ii][ii]
        for q in range(1, 4):
            a[k][q] = a[k][q] / avsq
        a[k][4] = a[k][4] / av
        a[k][5] = a[k][5] / av
        lnext[k] = -lnext[k]
        for q in range(1, lnp + 1):
            lnext[npts[q]] = -lnext[npts[q]]
    return Shepard(n, x, y, f, nr, lcell, lnext, xmn, ymn, ddx, ddy, math.sqrt(rsmx), rsq, a)


def qs2val(px, py, s: Shepard) -> float:
    """Value of the interpolant at (px, py) (toms660.f90:1209-1425, QS2VAL)."""
    if s.n < 6 or s.nr < 1 or s.dx <= 0.0 or s.dy <= 0.0 or s.rmax < 0.0:
        return 0.0
    imin = max(int((px - s.xmin - s.rmax) / s.dx) + 1, 1)
    imax = min(int((px - s.xmin + s.rmax) / s.dx) + 1, s.nr)
    jmin = max(int((py - s.ymin - s.rmax) / s.dy) + 1, 1)
    jmax = min(int((py - s.ymin + s.rmax) / s.dy) + 1, s.nr)
    if imax < imin or jmax < jmin:
        return 0.0
    sw = swq = 0.0
    for j in range(jmin, jmax + 1):
        for i in range(imin, imax + 1):
            k = s.lcell[i][j]
            if k == 0:
                continue
            while True:
                delx = px - s.x[k]
                dely = py - s.y[k]
                ds = delx * delx + dely * dely
                rs = s.rsq[k]
                if ds < rs:
                    if ds == 0.0:
                        return s.f[k]
                    rds = rs * ds
                    rd = math.sqrt(rds)
                    w = (rs + ds - rd - rd) / rds
                    sw = sw + w
                    ak = s.a[k]
                    swq = swq + w * (s.f[k] + ak[1] * delx * delx + ak[2] * delx * dely + ak[3] * dely * dely
                                     + ak[4] * delx + ak[5] * dely)
                kp = k
                k = s.lnext[kp]
                if k == kp:
                    break
    return 0.0 if sw == 0.0 else swq / sw


def cells_per_side(n: int) -> int:
    """nr = int(sqrt(float(n)/3.)) in single precision (geometry.f90:447-448)."""
    return int(np.sqrt(np.float32(n) / np.float32(3.0)))


# ---------------------------------------------------------------- grid_3d

@dataclass
class GridInput:
    """The arguments of grid_3d as read_input leaves them (read_input.f90:47-162):
    spacings, air height and depth below the interfaces, nodes per element, background
    conductivity, receivers, the input interfaces (nsf0 of them, each a list of points)
    and the inner model coordinates, all in the input's coordinates."""
    dx: float
    dy: float
    dz: float
    high: float
    depth: float
    nodes_per_elem: int
    sigma_bg: float
    rx: np.ndarray                      # [nsr, 3]
    interfaces: list                    # nsf0 arrays [n_l, 3]
    xm: np.ndarray                      # [mx]
    ym: np.ndarray                      # [my]
    zm: np.ndarray                      # [mx, my, mz]
    freqs: np.ndarray


@dataclass
class Grid:
    nord: int
    nextd: int
    nx: int            # g_nx (x grid lines)
    ny: int
    nz: int
    nzl: np.ndarray    # [nsf] layers per interface interval (g_nzl)
    x0: float
    y0: float
    z0: float
    ztop: float        # g_ztop
    xp: np.ndarray     # [nnx]
    yp: np.ndarray     # [nny]
    zp: np.ndarray     # [nnx * nny * nnz]
    rx: np.ndarray     # receivers after coord_transform
    xm: np.ndarray
    ym: np.ndarray
    zm: np.ndarray
    info: dict = field(default_factory=dict)


def grid_3d(g: GridInput) -> Grid:
    nord = 2 if g.nodes_per_elem == 8 else 3
    nsf0 = len(g.interfaces)
    nsf = nsf0 + 3
    for l, p in enumerate(g.interfaces):
        if len(p) < 20:
            raise GridError(f"interface {l + 1} has {len(p)} points; QSHEP2 needs at least 20")
    # interfaces 1..nsf (1-based, point lists 1-based too); 2..nsf0+1 are the input ones
    nsp = [0] * (nsf + 1)
    xto = [[0.0] for _ in range(nsf + 1)]
    yto = [[0.0] for _ in range(nsf + 1)]
    zto = [[0.0] for _ in range(nsf + 1)]
    for l, p in enumerate(g.interfaces):
        nsp[l + 2] = len(p)
        xto[l + 2] = [0.0] + [float(v) for v in p[:, 0]]
        yto[l + 2] = [0.0] + [float(v) for v in p[:, 1]]
        zto[l + 2] = [0.0] + [float(v) for v in p[:, 2]]
    xsr = [float(v) for v in g.rx[:, 0]]
    ysr = [float(v) for v in g.rx[:, 1]]
    zsr = [float(v) for v in g.rx[:, 2]]
    xm = np.array(g.xm, dtype=np.float64)
    ym = np.array(g.ym, dtype=np.float64)
    zm = np.array(g.zm, dtype=np.float64)

    # min_max_input (geometry.f90:157-220), ymin/ymax from xsr as there (Q14)
    xmin = ymin = zmin = 1.0e20
    xmax = ymax = zmax = -1.0e20
    x1 = y1 = zl = 1.0e20
    x2 = y2 = zu = -1.0e20
    for i in range(len(xsr)):
        if xsr[i] < xmin:
            xmin = xsr[i]
        if xsr[i] > xmax:
            xmax = xsr[i]
        if ysr[i] < ymin:
            ymin = xsr[i]
        if ysr[i] > ymax:
            ymax = xsr[i]
        if zsr[i] < zmin:
            zmin = zsr[i]
        if zsr[i] > zmax:
            zmax = zsr[i]
    for i in range(1, nsf - 2):
        for j in range(1, nsp[i + 1] + 1):
            x1 = xto[i + 1][j] if xto[i + 1][j] < x1 else x1
            x2 = xto[i + 1][j] if xto[i + 1][j] > x2 else x2
            y1 = yto[i + 1][j] if yto[i + 1][j] < y1 else y1
            y2 = yto[i + 1][j] if yto[i + 1][j] > y2 else y2
            zl = zto[i + 1][j] if zto[i + 1][j] < zl else zl
            zu = zto[i + 1][j] if zto[i + 1][j] > zu else zu
    xmin = min(xmin, x1)
    xmax = max(xmax, x2)
    ymin = min(ymin, y1)
    ymax = max(ymax, y2)
    zu = zu + g.high
    zl = zl - g.depth
    zmin = min(zmin, zl)
    zmax = max(zmax, zu)
    for v in xm:
        xmin = v if v < xmin else xmin
        xmax = v if v > xmax else xmax
    for v in ym:
        ymin = v if v < ymin else ymin
        ymax = v if v > ymax else ymax
    for v in zm.reshape(-1):
        zmin = v if v < zmin else zmin
        zmax = v if v > zmax else zmax

    # extension (geometry.f90:224-344)
    fact = 1.3
    nextd = 2
    ddx = min(xmax - xmin, ymax - ymin, zmax - zmin)
    minf = 1.0e20
    for fr in g.freqs:
        if fr < minf:
            minf = float(fr)
    depth = math.sqrt(2.0 / (MU_0 * g.sigma_bg * 2.0 * PI * minf))
    if ddx / depth >= 2.5:
        nd = 1.5
    elif ddx / depth < 2.5 and depth / ddx >= 1.5:
        nd = 2.0
    elif ddx / depth < 1.5:
        nd = 3.0
    else:
        nd = 2.0   # unset in the reference
    dmin_ = min(g.dx, g.dy, g.dz)
    while True:
        sum_ex = 0.0
        for i in range(1, nextd + 1):
            sum_ex = sum_ex + fact * dmin_ * float(i)
        if sum_ex > nd * depth:
            break
        nextd += 1
    dmx = [0.0] * (nextd + 1)
    dmy = [0.0] * (nextd + 1)
    x1, x2, y1, y2 = xmin, xmax, ymin, ymax
    for i in range(1, nextd + 1):
        dmx[i] = fact * float(i) * g.dx
        x1 = x1 - dmx[i]
        x2 = x2 + dmx[i]
    for i in range(1, nextd + 1):
        dmy[i] = fact * float(i) * g.dy
        y1 = y1 - dmy[i]
        y2 = y2 + dmy[i]
    x0 = 0.5 * (x1 + x2)
    y0 = 0.5 * (y1 + y2)
    x1, x2 = x1 - x0, x2 - x0
    y1, y2 = y1 - y0, y2 - y0
    xmin, xmax = xmin - x0, xmax - x0
    ymin, ymax = ymin - y0, ymax - y0
    nx0 = int((xmax - xmin) / g.dx) + 1
    ny0 = int((ymax - ymin) / g.dy) + 1
    g_nx = nx0 + 2 * nextd
    g_ny = ny0 + 2 * nextd
    x = [0.0] * (g_nx + 1)
    y = [0.0] * (g_ny + 1)
    x[1], y[1] = x1, y1
    for i in range(1, nextd + 1):
        x[i + 1] = x[i] + dmx[nextd + 1 - i]
    for i in range(1, nextd + 1):
        y[i + 1] = y[i] + dmy[nextd + 1 - i]
    for i in range(1, nx0 + 1):
        x[i + nextd] = x[nextd + 1] + float(i - 1) * g.dx
    for i in range(1, ny0 + 1):
        y[i + nextd] = y[nextd + 1] + float(i - 1) * g.dy
    i0 = nextd + nx0
    for i in range(1, nextd + 1):
        x[i0 + i] = x[i0 + i - 1] + dmx[i]
    i0 = nextd + ny0
    for i in range(1, nextd + 1):
        y[i0 + i] = y[i0 + i - 1] + dmy[i]
    dmz = [0.0] * (nextd + 1)
    zbot, ztop = zmin, zmax
    for i in range(1, nextd + 1):
        dmz[i] = fact * float(i) * g.dz
        zbot = zbot - dmz[i]
        ztop = ztop + dmz[i]
    nsp[1] = nsp[2]
    xto[1], yto[1] = list(xto[2]), list(yto[2])
    zto[1] = [0.0] + [zmin] * nsp[1]
    nsp[nsf - 1] = nsp[nsf - 2]
    xto[nsf - 1], yto[nsf - 1] = list(xto[nsf - 2]), list(yto[nsf - 2])
    zto[nsf - 1] = [0.0] + [zmax] * nsp[nsf - 1]
    nsp[nsf] = nsp[nsf - 1]
    xto[nsf], yto[nsf] = list(xto[nsf - 1]), list(yto[nsf - 1])
    zto[nsf] = [0.0] + [ztop] * nsp[nsf]
    z0 = zbot
    zmin, zmax = zmin - z0, zmax - z0

    # coord_transform (geometry.f90:367-411)
    xsr = [v - x0 for v in xsr]
    ysr = [v - y0 for v in ysr]
    zsr = [v - z0 for v in zsr]
    for l in range(1, nsf + 1):
        for j in range(1, nsp[l] + 1):
            xto[l][j] = xto[l][j] - x0
            yto[l][j] = yto[l][j] - y0
            zto[l][j] = zto[l][j] - z0
    g_ztop = 1.0e20
    for j in range(1, nsp[nsf - 2] + 1):
        if zto[nsf - 2][j] < g_ztop:
            g_ztop = zto[nsf - 2][j]
    xm = xm - x0
    ym = ym - y0
    zm = zm - z0

    # one QSHEP2 fit per (interface, nq, nw); nr from the interface's own count
    fits = {}

    def fit(l, nq, nw):
        key = (l, nq, nw)
        if key not in fits:
            n = nsp[l]
            fits[key] = qshep2(xto[l][1:n + 1], yto[l][1:n + 1], zto[l][1:n + 1], nq, nw, cells_per_side(n))
        return fits[key]

    # zblocks (geometry.f90:415-483)
    nzl = [0] * (nsf + 1)
    nzl[1] = nextd
    nzl[nsf] = nextd
    for l in range(2, nsf):
        np2, np1 = nsp[l], nsp[l - 1]
        nq = min(13, np1, np2)
        nw = min(19, np1, np2)
        s1, s2 = fit(l - 1, nq, nw), fit(l, nq, nw)
        h = 0.0
        for i in range(nextd + 1, g_nx - nextd):
            for j in range(nextd + 1, g_ny - nextd):
                dh = qs2val(x[i], y[j], s2) - qs2val(x[i], y[j], s1)
                if dh > h:
                    h = dh
        nzl[l] = max(int(h / g.dz), 1)
    g_nz = 1 + sum(nzl[1:])

    # gauss_grid (geometry.f90:487-586) and local_gqg (geometry.f90:744-768)
    nnx = (g_nx - 1) * (nord - 1) + 1
    nny = (g_ny - 1) * (nord - 1) + 1
    nnz = (g_nz - 1) * (nord - 1) + 1
    nyz = nny * nnz
    xp = np.zeros(nnx + 1)
    yp = np.zeros(nny + 1)
    zp = np.zeros(nnx * nny * nnz + 1)
    fn = 2.0 / float(nord - 1)
    asx = [0.0] + [-1.0 + float(j - 1) * fn for j in range(1, nord + 1)]
    for i in range(nextd + 1, g_nx - nextd):
        xa, xb = x[i], x[i + 1]
        for j in range(nextd + 1, g_ny - nextd + 2):
            ya, yb = y[j], y[j + 1]
            z2 = [[0.0] * (nord + 1) for _ in range(nord + 1)]
            z1 = [[0.0] * (nord + 1) for _ in range(nord + 1)]
            k = 0
            for l in range(1, nsf + 1):
                np2 = nsp[l]
                np1 = nsp[l] if l == 1 else nsp[l - 1]
                nq = min(13, np1, np2)
                nw = min(19, np1, np2)
                s2 = fit(l, nq, nw)
                s1 = None if l == 1 else fit(l - 1, nq, nw)
                for _l1 in range(1, nzl[l] + 1):
                    k += 1
                    no = (i - 1) * (nord - 1) * nyz + (j - 1) * (nord - 1) * nnz + (k - 1) * (nord - 1) + 1
                    for i1 in range(1, nord + 1):
                        xi = 0.5 * (xb - xa) * asx[i1] + 0.5 * (xa + xb)
                        for j1 in range(1, nord + 1):
                            yj = 0.5 * (yb - ya) * asx[j1] + 0.5 * (ya + yb)
                            z1[i1][j1] = z2[i1][j1]
                            h2 = qs2val(xi, yj, s2)
                            h1 = 0.0 if s1 is None else qs2val(xi, yj, s1)
                            dm = (h2 - h1) / float(nzl[l])
                            z2[i1][j1] = z1[i1][j1] + dm
                    for i1 in range(1, nord + 1):
                        xi = 0.5 * (xb - xa) * asx[i1] + 0.5 * (xa + xb)
                        xp[(i - 1) * (nord - 1) + i1] = xi
                        for j1 in range(1, nord + 1):
                            yj = 0.5 * (yb - ya) * asx[j1] + 0.5 * (ya + yb)
                            yp[(j - 1) * (nord - 1) + j1] = yj
                            for k1 in range(1, nord + 1):
                                zk = 0.5 * (z2[i1][j1] - z1[i1][j1]) * asx[k1] + 0.5 * (z1[i1][j1] + z2[i1][j1])
                                zp[no + (i1 - 1) * nyz + (j1 - 1) * nnz + (k1 - 1)] = zk

    # complete_grid (geometry.f90:588-711)
    def copy_block(i, j, i1, j1, l_of, m_of, xs=None, ys=None):
        for k in range(1, g_nz):
            no = (i - 1) * (nord - 1) * nyz + (j - 1) * (nord - 1) * nnz + (k - 1) * (nord - 1) + 1
            no1 = (i1 - 1) * (nord - 1) * nyz + (j1 - 1) * (nord - 1) * nnz + (k - 1) * (nord - 1) + 1
            for l in range(1, nord + 1):
                ll = l_of(l)
                ii = (i - 1) * (nord - 1) + l
                if xs is not None:
                    xp[ii] = 0.5 * (xs[1] - xs[0]) * asx[l] + 0.5 * (xs[0] + xs[1])
                else:
                    xp[ii] = xp[(i1 - 1) * (nord - 1) + ll]
                for m in range(1, nord + 1):
                    mm = m_of(m)
                    jj = (j - 1) * (nord - 1) + m
                    if ys is not None:
                        yp[jj] = 0.5 * (ys[1] - ys[0]) * asx[m] + 0.5 * (ys[0] + ys[1])
                    else:
                        yp[jj] = yp[(j1 - 1) * (nord - 1) + mm]
                    for n in range(1, nord + 1):
                        zp[no + (l - 1) * nyz + (m - 1) * nnz + (n - 1)] = \
                            zp[no1 + (ll - 1) * nyz + (mm - 1) * nnz + (n - 1)]

    ident = lambda v: v
    for i in range(1, nextd + 1):
        for j in range(nextd + 1, g_ny - nextd):
            copy_block(i, j, nextd + 1, j, lambda l: 1, ident, xs=(x[i], x[i + 1]))
    for i in range(g_nx - nextd, g_nx):
        for j in range(nextd + 1, g_ny - nextd):
            copy_block(i, j, g_nx - nextd - 1, j, lambda l: nord, ident, xs=(x[i], x[i + 1]))
    for i in range(1, g_nx):
        for j in range(1, nextd + 1):
            copy_block(i, j, i, nextd + 1, ident, lambda m: 1, ys=(y[j], y[j + 1]))
    for i in range(1, g_nx):
        for j in range(g_ny - nextd, g_ny):
            copy_block(i, j, i, g_ny - nextd - 1, ident, lambda m: nord, ys=(y[j], y[j + 1]))

    return Grid(nord=nord, nextd=nextd, nx=g_nx, ny=g_ny, nz=g_nz, nzl=np.array(nzl[1:], dtype=np.int32),
                x0=x0, y0=y0, z0=z0, ztop=g_ztop, xp=xp[1:].copy(), yp=yp[1:].copy(), zp=zp[1:].copy(),
                rx=np.stack([xsr, ysr, zsr], axis=1), xm=xm, ym=ym, zm=zm,
                info={"nd": nd, "skin_depth": depth, "x": np.array(x[1:]), "y": np.array(y[1:])})
