// Gridding of the model domain: the node coordinates that grid_3d (geometry.f90:48-118)
// leaves in the geometry module, built on the host in one pass.
//
// Steps, each with the reference routine whose arithmetic it keeps operation for
// operation (so that every coordinate comes out with the same bits):
//   bounds      min_max_input  geometry.f90:157-220 (ymin/ymax from the receivers' x)
//   padding     extension      geometry.f90:224-344 (skin-depth driven nextd, 1.3 i d)
//   shift       coord_transform geometry.f90:367-411
//   layering    zblocks        geometry.f90:415-483
//   nodes       gauss_grid + local_gqg  geometry.f90:487-586, 744-768
//   padding     complete_grid  geometry.f90:588-711
// The interfaces are interpolated with the modified quadratic Shepard method of ACM
// TOMS algorithm 660 (Renka 1988, QSHEP2/QS2VAL; the reference ships a Fortran 90
// version, toms660.f90).
//
// What is organised differently from the reference:
//   * each interface is fitted once.  zblocks and gauss_grid refit both interfaces of a
//     layer at every (x, y) cell (geometry.f90:459-460, 549-550); a fit depends on its
//     inputs only, so one fit per interface gives the same coefficients.
//   * node columns are independent and computed in parallel.  Where neighbouring cells
//     share a column, or neighbouring sub-layers a node, gauss_grid's last write wins;
//     here the writer is chosen up front: the cell of largest index in loop order
//     (x outer, y inner, the y loop running two cells into the padding as
//     geometry.f90:528 does) and, along z, the upper sub-layer.
//   * an interface with fewer than 20 points, or a fit QSHEP2 rejects (ier != 0), is an
//     error (MVF_E_ARG).  The reference ignores ier and then reads unset arrays.
//   * extension leaves nd unset for ddx/depth in [1.5, 2.5) (geometry.f90:246-252);
//     nd = 2 there, the middle branch's value.
// Compiled without floating-point contraction (-ffp-contract=off), so that x86 and Arm
// hosts give the same bits as the reference's unfused double arithmetic.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/movfem_gpu.h"

namespace mvf {
void set_host_error(const char *msg);
}

namespace {

constexpr double kPi = 3.1415926535897932384626433;
constexpr double kMu0 = 4.0 * kPi * 1.0e-7;

struct GridFail {
    std::string msg;
};

// ------------------------------------------------------------------ Shepard surface
// One interface z = f(x, y) fitted by QSHEP2: nodes, STORE2's nr x nr cell lists, the
// radius of influence rsq[k] and the five coefficients of node k's quadratic.
class Surface {
public:
    Surface(const double *x, const double *y, const double *f, int n, int nq, int nw);
    double value(double px, double py) const;  // QS2VAL

private:
    int n_, nr_;
    std::vector<double> x_, y_, f_;     // 1-based
    std::vector<int> cell_, next_;      // cell_[(j-1)*nr + (i-1)] first node; next_ chain, 1-based
    double xmin_, ymin_, dx_, dy_, rmax_;
    std::vector<double> rsq_;           // 1-based
    std::vector<double> a_;             // [n+1][5]

    int &cell(int i, int j) { return cell_[(size_t)(j - 1) * nr_ + (i - 1)]; }
    int cell(int i, int j) const { return cell_[(size_t)(j - 1) * nr_ + (i - 1)]; }
    int nearest(double px, double py, double *dsq);  // GETNP2, marks the node
};

// Givens rotation (GIVENS): a <- r, b <- reconstruction code; returns c, s.
void givens(double &a, double &b, double &c, double &s) {
    if (std::fabs(b) < std::fabs(a)) {
        const double u = 2.0 * a, v = b / u;
        const double r = std::sqrt(0.25 + v * v) * u;
        c = a / r;
        s = 2.0 * v * c;
        b = s;
        a = r;
    } else if (b != 0.0) {
        const double u = 2.0 * b, v = a / u;
        a = std::sqrt(0.25 + v * v) * u;
        s = b / a;
        c = 2.0 * v * s;
        b = c != 0.0 ? 1.0 / c : 1.0;
    } else {
        c = 1.0;
        s = 0.0;
    }
}

// The 6x6 work array of QSHEP2, column-major like the Fortran b(6,6): column `col`
// holds one equation (five coefficients and the right-hand side).
struct Tri {
    double b[6][6];  // b[col][row], 0-based
    double &at(int row, int col) { return b[col - 1][row - 1]; }
    // ROTATE on rows r0.. of columns cx, cy (1-based)
    void rot(int cnt, double c, double s, int r0, int cx, int cy) {
        if (cnt <= 0 || (c == 1.0 && s == 0.0)) return;
        for (int r = r0; r < r0 + cnt; ++r) {
            const double xi = at(r, cx), yi = at(r, cy);
            at(r, cx) = c * xi + s * yi;
            at(r, cy) = -(s * xi) + c * yi;
        }
    }
    // SETUP2: the weighted equation of node (xi, yi, fi) for node k
    void equation(int col, double xk, double yk, double fk, double xi, double yi, double fi, double s1, double s2,
                  double r) {
        const double dx = xi - xk, dy = yi - yk;
        const double d = std::sqrt(dx * dx + dy * dy);
        if (d <= 0.0 || r <= d) {
            for (int q = 1; q <= 6; ++q) at(q, col) = 0.0;
            return;
        }
        const double w = (r - d) / r / d;
        at(1, col) = dx * dx * w / s2;
        at(2, col) = dx * dy * w / s2;
        at(3, col) = dy * dy * w / s2;
        at(4, col) = dx * w / s1;
        at(5, col) = dy * w / s1;
        at(6, col) = (fi - fk) * w;
    }
    double dmin() {
        return std::min({std::fabs(at(1, 1)), std::fabs(at(2, 2)), std::fabs(at(3, 3)), std::fabs(at(4, 4)),
                         std::fabs(at(5, 5))});
    }
};

int Surface::nearest(double px, double py, double *dsq) {
    bool first = true;
    int imin = 1, imax = nr_, jmin = 1, jmax = nr_;
    const double delx = px - xmin_, dely = py - ymin_;
    const int i0 = std::min(std::max((int)(delx / dx_) + 1, 1), nr_);
    const int j0 = std::min(std::max((int)(dely / dy_) + 1, 1), nr_);
    int i1 = i0, i2 = i0, j1 = j0, j2 = j0, lmin = 0;
    double rsmin = 0.0;
    for (;;) {
        for (int j = j1; j <= j2; ++j) {
            if (jmax < j) break;
            if (j < jmin) continue;
            for (int i = i1; i <= i2; ++i) {
                if (imax < i) break;
                if (i < imin) continue;
                if (j != j1 && j != j2 && i != i1 && i != i2) continue;  // ring cells only
                int l = cell(i, j);
                if (l <= 0) continue;
                for (;;) {
                    const int ln = next_[l];
                    if (ln >= 0) {
                        const double ex = x_[l] - px, ey = y_[l] - py;
                        const double rsq = ex * ex + ey * ey;
                        if (first) {
                            lmin = l;
                            rsmin = rsq;
                            const double r = std::sqrt(rsmin);
                            imin = std::max((int)((delx - r) / dx_) + 1, 1);
                            imax = std::min((int)((delx + r) / dx_) + 1, nr_);
                            jmin = std::max((int)((dely - r) / dy_) + 1, 1);
                            jmax = std::min((int)((dely + r) / dy_) + 1, nr_);
                            first = false;
                        } else if (rsq < rsmin) {
                            lmin = l;
                            rsmin = rsq;
                        }
                    }
                    if (std::abs(ln) == l) break;
                    l = std::abs(ln);
                }
            }
        }
        // the reference's stop test (toms660.f90:267) has no condition on the left edge
        if (imax <= i2 && j1 <= jmin && jmax <= j2) break;
        --i1;
        ++i2;
        --j1;
        ++j2;
    }
    if (first) {
        *dsq = 0.0;
        return 0;
    }
    next_[lmin] = -next_[lmin];
    *dsq = rsmin;
    return lmin;
}

Surface::Surface(const double *x, const double *y, const double *f, int n, int nq, int nw)
    : n_(n), x_(n + 1), y_(n + 1), f_(n + 1), rsq_(n + 1, 0.0), a_((size_t)(n + 1) * 5, 0.0) {
    constexpr double kDtol = 0.01, kRtol = 1.0e-05, kSf = 1.0;
    for (int k = 1; k <= n; ++k) {
        x_[k] = x[k - 1];
        y_[k] = y[k - 1];
        f_[k] = f[k - 1];
    }
    nr_ = (int)std::sqrt((float)n / 3.0f);  // int(sqrt(float(np)/3.)), single precision
    const int nqwmax = std::max(nq, nw), lmax = std::min(40, n - 1);
    if (nq < 5 || nw < 1 || lmax < nqwmax || nr_ < 1) throw GridFail{"interface fit: too few points (QSHEP2 ier = 1)"};
    // STORE2: cell lists, nodes entered from n down to 1
    xmin_ = *std::min_element(x_.begin() + 1, x_.end());
    const double xmax = *std::max_element(x_.begin() + 1, x_.end());
    ymin_ = *std::min_element(y_.begin() + 1, y_.end());
    const double ymax = *std::max_element(y_.begin() + 1, y_.end());
    dx_ = (xmax - xmin_) / (double)nr_;
    dy_ = (ymax - ymin_) / (double)nr_;
    if (dx_ == 0.0 || dy_ == 0.0) throw GridFail{"interface fit: points on a line (STORE2 ier = 2)"};
    cell_.assign((size_t)nr_ * nr_, 0);
    next_.assign(n + 1, 0);
    for (int k = n; k >= 1; --k) {
        const int i = std::min((int)((x_[k] - xmin_) / dx_) + 1, nr_);
        const int j = std::min((int)((y_[k] - ymin_) / dy_) + 1, nr_);
        const int l = cell(i, j);
        next_[k] = l != 0 ? l : k;
        cell(i, j) = k;
    }
    double rsmx = 0.0;
    Tri B;
    std::memset(&B, 0, sizeof(B));
    for (int k = 1; k <= n; ++k) {
        const double xk = x_[k], yk = y_[k], fk = f_[k];
        next_[k] = -next_[k];
        double rs = 0.0, sum2 = 0.0, rws = 0.0, rq = 0.0, avsq = 0.0, rsold;
        int lnp = 0, neq = 0;
        int npts[41] = {0};
        // nearest nodes until nq and nw are both passed
        for (;;) {
            sum2 += rs;
            if (lnp == lmax) {
                if (rws == 0.0) rws = 1.1 * rs;
                if (rq == 0.0) {
                    neq = lmax;
                    rq = std::sqrt(1.1 * rs);
                    avsq = sum2 / (double)neq;
                }
                break;
            }
            ++lnp;
            rsold = rs;
            npts[lnp] = nearest(xk, yk, &rs);
            if (rs == 0.0) throw GridFail{"interface fit: duplicate points (QSHEP2 ier = 2)"};
            if ((rs - rsold) / rs < kRtol) continue;
            if (rws == 0.0 && nw < lnp) rws = rs;
            if (rq == 0.0 && nq < lnp) {
                neq = lnp - 1;
                rq = std::sqrt(rs);
                avsq = sum2 / (double)neq;
            }
            if (nqwmax < lnp) break;
        }
        rsq_[k] = rws;
        rsmx = std::max(rsmx, rws);
        const double av = std::sqrt(avsq);
        // least squares by Givens rotations, equation by equation
        int i = 0;
        for (;;) {
            ++i;
            const int np = npts[i], irow = std::min(i, 6);
            B.equation(irow, xk, yk, fk, x_[np], y_[np], f_[np], av, avsq, rq);
            if (i == 1) continue;
            for (int j = 1; j < irow; ++j) {
                double c, s;
                givens(B.at(j, j), B.at(j, irow), c, s);
                B.rot(6 - j, c, s, j + 1, j, irow);
            }
            if (i < neq) continue;
            if (kDtol <= B.dmin() * rq) break;
            if (neq == lmax) {
                // still ill-conditioned with every equation: damp the quadratic terms
                for (int ii = 1; ii <= 3; ++ii) {
                    B.at(ii, 6) = kSf;
                    for (int q = ii + 1; q <= 6; ++q) B.at(q, 6) = 0.0;
                    for (int j = ii; j <= 5; ++j) {
                        double c, s;
                        givens(B.at(j, j), B.at(j, 6), c, s);
                        B.rot(6 - j, c, s, j + 1, j, 6);
                    }
                }
                if (B.dmin() * rq < kDtol) throw GridFail{"interface fit: ill-conditioned (QSHEP2 ier = 3)"};
                break;
            }
            // one more equation: grow the radius to the next distinct node
            for (;;) {
                rsold = rs;
                ++neq;
                if (neq == lmax) {
                    rq = std::sqrt(1.1 * rs);
                    break;
                }
                if (neq != lnp) {
                    const int np2 = npts[neq + 1];
                    const double ex = x_[np2] - xk, ey = y_[np2] - yk;
                    rs = ex * ex + ey * ey;
                    if ((rs - rsold) / rs < kRtol) continue;
                    rq = std::sqrt(rs);
                    break;
                }
                ++lnp;
                const int np2 = nearest(xk, yk, &rs);
                if (np2 == 0) throw GridFail{"interface fit: no further point (QSHEP2 ier = 2)"};
                npts[lnp] = np2;
                if ((rs - rsold) / rs < kRtol) continue;
                rq = std::sqrt(rs);
                break;
            }
        }
        double *ak = &a_[(size_t)k * 5];  // ak[0..4] = a(1..5, k)
        for (int r = 5; r >= 1; --r) {
            double t = 0.0;
            for (int j = r + 1; j <= 5; ++j) t = t + B.at(j, r) * ak[j - 1];
            ak[r - 1] = (B.at(6, r) - t) / B.at(r, r);
        }
        for (int q = 0; q < 3; ++q) ak[q] = ak[q] / avsq;
        ak[3] = ak[3] / av;
        ak[4] = ak[4] / av;
        next_[k] = -next_[k];
        for (int q = 1; q <= lnp; ++q) next_[npts[q]] = -next_[npts[q]];
    }
    rmax_ = std::sqrt(rsmx);
}

double Surface::value(double px, double py) const {
    if (n_ < 6 || nr_ < 1 || dx_ <= 0.0 || dy_ <= 0.0 || rmax_ < 0.0) return 0.0;
    const int imin = std::max((int)((px - xmin_ - rmax_) / dx_) + 1, 1);
    const int imax = std::min((int)((px - xmin_ + rmax_) / dx_) + 1, nr_);
    const int jmin = std::max((int)((py - ymin_ - rmax_) / dy_) + 1, 1);
    const int jmax = std::min((int)((py - ymin_ + rmax_) / dy_) + 1, nr_);
    if (imax < imin || jmax < jmin) return 0.0;
    double sw = 0.0, swq = 0.0;
    for (int j = jmin; j <= jmax; ++j)
        for (int i = imin; i <= imax; ++i) {
            int k = cell(i, j);
            if (k == 0) continue;
            for (;;) {
                const double delx = px - x_[k], dely = py - y_[k];
                const double ds = delx * delx + dely * dely, rs = rsq_[k];
                if (ds < rs) {
                    if (ds == 0.0) return f_[k];
                    const double rds = rs * ds, rd = std::sqrt(rds);
                    const double w = (rs + ds - rd - rd) / rds;
                    const double *ak = &a_[(size_t)k * 5];
                    sw = sw + w;
                    swq = swq + w * (f_[k] + ak[0] * delx * delx + ak[1] * delx * dely + ak[2] * dely * dely +
                                     ak[3] * delx + ak[4] * dely);
                }
                const int kp = k;
                k = next_[kp];
                if (k == kp) break;
            }
        }
    return sw == 0.0 ? 0.0 : swq / sw;
}

// ------------------------------------------------------------------ grid_3d

struct Built {
    mvf_grid_info info{};
    std::vector<double> xp, yp, zp;
    std::vector<int32_t> nzl;
};

void build_grid(const mvf_grid_in &in, Built &g) {
    if (in.nodes_per_elem != 8 && in.nodes_per_elem != 20 && in.nodes_per_elem != 27)
        throw GridFail{"nodes_per_elem must be 8, 20 or 27"};
    if (in.nsf0 < 1 || !in.nsp || !in.pts) throw GridFail{"at least one interface is required"};
    if (in.nsr < 0 || (in.nsr > 0 && !in.rx)) throw GridFail{"bad receiver arrays"};
    if (in.mx < 1 || in.my < 1 || in.mz < 1 || !in.xm || !in.ym || !in.zm) throw GridFail{"bad inner model arrays"};
    if (in.nf < 1 || !in.freqs) throw GridFail{"at least one frequency is required"};
    if (!(in.dx > 0.0 && in.dy > 0.0 && in.dz > 0.0) || !(in.sigma_bg > 0.0))
        throw GridFail{"cell sizes and background conductivity must be positive"};
    const int nord = in.nodes_per_elem == 8 ? 2 : 3, nsf0 = in.nsf0, nsf = nsf0 + 3;
    // interfaces 1..nsf: 1 bottom, 2..nsf0+1 the input ones, nsf-1 air, nsf top
    std::vector<int> nsp(nsf + 1, 0);
    std::vector<std::vector<double>> xto(nsf + 1), yto(nsf + 1), zto(nsf + 1);
    {
        int64_t off = 0;
        for (int l = 0; l < nsf0; ++l) {
            const int n = in.nsp[l];
            if (n < 20) throw GridFail{"interface " + std::to_string(l + 1) + " has fewer than 20 points"};
            nsp[l + 2] = n;
            for (int q = 0; q < n; ++q, ++off) {
                xto[l + 2].push_back(in.pts[3 * off]);
                yto[l + 2].push_back(in.pts[3 * off + 1]);
                zto[l + 2].push_back(in.pts[3 * off + 2]);
            }
        }
    }
    const int64_t nm = (int64_t)in.mx * in.my * in.mz;

    // min_max_input
    double xmin = 1.0e20, xmax = -1.0e20, ymin = 1.0e20, ymax = -1.0e20, zmin = 1.0e20, zmax = -1.0e20;
    double x1 = 1.0e20, x2 = -1.0e20, y1 = 1.0e20, y2 = -1.0e20, zl = 1.0e20, zu = -1.0e20;
    for (int i = 0; i < in.nsr; ++i) {
        const double xs = in.rx[3 * i], ys = in.rx[3 * i + 1], zs = in.rx[3 * i + 2];
        if (xs < xmin) xmin = xs;
        if (xs > xmax) xmax = xs;
        if (ys < ymin) ymin = xs;  // the reference takes x here (Q14)
        if (ys > ymax) ymax = xs;
        if (zs < zmin) zmin = zs;
        if (zs > zmax) zmax = zs;
    }
    for (int l = 2; l <= nsf - 2; ++l)
        for (int q = 0; q < nsp[l]; ++q) {
            if (xto[l][q] < x1) x1 = xto[l][q];
            if (xto[l][q] > x2) x2 = xto[l][q];
            if (yto[l][q] < y1) y1 = yto[l][q];
            if (yto[l][q] > y2) y2 = yto[l][q];
            if (zto[l][q] < zl) zl = zto[l][q];
            if (zto[l][q] > zu) zu = zto[l][q];
        }
    xmin = std::min(xmin, x1);
    xmax = std::max(xmax, x2);
    ymin = std::min(ymin, y1);
    ymax = std::max(ymax, y2);
    zu = zu + in.high;
    zl = zl - in.depth;
    zmin = std::min(zmin, zl);
    zmax = std::max(zmax, zu);
    for (int i = 0; i < in.mx; ++i) {
        if (in.xm[i] < xmin) xmin = in.xm[i];
        if (in.xm[i] > xmax) xmax = in.xm[i];
    }
    for (int i = 0; i < in.my; ++i) {
        if (in.ym[i] < ymin) ymin = in.ym[i];
        if (in.ym[i] > ymax) ymax = in.ym[i];
    }
    for (int64_t p = 0; p < nm; ++p) {
        if (in.zm[p] < zmin) zmin = in.zm[p];
        if (in.zm[p] > zmax) zmax = in.zm[p];
    }

    // extension: padding cells from the skin depth at the lowest frequency
    const double fact = 1.3;
    double minf = 1.0e20;
    for (int i = 0; i < in.nf; ++i)
        if (in.freqs[i] < minf) minf = in.freqs[i];
    const double ddx = std::min({xmax - xmin, ymax - ymin, zmax - zmin});
    const double depth = std::sqrt(2.0 / (kMu0 * in.sigma_bg * 2.0 * kPi * minf));
    double nd = 2.0;
    if (ddx / depth >= 2.5)
        nd = 1.5;
    else if (ddx / depth < 2.5 && depth / ddx >= 1.5)
        nd = 2.0;
    else if (ddx / depth < 1.5)
        nd = 3.0;
    const double dmin = std::min({in.dx, in.dy, in.dz});
    int nextd = 2;
    for (;; ++nextd) {
        double sum_ex = 0.0;
        for (int i = 1; i <= nextd; ++i) sum_ex = sum_ex + fact * dmin * (double)i;
        if (sum_ex > nd * depth) break;
        if (nextd > 100000) throw GridFail{"extension: no padding width reaches the skin depth"};
    }
    std::vector<double> dmx(nextd + 1), dmy(nextd + 1), dmz(nextd + 1);
    x1 = xmin;
    x2 = xmax;
    y1 = ymin;
    y2 = ymax;
    for (int i = 1; i <= nextd; ++i) {
        dmx[i] = fact * (double)i * in.dx;
        x1 = x1 - dmx[i];
        x2 = x2 + dmx[i];
    }
    for (int i = 1; i <= nextd; ++i) {
        dmy[i] = fact * (double)i * in.dy;
        y1 = y1 - dmy[i];
        y2 = y2 + dmy[i];
    }
    const double x0 = 0.5 * (x1 + x2), y0 = 0.5 * (y1 + y2);
    x1 = x1 - x0;
    x2 = x2 - x0;
    y1 = y1 - y0;
    y2 = y2 - y0;
    xmin = xmin - x0;
    xmax = xmax - x0;
    ymin = ymin - y0;
    ymax = ymax - y0;
    const int nx0 = (int)((xmax - xmin) / in.dx) + 1, ny0 = (int)((ymax - ymin) / in.dy) + 1;
    const int gnx = nx0 + 2 * nextd, gny = ny0 + 2 * nextd;
    std::vector<double> x(gnx + 1), y(gny + 1);  // grid lines, 1-based
    x[1] = x1;
    y[1] = y1;
    for (int i = 1; i <= nextd; ++i) x[i + 1] = x[i] + dmx[nextd + 1 - i];
    for (int i = 1; i <= nextd; ++i) y[i + 1] = y[i] + dmy[nextd + 1 - i];
    for (int i = 1; i <= nx0; ++i) x[i + nextd] = x[nextd + 1] + (double)(i - 1) * in.dx;
    for (int i = 1; i <= ny0; ++i) y[i + nextd] = y[nextd + 1] + (double)(i - 1) * in.dy;
    for (int i = 1; i <= nextd; ++i) x[nextd + nx0 + i] = x[nextd + nx0 + i - 1] + dmx[i];
    for (int i = 1; i <= nextd; ++i) y[nextd + ny0 + i] = y[nextd + ny0 + i - 1] + dmy[i];
    double zbot = zmin, ztop = zmax;
    for (int i = 1; i <= nextd; ++i) {
        dmz[i] = fact * (double)i * in.dz;
        zbot = zbot - dmz[i];
        ztop = ztop + dmz[i];
    }
    // the three added interfaces take the points of their neighbour, flat
    nsp[1] = nsp[2];
    xto[1] = xto[2];
    yto[1] = yto[2];
    zto[1].assign(nsp[1], zmin);
    nsp[nsf - 1] = nsp[nsf - 2];
    xto[nsf - 1] = xto[nsf - 2];
    yto[nsf - 1] = yto[nsf - 2];
    zto[nsf - 1].assign(nsp[nsf - 1], zmax);
    nsp[nsf] = nsp[nsf - 1];
    xto[nsf] = xto[nsf - 1];
    yto[nsf] = yto[nsf - 1];
    zto[nsf].assign(nsp[nsf], ztop);
    const double z0 = zbot;

    // coord_transform of the interfaces; g_ztop
    for (int l = 1; l <= nsf; ++l)
        for (int q = 0; q < nsp[l]; ++q) {
            xto[l][q] = xto[l][q] - x0;
            yto[l][q] = yto[l][q] - y0;
            zto[l][q] = zto[l][q] - z0;
        }
    double gztop = 1.0e20;
    for (int q = 0; q < nsp[nsf - 2]; ++q)
        if (zto[nsf - 2][q] < gztop) gztop = zto[nsf - 2][q];

    // one fit per interface: every interface has >= 20 points, so nq = 13, nw = 19
    std::vector<std::unique_ptr<Surface>> surf(nsf + 1);
    for (int l = 1; l <= nsf; ++l)
        surf[l].reset(new Surface(xto[l].data(), yto[l].data(), zto[l].data(), nsp[l], 13, 19));

    // zblocks: sub-layers of each interval from its thickest point over the core grid lines
    std::vector<int> nzl(nsf + 1);
    nzl[1] = nextd;
    nzl[nsf] = nextd;
    for (int l = 2; l <= nsf - 1; ++l) {
        double h = 0.0;
#pragma omp parallel for reduction(max : h) schedule(static)
        for (int i = nextd + 1; i <= gnx - nextd - 1; ++i)
            for (int j = nextd + 1; j <= gny - nextd - 1; ++j) {
                const double dh = surf[l]->value(x[i], y[j]) - surf[l - 1]->value(x[i], y[j]);
                if (dh > h) h = dh;
            }
        nzl[l] = std::max((int)(h / in.dz), 1);
    }
    int gnz = 1;
    for (int l = 1; l <= nsf; ++l) gnz += nzl[l];

    const int64_t nnx = (int64_t)(gnx - 1) * (nord - 1) + 1, nny = (int64_t)(gny - 1) * (nord - 1) + 1;
    const int64_t nnz = (int64_t)(gnz - 1) * (nord - 1) + 1, nyz = nny * nnz;
    g.xp.assign(nnx, 0.0);
    g.yp.assign(nny, 0.0);
    g.zp.assign(nnx * nny * nnz, 0.0);
    double as[4];
    const double fn = 2.0 / (double)(nord - 1);
    for (int q = 1; q <= nord; ++q) as[q] = -1 + (double)(q - 1) * fn;

    // gauss_grid: the writer of each node column is the last cell in loop order
    const int ilo = nextd + 1, ihi = gnx - nextd - 1, jlo = nextd + 1, jhi = gny - nextd + 1;
    const int64_t ii0 = (int64_t)(ilo - 1) * (nord - 1) + 1, ii1 = (int64_t)ihi * (nord - 1) + 1;
    const int64_t jj0 = (int64_t)(jlo - 1) * (nord - 1) + 1, jj1 = (int64_t)jhi * (nord - 1) + 1;
    auto owner = [nord](int64_t node, int hi, int *loc) {  // last cell (<= hi) holding `node`
        int c = (int)((node - 1) / (nord - 1)) + 1;
        if (c > hi) c = hi;
        *loc = (int)(node - (int64_t)(c - 1) * (nord - 1));
        return c;
    };
    for (int64_t ii = ii0; ii <= ii1; ++ii) {
        int i1;
        const int i = owner(ii, ihi, &i1);
        g.xp[ii - 1] = 0.5 * (x[i + 1] - x[i]) * as[i1] + 0.5 * (x[i] + x[i + 1]);
    }
    for (int64_t jj = jj0; jj <= jj1; ++jj) {
        int j1;
        const int j = owner(jj, jhi, &j1);
        g.yp[jj - 1] = 0.5 * (y[j + 1] - y[j]) * as[j1] + 0.5 * (y[j] + y[j + 1]);
    }
#pragma omp parallel for collapse(2) schedule(static)
    for (int64_t ii = ii0; ii <= ii1; ++ii)
        for (int64_t jj = jj0; jj <= jj1; ++jj) {
            int i1, j1;
            const int i = owner(ii, ihi, &i1), j = owner(jj, jhi, &j1);
            const double xi = 0.5 * (x[i + 1] - x[i]) * as[i1] + 0.5 * (x[i] + x[i + 1]);
            const double yj = 0.5 * (y[j + 1] - y[j]) * as[j1] + 0.5 * (y[j] + y[j + 1]);
            double *col = &g.zp[(size_t)((ii - 1) * nyz + (jj - 1) * nnz)];
            double z2 = 0.0;
            int k = 0;
            for (int l = 1; l <= nsf; ++l) {
                const double h2 = surf[l]->value(xi, yj);
                const double h1 = l == 1 ? 0.0 : surf[l - 1]->value(xi, yj);  // layer 1 starts at z = 0
                const double dm = (h2 - h1) / (double)nzl[l];
                for (int s = 1; s <= nzl[l]; ++s) {
                    ++k;
                    const double z1 = z2;
                    z2 = z1 + dm;
                    const int64_t base = (int64_t)(k - 1) * (nord - 1);
                    for (int k1 = 1; k1 <= nord; ++k1) col[base + k1 - 1] = 0.5 * (z2 - z1) * as[k1] + 0.5 * (z1 + z2);
                }
            }
        }

    // complete_grid: the padding columns copy the core's edge columns
    auto block = [&](int i, int j, int ic, int jc, int lsrc, int msrc, bool setx, bool sety) {
        for (int k = 1; k <= gnz - 1; ++k) {
            const int64_t no = (int64_t)(i - 1) * (nord - 1) * nyz + (int64_t)(j - 1) * (nord - 1) * nnz +
                               (int64_t)(k - 1) * (nord - 1);
            const int64_t no1 = (int64_t)(ic - 1) * (nord - 1) * nyz + (int64_t)(jc - 1) * (nord - 1) * nnz +
                                (int64_t)(k - 1) * (nord - 1);
            for (int l = 1; l <= nord; ++l) {
                const int l1 = lsrc ? lsrc : l;
                if (setx) g.xp[(i - 1) * (nord - 1) + l - 1] = 0.5 * (x[i + 1] - x[i]) * as[l] + 0.5 * (x[i] + x[i + 1]);
                for (int m = 1; m <= nord; ++m) {
                    const int m1 = msrc ? msrc : m;
                    if (sety)
                        g.yp[(j - 1) * (nord - 1) + m - 1] = 0.5 * (y[j + 1] - y[j]) * as[m] + 0.5 * (y[j] + y[j + 1]);
                    for (int n = 1; n <= nord; ++n)
                        g.zp[no + (int64_t)(l - 1) * nyz + (int64_t)(m - 1) * nnz + (n - 1)] =
                            g.zp[no1 + (int64_t)(l1 - 1) * nyz + (int64_t)(m1 - 1) * nnz + (n - 1)];
                }
            }
        }
    };
    for (int i = 1; i <= nextd; ++i)
        for (int j = nextd + 1; j <= gny - nextd - 1; ++j) block(i, j, nextd + 1, j, 1, 0, true, false);
    for (int i = gnx - nextd; i <= gnx - 1; ++i)
        for (int j = nextd + 1; j <= gny - nextd - 1; ++j) block(i, j, gnx - nextd - 1, j, nord, 0, true, false);
    for (int i = 1; i <= gnx - 1; ++i)
        for (int j = 1; j <= nextd; ++j) block(i, j, i, nextd + 1, 0, 1, false, true);
    for (int i = 1; i <= gnx - 1; ++i)
        for (int j = gny - nextd; j <= gny - 1; ++j) block(i, j, i, gny - nextd - 1, 0, nord, false, true);

    g.nzl.assign(nzl.begin() + 1, nzl.end());
    mvf_grid_info &f = g.info;
    f.nodes_per_elem = in.nodes_per_elem;
    f.nextd = nextd;
    f.nsf = nsf;
    f.nx = gnx - 1;
    f.ny = gny - 1;
    f.nz = gnz - 1;
    f.nnx = nnx;
    f.nny = nny;
    f.nnz = nnz;
    f.npt = nnx * nny * nnz;
    f.nzl_top = nzl[nsf];
    f.nzl_air = nzl[nsf - 1];
    f.x0 = x0;
    f.y0 = y0;
    f.z0 = z0;
    f.ztop = gztop;
    f.skin_depth = depth;
    f.nd = nd;
}

}  // namespace

struct mvf_grid {
    Built g;
};

extern "C" int mvf_grid_3d(const mvf_grid_in *in, mvf_grid **out) {
    if (!in || !out) {
        mvf::set_host_error("null argument");
        return MVF_E_ARG;
    }
    *out = nullptr;
    std::unique_ptr<mvf_grid> h(new mvf_grid);
    try {
        build_grid(*in, h->g);
    } catch (const GridFail &e) {
        mvf::set_host_error(e.msg.c_str());
        return MVF_E_ARG;
    } catch (const std::bad_alloc &) {
        mvf::set_host_error("host allocation failed");
        return MVF_E_NOMEM;
    }
    *out = h.release();
    return 0;
}

extern "C" int mvf_grid_get_info(const mvf_grid *g, mvf_grid_info *info) {
    if (!g || !info) return MVF_E_ARG;
    *info = g->g.info;
    return 0;
}

extern "C" int mvf_grid_export(const mvf_grid *g, double *xp, double *yp, double *zp, int32_t *nzl) {
    if (!g) return MVF_E_ARG;
    const Built &b = g->g;
    if (xp) std::memcpy(xp, b.xp.data(), b.xp.size() * sizeof(double));
    if (yp) std::memcpy(yp, b.yp.data(), b.yp.size() * sizeof(double));
    if (zp) std::memcpy(zp, b.zp.data(), b.zp.size() * sizeof(double));
    if (nzl) std::memcpy(nzl, b.nzl.data(), b.nzl.size() * sizeof(int32_t));
    return 0;
}

extern "C" void mvf_grid_destroy(mvf_grid *g) { delete g; }
