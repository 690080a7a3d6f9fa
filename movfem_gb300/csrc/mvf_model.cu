// mvf_model.cu -- nodal conductivity and permeability of the grid from the inner
// geomodel (innermodel_gqg, min_dd_inner, assign_model: geometry.f90:804-1085).
//
// The reference visits every node of every inner element and scans all mx*my*mz
// model points for it (O(nodes x points), repeated for each element sharing the
// node).  The node's value depends only on its coordinates: the first point in point
// order within 1e-5 m, else the first point at the smallest distance.  Here one
// thread maps one node of the inner box, once, with an exact pruned scan:
//
//  1. seed: the distances to the points of the column nearest in x and in y give an
//     upper bound T = max(seed minimum, 1e-5) on the distance of the answer;
//  2. scan the points in the reference's order, skipping an x row, a column or a
//     point whose partial squared distance already exceeds T^2 (1 + 1e-14).  The
//     partial sums are the reference's own left-to-right sums, each term >= 0, so a
//     skipped point's rounded distance is > T: it could be neither within 1e-5 nor a
//     new minimum.  The points that remain see the reference's comparisons (<= 1e-5
//     first, strict < for the minimum), so ties resolve to the same point.
//  3. where xm, ym or a column's zm are sorted (ascending; columns either way), the
//     rows, columns or points whose own squared term is within T^2 (1 + 1e-14) form one
//     contiguous run -- the rounded square of a rounded difference is monotone on each
//     side of the node's coordinate -- found by binary search; everything outside that
//     run is exactly what step 2 would skip.  Unsorted arrays are scanned in full.
//
// Distances are the reference's sqrt((x-xm)^2 + (y-ym)^2 + (z-zm)^2) with explicitly
// rounded operations (no contraction into FMA), so the comparisons see the same
// values as the FP64 oracle.  The five copy phases that follow run as one launch
// each, in the reference's order: x-extension planes, y-extension planes, the layers
// below the inner elements, the air, and the negative-entry pass (each negative real
// part takes the node below's value; one thread per node column, bottom to top).
#include <cmath>
#include <cstdio>
#include <string>

#include "mvf_internal.cuh"

namespace mvf {
namespace {

thread_local std::string g_map_err;

int map_fail(int code, const std::string &msg) {
    g_map_err = msg;
    return code;
}

struct MapDims {
    int64_t nnx, nny, nnz, nyz;
    int E;            // extension nodes per side: nextd * (nord - 1)
    int64_t ktop;     // first air node (0-based): nnz - (nzl_top + nzl_air) * (nord - 1)
    int64_t bi0, bj0, bk0, bni, bnj, bnk;  // inner box: origin and extent in nodes
};

struct ModelDev {
    int32_t mx, my, mz, isigma, imu;
    const double *xm, *ym, *zm, *sigma, *mu;
    const int8_t *zsort;                 // [mx*my]: +1 zm ascending, -1 descending, 0 neither
    int32_t xsorted, ysorted;            // xm / ym ascending
    int8_t slot_sigma[16], slot_mu[16];  // component -> 0-based packed slot
};

constexpr double MU0 = 4.0 * 3.1415926535897932384626433 * 1.e-7;  // geometry.f90:25
constexpr double HIT = 1.e-5;   // min_dd_inner's coincidence distance
constexpr double FAR = 1.e20;   // min_dd_inner's initial minimum
constexpr double MARGIN = 1.0 + 1e-14;

__device__ __forceinline__ double sq(double a) { return __dmul_rn(a, a); }

// reference distance: sqrt(((x-xm)^2 + (y-ym)^2) + (z-zm)^2), every step rounded
__device__ __forceinline__ double part_xy(double x, double y, double xm, double ym) {
    return __dadd_rn(sq(__dsub_rn(x, xm)), sq(__dsub_rn(y, ym)));
}

// [lo, hi] of the entries v[0..n) (sorted: dir +1 ascending, -1 descending) whose
// rounded squared difference to t is <= T2; lo > hi when there is none.  The predicate
// "on t's lower side, or close enough" is monotone along the array, and so is "on t's
// upper side, or close enough", so two bisections find the run.
__device__ __forceinline__ int2 close_run(const double *__restrict__ v, int n, int dir, double t, double T2) {
    int lo = 0, hi = n;  // first c with (past t or close)
    while (lo < hi) {
        const int c = (lo + hi) >> 1;
        const double a = __ldg(v + c);
        const bool past = dir > 0 ? a >= t : a <= t;
        if (past || sq(__dsub_rn(t, a)) <= T2) hi = c;
        else lo = c + 1;
    }
    const int first = lo;
    lo = -1;
    hi = n - 1;  // last c with (before t or close)
    while (lo < hi) {
        const int c = (lo + hi + 1) >> 1;
        const double a = __ldg(v + c);
        const bool before = dir > 0 ? a <= t : a >= t;
        if (before || sq(__dsub_rn(t, a)) <= T2) lo = c;
        else hi = c - 1;
    }
    return make_int2(first, lo);
}

// index of an entry of the ascending v[0..n) nearest to t (any one of equal distance)
__device__ __forceinline__ int nearest_sorted(const double *__restrict__ v, int n, double t) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int c = (lo + hi) >> 1;
        if (__ldg(v + c) < t) lo = c + 1;
        else hi = c;
    }
    if (lo == n) return n - 1;
    if (lo > 0 && fabs(t - __ldg(v + lo - 1)) < fabs(__ldg(v + lo) - t)) return lo - 1;
    return lo;
}

__device__ void assign(const ModelDev &m, int64_t p, double ieps, double *__restrict__ sigma,
                       double *__restrict__ mu, int64_t id) {
    double s[12], u[6];
#pragma unroll
    for (int c = 0; c < 12; ++c) s[c] = 0.0;
#pragma unroll
    for (int c = 0; c < 6; ++c) u[c] = 0.0;
    if (m.isigma == 1) {
        const double v = m.sigma[p];
        s[0] = v; s[1] = ieps; s[6] = v; s[7] = ieps; s[10] = v; s[11] = ieps;
    } else {
        for (int c = 0; c < m.isigma; ++c) {
            const int k = m.slot_sigma[c];
            s[2 * k] = m.sigma[p * m.isigma + c];
            s[2 * k + 1] = 0.0;
        }
        s[0] = __dadd_rn(s[0], 0.0); s[1] = __dadd_rn(s[1], ieps);
        s[6] = __dadd_rn(s[6], 0.0); s[7] = __dadd_rn(s[7], ieps);
        s[10] = __dadd_rn(s[10], 0.0); s[11] = __dadd_rn(s[11], ieps);
    }
    if (m.imu <= 1) {
        const double v = __dmul_rn(MU0, m.imu == 0 ? 1.0 : m.mu[p]);
        u[0] = v; u[3] = v; u[5] = v;
    } else {
        for (int c = 0; c < m.imu; ++c) u[m.slot_mu[c]] = __dmul_rn(MU0, m.mu[p * m.imu + c]);
    }
    double2 *s2 = reinterpret_cast<double2 *>(sigma + id * 12);
#pragma unroll
    for (int c = 0; c < 6; ++c) s2[c] = make_double2(s[2 * c], s[2 * c + 1]);
#pragma unroll
    for (int c = 0; c < 6; ++c) mu[id * 6 + c] = u[c];
}

// one thread per node of the inner box (k fastest, so a warp shares x and y and takes
// the same branches of the pruned scan)
__global__ void __launch_bounds__(256) map_nearest(MapDims g, ModelDev m, double ieps,
                                                   const double *__restrict__ xp, const double *__restrict__ yp,
                                                   const double *__restrict__ zp, double *__restrict__ sigma,
                                                   double *__restrict__ mu, uint8_t *__restrict__ valued,
                                                   int32_t *__restrict__ err) {
    const int64_t nbox = g.bni * g.bnj * g.bnk;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nbox; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t bk = t % g.bnk, r = t / g.bnk;
        const int64_t i = g.bi0 + r / g.bnj, j = g.bj0 + r % g.bnj, k = g.bk0 + bk;
        const int64_t id = i * g.nyz + j * g.nnz + k;
        const double x = xp[i], y = yp[j], z = zp[id];
        // 1. seed column: nearest xm and nearest ym
        int ia = 0, ja = 0;
        if (m.xsorted) {
            ia = nearest_sorted(m.xm, m.mx, x);
        } else {
            double bx = fabs(x - __ldg(m.xm));
            for (int a = 1; a < m.mx; ++a) {
                const double v = fabs(x - __ldg(m.xm + a));
                if (v < bx) { bx = v; ia = a; }
            }
        }
        if (m.ysorted) {
            ja = nearest_sorted(m.ym, m.my, y);
        } else {
            double by = fabs(y - __ldg(m.ym));
            for (int b = 1; b < m.my; ++b) {
                const double v = fabs(y - __ldg(m.ym + b));
                if (v < by) { by = v; ja = b; }
            }
        }
        double seed = FAR;
        {
            const double cxy = part_xy(x, y, __ldg(m.xm + ia), __ldg(m.ym + ja));
            const double *zc = m.zm + ((int64_t)ia * m.my + ja) * m.mz;
            const int dir = m.zsort[(int64_t)ia * m.my + ja];
            int c0 = 0, c1 = m.mz - 1;
            if (dir != 0) {
                // the entries either side of z in the sorted column
                int lo = 0, hi = m.mz;
                while (lo < hi) {
                    const int c = (lo + hi) >> 1;
                    if (dir > 0 ? __ldg(zc + c) < z : __ldg(zc + c) > z) lo = c + 1;
                    else hi = c;
                }
                c0 = max(lo - 1, 0);
                c1 = min(lo, m.mz - 1);
            }
            for (int c = c0; c <= c1; ++c) {
                const double dd = __dsqrt_rn(__dadd_rn(cxy, sq(__dsub_rn(z, __ldg(zc + c)))));
                if (dd < seed) seed = dd;
            }
        }
        const double T = seed > HIT ? seed : HIT;
        const double T2 = T * T * MARGIN;
        // 2. the reference's scan over the points that can still matter
        const int2 xr = m.xsorted ? close_run(m.xm, m.mx, 1, x, T2) : make_int2(0, m.mx - 1);
        const int2 yr = m.ysorted ? close_run(m.ym, m.my, 1, y, T2) : make_int2(0, m.my - 1);
        double ddmin = FAR;
        int64_t best = -1;
        bool hit = false;
        for (int a = xr.x; a <= xr.y && !hit; ++a) {
            const double cx = sq(__dsub_rn(x, __ldg(m.xm + a)));
            if (cx > T2) continue;
            for (int b = yr.x; b <= yr.y && !hit; ++b) {
                const double cxy = __dadd_rn(cx, sq(__dsub_rn(y, __ldg(m.ym + b))));
                if (cxy > T2) continue;
                const int64_t base = ((int64_t)a * m.my + b) * m.mz;
                const int dir = m.zsort[(int64_t)a * m.my + b];
                const int2 zr = dir != 0 ? close_run(m.zm + base, m.mz, dir, z, T2) : make_int2(0, m.mz - 1);
                for (int c = zr.x; c <= zr.y; ++c) {
                    const double s = __dadd_rn(cxy, sq(__dsub_rn(z, __ldg(m.zm + base + c))));
                    if (s > T2) continue;
                    const double dd = __dsqrt_rn(s);
                    if (dd <= HIT) {
                        best = base + c;
                        hit = true;
                        break;
                    }
                    if (dd < ddmin) {
                        ddmin = dd;
                        best = base + c;
                    }
                }
            }
        }
        if (best < 0) {
            atomicExch(err, 1);
            continue;
        }
        assign(m, best, ieps, sigma, mu, id);
        valued[id] = 1;
    }
}

__device__ __forceinline__ void copy_node(double *__restrict__ sigma, double *__restrict__ mu,
                                          uint8_t *__restrict__ valued, int64_t id, int64_t ip) {
    if (valued[id]) return;
    double2 *sd = reinterpret_cast<double2 *>(sigma + id * 12);
    const double2 *ss = reinterpret_cast<const double2 *>(sigma + ip * 12);
#pragma unroll
    for (int c = 0; c < 6; ++c) sd[c] = ss[c];
#pragma unroll
    for (int c = 0; c < 6; ++c) mu[id * 6 + c] = mu[ip * 6 + c];
    valued[id] = 1;
}

// phases 1 and 2 (geometry.f90:854-913): the two extension slabs normal to `axis`
// (0: x, 1: y) take the value of the last inner plane, over node layers [E-1, ktop).
// The sources are never destinations of the same phase.
__global__ void map_planes(MapDims g, int axis, double *__restrict__ sigma, double *__restrict__ mu,
                           uint8_t *__restrict__ valued) {
    const int64_t nk = g.ktop - (g.E - 1);
    const int64_t na = 2 * (int64_t)g.E;                             // slab planes
    const int64_t nb = axis == 0 ? g.nny - 2 * (int64_t)g.E : g.nnx;  // other horizontal axis
    const int64_t n = na * nb * nk;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = (g.E - 1) + t % nk, r = t / nk;
        const int64_t b = r % nb, a = r / nb;
        const int64_t len = axis == 0 ? g.nnx : g.nny;
        const int64_t pa = a < g.E ? a : len - 2 * g.E + a;  // plane index along the axis
        const int64_t src = a < g.E ? g.E : len - g.E - 1;
        int64_t id, ip;
        if (axis == 0) {
            const int64_t j = g.E + b;
            id = pa * g.nyz + j * g.nnz + k;
            ip = src * g.nyz + j * g.nnz + k;
        } else {
            id = b * g.nyz + pa * g.nnz + k;
            ip = b * g.nyz + src * g.nnz + k;
        }
        copy_node(sigma, mu, valued, id, ip);
    }
}

// phase 3 (geometry.f90:915-926): node layers [0, E-1) take layer E-1
__global__ void map_bottom(MapDims g, double *__restrict__ sigma, double *__restrict__ mu,
                           uint8_t *__restrict__ valued) {
    const int64_t nk = g.E - 1;
    const int64_t n = g.nnx * g.nny * nk;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = t % nk, col = t / nk;
        copy_node(sigma, mu, valued, col * g.nnz + k, col * g.nnz + (g.E - 1));
    }
}

// phase 4 (geometry.f90:928-940): air layers [ktop, nnz)
__global__ void map_air(MapDims g, double ieps, double *__restrict__ sigma, double *__restrict__ mu) {
    const int64_t nk = g.nnz - g.ktop;
    const int64_t n = g.nnx * g.nny * nk;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t id = (t / nk) * g.nnz + g.ktop + t % nk;
        double2 *s2 = reinterpret_cast<double2 *>(sigma + id * 12);
#pragma unroll
        for (int c = 0; c < 6; ++c) s2[c] = make_double2(0.0, (c == 0 || c == 3 || c == 5) ? ieps : 0.0);
#pragma unroll
        for (int c = 0; c < 6; ++c) mu[id * 6 + c] = (c == 0 || c == 3 || c == 5) ? MU0 : 0.0;
    }
}

// phase 5 (geometry.f90:942-955): a negative real part takes the previous node's
// value, in node order.  One thread per (column, component), bottom to top.  The
// bottom node of column c > 0 reads the top node of column c-1: an air node, which
// this pass never changes, so the columns are independent.  Node 0 has no
// predecessor (the reference reads before its array there) and is left as it is.
__global__ void map_fixup(MapDims g, double *__restrict__ sigma, double *__restrict__ mu) {
    const int64_t n = g.nnx * g.nny * 6;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(t % 6);
        const int64_t col = t / 6;
        for (int64_t k = 0; k < g.nnz; ++k) {
            const int64_t id = col * g.nnz + k;
            if (id == 0) continue;
            double2 *s = reinterpret_cast<double2 *>(sigma + id * 12) + c;
            if (s->x < 0) *s = *(reinterpret_cast<const double2 *>(sigma + (id - 1) * 12) + c);
            if (mu[id * 6 + c] < 0) mu[id * 6 + c] = mu[(id - 1) * 6 + c];
        }
    }
}

__global__ void map_init(int64_t npt, double *__restrict__ sigma, double *__restrict__ mu, uint8_t *__restrict__ valued) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < npt; t += (int64_t)gridDim.x * blockDim.x) {
        double2 *s2 = reinterpret_cast<double2 *>(sigma + t * 12);
#pragma unroll
        for (int c = 0; c < 6; ++c) s2[c] = make_double2(-1.0, 0.0);  // g_sigma = cmplx(-1, 0)
#pragma unroll
        for (int c = 0; c < 6; ++c) mu[t * 6 + c] = -1.0;              // g_mu = -1
        valued[t] = 0;
    }
}

unsigned grid_for(int64_t n, int threads) {
    const int64_t b = (n + threads - 1) / threads;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, 152LL * 64));
}

bool components_ok(int32_t n, const int32_t *ij, int8_t *slot) {
    if (n > 16 || !ij) return false;
    for (int c = 0; c < n; ++c) {
        const int a = ij[c], b = ij[n + c];
        if (a < 1 || a > 3 || b < 1 || b > 3) return false;
        slot[c] = (int8_t)((a == 1 ? b : a + b) - 1);  // assign_model's select case
    }
    return true;
}

struct DevBuf {
    void *p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

}  // namespace
}  // namespace mvf

using namespace mvf;

extern "C" int mvf_map_model(const mvf_mesh *grid, const mvf_model *md, double omega, double *sigma_out,
                             double *mu_out, double *seconds, int32_t device) {
    g_map_err.clear();
    if (!grid || !md || !sigma_out || !mu_out) return map_fail(MVF_E_ARG, "null argument");
    const mvf_mesh &m = *grid;
    if (m.nodes_per_elem != 8 && m.nodes_per_elem != 20 && m.nodes_per_elem != 27)
        return map_fail(MVF_E_ARG, "nodes_per_elem must be 8, 20 or 27");
    if (!m.xp || !m.yp || !m.zp) return map_fail(MVF_E_ARG, "grid coordinates missing");
    const int o = m.nodes_per_elem == 8 ? 1 : 2;
    const int nair = m.nzl_top + m.nzl_air;
    if (m.nextd < 1) return map_fail(MVF_E_ARG, "nextd must be >= 1 (the mapping visits element layer nextd)");
    if (nair < 1) return map_fail(MVF_E_ARG, "nzl_top + nzl_air must be >= 1 (the grid needs an air zone)");
    if (m.nx - 2 * m.nextd < 1 || m.ny - 2 * m.nextd < 1 || m.nz - nair < m.nextd)
        return map_fail(MVF_E_ARG, "no inner elements: nx, ny > 2*nextd and nz - nzl_top - nzl_air >= nextd needed");
    if (md->mx < 1 || md->my < 1 || md->mz < 1 || !md->xm || !md->ym || !md->zm)
        return map_fail(MVF_E_ARG, "empty inner model");
    if (md->isigma < 1 || !md->sigma) return map_fail(MVF_E_ARG, "isigma must be >= 1");
    if (md->imu < 0 || (md->imu >= 1 && !md->mu)) return map_fail(MVF_E_ARG, "imu must be >= 0 with mu given");
    ModelDev dm{};
    dm.mx = md->mx; dm.my = md->my; dm.mz = md->mz; dm.isigma = md->isigma; dm.imu = md->imu;
    if (md->isigma > 1 && !components_ok(md->isigma, md->ijsigma, dm.slot_sigma))
        return map_fail(MVF_E_ARG, "ijsigma: up to 16 components with indices in 1..3");
    if (md->imu > 1 && !components_ok(md->imu, md->ijmu, dm.slot_mu))
        return map_fail(MVF_E_ARG, "ijmu: up to 16 components with indices in 1..3");

    MapDims g{};
    g.nnx = (int64_t)m.nx * o + 1;
    g.nny = (int64_t)m.ny * o + 1;
    g.nnz = (int64_t)m.nz * o + 1;
    g.nyz = g.nny * g.nnz;
    g.E = m.nextd * o;
    g.ktop = g.nnz - (int64_t)nair * o;
    g.bi0 = g.E;
    g.bj0 = g.E;
    g.bk0 = (int64_t)(m.nextd - 1) * o;
    g.bni = (int64_t)(m.nx - 2 * m.nextd) * o + 1;
    g.bnj = (int64_t)(m.ny - 2 * m.nextd) * o + 1;
    g.bnk = (int64_t)(m.nz - nair - m.nextd + 1) * o + 1;
    const int64_t npt = g.nnx * g.nyz;
    const int64_t npts = (int64_t)md->mx * md->my * md->mz;
    const double ieps = (m.quirks & MVF_Q_FP32_CONST) ? (double)(float)(8.854187817e-12 * omega)
                                                      : 8.854187817e-12 * omega;

    // the caller's current device is restored on return (after the buffers are freed)
    struct DeviceGuard {
        int prev = -1;
        ~DeviceGuard() {
            if (prev >= 0) cudaSetDevice(prev);
        }
    } guard;
    if (device >= 0) {
        int cur = 0;
        cudaError_t e = cudaGetDevice(&cur);
        if (e == cudaSuccess && cur != device) {
            e = cudaSetDevice(device);
            if (e == cudaSuccess) guard.prev = cur;
        }
        if (e != cudaSuccess) return map_fail(MVF_E_CUDA, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
    }
    // sortedness of the model's coordinate arrays (a NaN makes an array unsorted)
    auto ascending = [](const double *v, int64_t n, int64_t stride) {
        for (int64_t c = 0; c + 1 < n; ++c)
            if (!(v[c * stride] <= v[(c + 1) * stride])) return false;
        return true;
    };
    dm.xsorted = ascending(md->xm, md->mx, 1);
    dm.ysorted = ascending(md->ym, md->my, 1);
    std::vector<int8_t> zsort((size_t)md->mx * md->my);
    for (int64_t col = 0; col < (int64_t)md->mx * md->my; ++col) {
        const double *zc = md->zm + col * md->mz;
        bool up = true, down = true;
        for (int c = 0; c + 1 < md->mz && (up || down); ++c) {
            if (!(zc[c] <= zc[c + 1])) up = false;
            if (!(zc[c] >= zc[c + 1])) down = false;
        }
        zsort[col] = up ? 1 : down ? -1 : 0;
    }
    DevBuf bxp, byp, bzp, bxm, bym, bzm, bsig, bmu, bs, bu, bv, berr, bzs;
    auto alloc = [](DevBuf &b, size_t bytes) { return cudaMalloc(&b.p, std::max<size_t>(bytes, 16)); };
    auto put = [](DevBuf &b, const void *h, size_t bytes) {
        cudaError_t e = cudaMalloc(&b.p, std::max<size_t>(bytes, 16));
        return e != cudaSuccess ? e : cudaMemcpy(b.p, h, bytes, cudaMemcpyHostToDevice);
    };
    cudaError_t e = cudaSuccess;
    const int64_t msig = npts * md->isigma, mmu = md->imu >= 1 ? npts * md->imu : 0;
    if (e == cudaSuccess) e = put(bxp, m.xp, sizeof(double) * g.nnx);
    if (e == cudaSuccess) e = put(byp, m.yp, sizeof(double) * g.nny);
    if (e == cudaSuccess) e = put(bzp, m.zp, sizeof(double) * npt);
    if (e == cudaSuccess) e = put(bxm, md->xm, sizeof(double) * md->mx);
    if (e == cudaSuccess) e = put(bym, md->ym, sizeof(double) * md->my);
    if (e == cudaSuccess) e = put(bzm, md->zm, sizeof(double) * npts);
    if (e == cudaSuccess) e = put(bzs, zsort.data(), zsort.size());
    if (e == cudaSuccess) e = put(bsig, md->sigma, sizeof(double) * msig);
    if (e == cudaSuccess && mmu) e = put(bmu, md->mu, sizeof(double) * mmu);
    if (e == cudaSuccess) e = alloc(bs, sizeof(double) * 12 * npt);
    if (e == cudaSuccess) e = alloc(bu, sizeof(double) * 6 * npt);
    if (e == cudaSuccess) e = alloc(bv, npt);
    if (e == cudaSuccess) e = alloc(berr, sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMemset(berr.p, 0, sizeof(int32_t));
    if (e != cudaSuccess)
        return map_fail(e == cudaErrorMemoryAllocation ? MVF_E_NOMEM : MVF_E_CUDA,
                        std::string("model mapping set-up: ") + cudaGetErrorString(e));
    dm.xm = (const double *)bxm.p;
    dm.ym = (const double *)bym.p;
    dm.zm = (const double *)bzm.p;
    dm.sigma = (const double *)bsig.p;
    dm.mu = (const double *)bmu.p;
    dm.zsort = (const int8_t *)bzs.p;
    double *sig = (double *)bs.p, *mu = (double *)bu.p;
    uint8_t *val = (uint8_t *)bv.p;

    cudaEvent_t t0 = nullptr, t1 = nullptr;
    e = cudaEventCreate(&t0);
    if (e == cudaSuccess) e = cudaEventCreate(&t1);
    if (e != cudaSuccess) {
        if (t0) cudaEventDestroy(t0);
        return map_fail(MVF_E_CUDA, std::string("model mapping events: ") + cudaGetErrorString(e));
    }
    cudaEventRecord(t0, 0);
    map_init<<<grid_for(npt, 256), 256>>>(npt, sig, mu, val);
    count_launch();
    map_nearest<<<grid_for(g.bni * g.bnj * g.bnk, 256), 256>>>(g, dm, ieps, (const double *)bxp.p,
                                                               (const double *)byp.p, (const double *)bzp.p, sig,
                                                               mu, val, (int32_t *)berr.p);
    count_launch();
    const int64_t nk = g.ktop - (g.E - 1);
    map_planes<<<grid_for(2 * (int64_t)g.E * (g.nny - 2 * (int64_t)g.E) * nk, 256), 256>>>(g, 0, sig, mu, val);
    count_launch();
    map_planes<<<grid_for(2 * (int64_t)g.E * g.nnx * nk, 256), 256>>>(g, 1, sig, mu, val);
    count_launch();
    if (g.E > 1) {
        map_bottom<<<grid_for(g.nnx * g.nny * (g.E - 1), 256), 256>>>(g, sig, mu, val);
        count_launch();
    }
    map_air<<<grid_for(g.nnx * g.nny * (g.nnz - g.ktop), 256), 256>>>(g, ieps, sig, mu);
    count_launch();
    map_fixup<<<grid_for(g.nnx * g.nny * 6, 128), 128>>>(g, sig, mu);
    count_launch();
    cudaEventRecord(t1, 0);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventSynchronize(t1);
    float ms = 0.f;
    if (e == cudaSuccess) cudaEventElapsedTime(&ms, t0, t1);
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (e != cudaSuccess) return map_fail(MVF_E_CUDA, std::string("model mapping kernels: ") + cudaGetErrorString(e));
    int32_t herr = 0;
    e = cudaMemcpy(&herr, berr.p, sizeof herr, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(sigma_out, sig, sizeof(double) * 12 * npt, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(mu_out, mu, sizeof(double) * 6 * npt, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return map_fail(MVF_E_CUDA, std::string("model mapping copy-out: ") + cudaGetErrorString(e));
    if (herr) return map_fail(MVF_E_ARG, "a grid node found no model point closer than 1e20 m (non-finite coordinates?)");
    if (seconds) *seconds = 1e-3 * ms;
    return MVF_OK;
}

namespace mvf {
const char *map_last_error() { return g_map_err.c_str(); }
void set_host_error(const char *msg) { g_map_err = msg; }
}  // namespace mvf
