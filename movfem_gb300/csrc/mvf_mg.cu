// mvf_mg.cu -- multilevel preconditioner of the 36- and 54-DOF edge systems.
//
// The one-level vertex-patch Schwarz method stalls on the quadratic and Lagrangian
// systems: nothing in it removes the smooth error components.  This file adds the
// coarse levels.  Level 0 is the 36/54-DOF system with its vertex patches (mvf_patch.cu).
// Level 1 is the lowest-order (12-edge) space on the same cells: it is contained in the
// 36/54-DOF spaces (each 12-edge basis function is an exact combination of at most 4 or
// 8 of the element's own basis functions, p_local), so the prolongation is exact and the
// level-1 operator is the Galerkin product P^T A P, formed element by element inside the
// assembly kernel.  Levels 2, 3, ... merge the cells of the level above in pairs along
// each axis; the 12-edge space of a merged cell is contained in that of its children on
// box cells, and its operator is again the Galerkin product, built from the children's
// element matrices.  Every level smooths with multiplicative vertex-patch Schwarz (the
// patches of one vertex-parity colour share no DOF and no matrix entry, so a colour is
// one launch with a block per patch: residual of the patch rows, local solve, update);
// the coarsest level is one patch holding every DOF, i.e. a direct solve.
//
// The preconditioner works on K + i w Mp, not on the true A = K + i w M.  Mp is the mass
// matrix of a modified conductivity, formed in the element kernel at every Gauss point:
//  * the reference interpolates the nodal sigma with the element's quadratic shape
//    functions (problem.f90:132-149), which undershoot below zero next to a jump (the
//    surface, layer and block boundaries), so M is indefinite on gradients and
//    K + i w M (+ any regularisation) passes near singular on some of them; Mp uses the
//    interpolated tensor shifted to be positive semidefinite (|sigma| when isotropic);
//  * the air carries no conductivity (Re sigma = 0; the reference keeps only real
//    parts, integration.f90:154-238), so gradients of nodal functions supported in the
//    air are in the kernel of A; Mp adds a floor conductivity (default 1e-8 S/m), which
//    makes them regular without changing the earth's operator measurably.
// FGMRES keeps the true A as its operator, so the solution is that of the reference's
// system; Mp only changes how well the preconditioner approximates A^-1.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <numeric>
#include <vector>

#include "mvf_internal.cuh"

namespace mvf {

static constexpr int MG_COARSE = 96;   // a level with at most this many DOFs is solved directly
static constexpr int MG_MAXDIRECT = 400;

// ------------------------------------------------------------------ local maps (host)
static inline double lin1h(int a, double t) { return 0.5 * (1.0 + a * t); }

// 12-edge basis function a as a combination of the mn-node element's basis functions:
// both are L(xi) grad(xi_dir) with the same grad(xi_dir), so the scalar factors are
// matched by least squares on sample points (the fit is exact; coefficients are
// multiples of 1/8).
void p_local(int mn, PLoc &P) {
    OrderTables T12, Tq;
    build_tables(8, 0, T12);
    build_tables(mn, 0, Tq);
    const double s[5] = {-0.93, -0.41, 0.07, 0.52, 0.88};
    std::vector<std::array<double, 3>> pts;
    for (double a : s)
        for (double b : s)
            for (double c : s) pts.push_back({a, b, c});
    memset(&P, 0, sizeof P);
    for (int a = 0; a < 12; ++a) {
        const int d = T12.edge_dir[a];
        std::vector<int> idx;
        for (int i = 0; i < Tq.me; ++i)
            if (Tq.edge_dir[i] == d) idx.push_back(i);
        const int nb = (int)idx.size();
        std::vector<double> G((size_t)nb * nb, 0.0), rhs(nb, 0.0), B(nb);
        for (auto &t : pts) {
            double L, g[3], tl;
            edge_factor(8, T12.edge_node[a], d, t.data(), tl, g);
            for (int q = 0; q < nb; ++q) {
                edge_factor(mn, Tq.edge_node[idx[q]], d, t.data(), L, g);
                B[q] = L;
            }
            for (int q = 0; q < nb; ++q) {
                rhs[q] += B[q] * tl;
                for (int r = 0; r < nb; ++r) G[(size_t)q * nb + r] += B[q] * B[r];
            }
        }
        // Gauss elimination with partial pivoting on the normal equations
        for (int k = 0; k < nb; ++k) {
            int pv = k;
            for (int i = k + 1; i < nb; ++i)
                if (std::fabs(G[(size_t)i * nb + k]) > std::fabs(G[(size_t)pv * nb + k])) pv = i;
            for (int j = 0; j < nb; ++j) std::swap(G[(size_t)k * nb + j], G[(size_t)pv * nb + j]);
            std::swap(rhs[k], rhs[pv]);
            for (int i = k + 1; i < nb; ++i) {
                const double f = G[(size_t)i * nb + k] / G[(size_t)k * nb + k];
                for (int j = k; j < nb; ++j) G[(size_t)i * nb + j] -= f * G[(size_t)k * nb + j];
                rhs[i] -= f * rhs[k];
            }
        }
        std::vector<double> x(nb);
        for (int i = nb - 1; i >= 0; --i) {
            double t = rhs[i];
            for (int j = i + 1; j < nb; ++j) t -= G[(size_t)i * nb + j] * x[j];
            x[i] = t / G[(size_t)i * nb + i];
        }
        for (int q = 0; q < nb; ++q) {
            const double v = std::round(x[q] * 8.0) / 8.0;
            if (v == 0.0) continue;
            P.idx[a][P.cnt[a]] = idx[q];
            P.val[a][P.cnt[a]] = v;
            P.cnt[a]++;
        }
    }
}

// ------------------------------------------------------------------ kernels
// Multiplicative vertex-patch smoothing, one colour: for each patch (one block),
// r = b - A x on the patch rows, then x += A_v^-1 r.  A = K + i w_q (M + tau diag K)
// for right-hand side q; the inverse of right-hand side q is that of its frequency.
__global__ void __launch_bounds__(128) mg_smooth(int64_t p0, int64_t p1, const int64_t *__restrict__ pptr,
                                                 const int32_t *__restrict__ pdof, const int64_t *__restrict__ ioff,
                                                 const double2 *__restrict__ inv, int64_t fstride,
                                                 const int64_t *__restrict__ rowptr, const int32_t *__restrict__ col,
                                                 const double *__restrict__ K, const double *__restrict__ M,
                                                 double tau, const double *__restrict__ wq, int R, int npol, int nfi,
                                                 const double2 *__restrict__ b, double2 *__restrict__ x) {
    extern __shared__ double2 rs[];  // [P][R]
    for (int64_t p = p0 + blockIdx.x; p < p1; p += gridDim.x) {
        const int64_t b0 = pptr[p];
        const int P = (int)(pptr[p + 1] - b0);
        for (int t = threadIdx.x; t < P * R; t += blockDim.x) {
            const int i = t / R, q = t % R;
            const int32_t g = pdof[b0 + i];
            const double w = wq[q];
            double2 acc = b[(int64_t)g * R + q];
            for (int64_t k = rowptr[g]; k < rowptr[g + 1]; ++k) {
                const int32_t j = col[k];
                const double kv = K[k];
                const double mv = M[k] + (j == g ? tau * kv : 0.0);
                const double2 xv = x[(int64_t)j * R + q];
                const double ai = w * mv;
                acc.x -= kv * xv.x - ai * xv.y;
                acc.y -= kv * xv.y + ai * xv.x;
            }
            rs[t] = acc;
        }
        __syncthreads();
        const double2 *A = inv + ioff[p];
        for (int t = threadIdx.x; t < P * R; t += blockDim.x) {
            const int i = t / R, q = t % R;
            const double2 *Ai = A + (int64_t)min(q / npol, nfi - 1) * fstride + (int64_t)i * P;
            double sr = 0.0, si = 0.0;
            for (int j = 0; j < P; ++j) {
                const double2 a = Ai[j];
                const double2 v = rs[j * R + q];
                sr += a.x * v.x - a.y * v.y;
                si += a.x * v.y + a.y * v.x;
            }
            double2 &o = x[(int64_t)pdof[b0 + i] * R + q];
            o.x += sr;
            o.y += si;
        }
        __syncthreads();
    }
}

// The same colour sweep in float-float arithmetic on the FP32 pipe (the mixed mode's
// level 0, where the FP64 version is bound by GB300's FP64 rate): K, Mp, the inverses,
// the right-hand side and the iterate all held as hi + lo FP32 pairs, every row sum and
// every inverse row a compensated dot product (dot2_mac), every update a float-float
// addition -- about twice FP32's precision, with no FP64 instruction in the sweep.
struct ffv {
    float h, l;
};
__device__ __forceinline__ ffv ff_norm(float s, float e) {
    const float h = s + e;
    return {h, e - (h - s)};
}
__device__ __forceinline__ ffv ff_add(ffv a, ffv b) {
    const float s = a.h + b.h;
    const float bb = s - a.h;
    const float e = (a.h - (s - bb)) + (b.h - bb) + a.l + b.l;
    return ff_norm(s, e);
}
__device__ __forceinline__ ffv ff_mul(ffv a, ffv b) {
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, fmaf(a.l, b.h, e));
    return ff_norm(p, e);
}
__device__ __forceinline__ void split_d(double v, float &h, float &l) {
    h = __double2float_rn(v);
    l = __double2float_rn(v - (double)h);
}

// row g of b - (K + i w Mp) x for right-hand side q, float-float: (re, im)
__device__ __forceinline__ void ff_row(int32_t g, int q, int R, const int64_t *__restrict__ rowptr,
                                       const int32_t *__restrict__ col, const float2 *__restrict__ K,
                                       const float2 *__restrict__ M, ffv w, float4 bv, const float4 *__restrict__ x,
                                       ffv &rr, ffv &ri) {
    float krh = 0.f, krl = 0.f, kih = 0.f, kil = 0.f, mrh = 0.f, mrl = 0.f, mih = 0.f, mil = 0.f;
    for (int64_t k = rowptr[g]; k < rowptr[g + 1]; ++k) {
        const float2 kv = K[k], mv = M[k];
        const float4 xv = x[(int64_t)col[k] * R + q];  // (re_hi, im_hi, re_lo, im_lo)
        dot2_mac(krh, krl, kv.x, kv.y, xv.x, xv.z);
        dot2_mac(kih, kil, kv.x, kv.y, xv.y, xv.w);
        dot2_mac(mrh, mrl, mv.x, mv.y, xv.x, xv.z);
        dot2_mac(mih, mil, mv.x, mv.y, xv.y, xv.w);
    }
    const ffv kr = ff_norm(krh, krl), ki = ff_norm(kih, kil), mr = ff_norm(mrh, mrl), mi = ff_norm(mih, mil);
    const ffv wmi = ff_mul(w, mi), wmr = ff_mul(w, mr);
    // b - (Kx_re - w Mx_im), b - (Kx_im + w Mx_re)
    rr = ff_add(ff_add({bv.x, bv.z}, {-kr.h, -kr.l}), wmi);
    ri = ff_add(ff_add({bv.y, bv.w}, {-ki.h, -ki.l}), {-wmr.h, -wmr.l});
}

__global__ void __launch_bounds__(128) mg_smooth_ff(int64_t p0, int64_t p1, const int64_t *__restrict__ pptr,
                                                    const int32_t *__restrict__ pdof, const int64_t *__restrict__ ioff,
                                                    const float4 *__restrict__ inv, int64_t fstride,
                                                    const int64_t *__restrict__ rowptr, const int32_t *__restrict__ col,
                                                    const float2 *__restrict__ K, const float2 *__restrict__ M,
                                                    const float2 *__restrict__ wq, int R, int npol, int nfi,
                                                    const float4 *__restrict__ b, float4 *__restrict__ x) {
    extern __shared__ float4 rsf[];  // [P][R]: (re_hi, im_hi, re_lo, im_lo)
    for (int64_t p = p0 + blockIdx.x; p < p1; p += gridDim.x) {
        const int64_t b0 = pptr[p];
        const int P = (int)(pptr[p + 1] - b0);
        for (int t = threadIdx.x; t < P * R; t += blockDim.x) {
            const int i = t / R, q = t % R;
            const int32_t g = pdof[b0 + i];
            const float2 w2 = wq[q];
            ffv rr, ri;
            ff_row(g, q, R, rowptr, col, K, M, {w2.x, w2.y}, b[(int64_t)g * R + q], x, rr, ri);
            rsf[t] = make_float4(rr.h, ri.h, rr.l, ri.l);
        }
        __syncthreads();
        const float4 *A = inv + ioff[p];
        for (int t = threadIdx.x; t < P * R; t += blockDim.x) {
            const int i = t / R, q = t % R;
            const float4 *Ai = A + (int64_t)min(q / npol, nfi - 1) * fstride + (int64_t)i * P;
            float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
            for (int j = 0; j < P; ++j) {
                const float4 a = Ai[j];
                const float4 v = rsf[j * R + q];
                dot2_mac(rh, rl, a.x, a.z, v.x, v.z);
                dot2_mac(rh, rl, -a.y, -a.w, v.y, v.w);
                dot2_mac(ih, il, a.x, a.z, v.y, v.w);
                dot2_mac(ih, il, a.y, a.w, v.x, v.z);
            }
            float4 &o = x[(int64_t)pdof[b0 + i] * R + q];
            const ffv zr = ff_add({o.x, o.z}, ff_norm(rh, rl)), zi = ff_add({o.y, o.w}, ff_norm(ih, il));
            o = make_float4(zr.h, zi.h, zr.l, zi.l);
        }
        __syncthreads();
    }
}

// t = b - A x over all rows (level 0 of the mixed mode), FP64 out
__global__ void mg_resid_ff(int32_t n, const int64_t *__restrict__ rowptr, const int32_t *__restrict__ col,
                            const float2 *__restrict__ K, const float2 *__restrict__ M, const float2 *__restrict__ wq,
                            int R, const float4 *__restrict__ b, const float4 *__restrict__ x,
                            double2 *__restrict__ t) {
    const int64_t nt = (int64_t)n * R;
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < nt; u += (int64_t)gridDim.x * blockDim.x) {
        const int32_t g = (int32_t)(u / R);
        const int q = (int)(u % R);
        const float2 w2 = wq[q];
        ffv rr, ri;
        ff_row(g, q, R, rowptr, col, K, M, {w2.x, w2.y}, b[u], x, rr, ri);
        t[u] = make_double2((double)rr.h + (double)rr.l, (double)ri.h + (double)ri.l);
    }
}

// float-float copies of complex FP64 vectors and back
__global__ void mg_to_ff(int64_t n, const double2 *__restrict__ a, float4 *__restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 v = a[i];
        float rh, rl, ih, il;
        split_d(v.x, rh, rl);
        split_d(v.y, ih, il);
        out[i] = make_float4(rh, ih, rl, il);
    }
}
__global__ void mg_from_ff(int64_t n, const float4 *__restrict__ a, double2 *__restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 v = a[i];
        out[i] = make_double2((double)v.x + (double)v.z, (double)v.y + (double)v.w);
    }
}

// x (float-float) += S y for a real sparse S (the prolongation into level 0)
__global__ void mg_prolong_ff(int32_t n, const int64_t *__restrict__ rowptr, const int32_t *__restrict__ col,
                              const double *__restrict__ val, int R, const double2 *__restrict__ y,
                              float4 *__restrict__ x) {
    const int64_t nt = (int64_t)n * R;
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < nt; u += (int64_t)gridDim.x * blockDim.x) {
        const int32_t g = (int32_t)(u / R);
        const int q = (int)(u % R);
        double sr = 0.0, si = 0.0;
        for (int64_t k = rowptr[g]; k < rowptr[g + 1]; ++k) {
            const double2 v = y[(int64_t)col[k] * R + q];
            sr += val[k] * v.x;
            si += val[k] * v.y;
        }
        const float4 o = x[u];
        float h, l;
        split_d(sr, h, l);
        const ffv zr = ff_add({o.x, o.z}, {h, l});
        split_d(si, h, l);
        const ffv zi = ff_add({o.y, o.w}, {h, l});
        x[u] = make_float4(zr.h, zi.h, zr.l, zi.l);
    }
}

// FP64 values as hi + lo FP32 halves; inverses in place (double2 -> float4, same bytes)
__global__ void mg_split(int64_t n, const double *__restrict__ a, float2 *__restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float h, l;
        split_d(a[i], h, l);
        out[i] = make_float2(h, l);
    }
}
__global__ void mg_split_inv(int64_t n, double2 *__restrict__ a) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 v = a[i];
        float rh, rl, ih, il;
        split_d(v.x, rh, rl);
        split_d(v.y, ih, il);
        reinterpret_cast<float4 *>(a)[i] = make_float4(rh, ih, rl, il);
    }
}

// t = b - A x over all rows of a level
__global__ void mg_resid(int32_t n, const int64_t *__restrict__ rowptr, const int32_t *__restrict__ col,
                         const double *__restrict__ K, const double *__restrict__ M, double tau,
                         const double *__restrict__ wq, int R, const double2 *__restrict__ b,
                         const double2 *__restrict__ x, double2 *__restrict__ t) {
    const int64_t nt = (int64_t)n * R;
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < nt; u += (int64_t)gridDim.x * blockDim.x) {
        const int32_t g = (int32_t)(u / R);
        const int q = (int)(u % R);
        const double w = wq[q];
        double2 acc = b[u];
        for (int64_t k = rowptr[g]; k < rowptr[g + 1]; ++k) {
            const int32_t j = col[k];
            const double kv = K[k];
            const double mv = M[k] + (j == g ? tau * kv : 0.0);
            const double2 xv = x[(int64_t)j * R + q];
            const double ai = w * mv;
            acc.x -= kv * xv.x - ai * xv.y;
            acc.y -= kv * xv.y + ai * xv.x;
        }
        t[u] = acc;
    }
}

// y (+)= S x for a real sparse S (prolongation or its transpose), R right-hand sides
__global__ void mg_spmv(int32_t n, const int64_t *__restrict__ rowptr, const int32_t *__restrict__ col,
                        const double *__restrict__ val, int R, const double2 *__restrict__ x, double2 *__restrict__ y,
                        int accumulate) {
    const int64_t nt = (int64_t)n * R;
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < nt; u += (int64_t)gridDim.x * blockDim.x) {
        const int32_t g = (int32_t)(u / R);
        const int q = (int)(u % R);
        double2 acc = accumulate ? y[u] : make_double2(0.0, 0.0);
        for (int64_t k = rowptr[g]; k < rowptr[g + 1]; ++k) {
            const double v = val[k];
            const double2 xv = x[(int64_t)col[k] * R + q];
            acc.x += v * xv.x;
            acc.y += v * xv.y;
        }
        y[u] = acc;
    }
}

// Element matrices of a merged cell: K_E = sum_c Q_c^T K_c Q_c over its children c
// (likewise M).  One block of 144 threads per merged cell.
__global__ void __launch_bounds__(144) mg_galerkin(int64_t ne, const int32_t *__restrict__ child,
                                                   const double *__restrict__ Q, const double *__restrict__ Kf,
                                                   const double *__restrict__ Mf, double *__restrict__ Kc,
                                                   double *__restrict__ Mc) {
    __shared__ double q[144], kf[144], mf[144], tk[144], tm[144];
    const int t = threadIdx.x, a = t / 12, bb = t % 12;
    for (int64_t E = blockIdx.x; E < ne; E += gridDim.x) {
        double ak = 0.0, am = 0.0;
        for (int c = 0; c < 8; ++c) {
            const int32_t ch = child[E * 8 + c];
            if (ch < 0) continue;  // uniform across the block
            q[t] = Q[(E * 8 + c) * 144 + t];
            kf[t] = Kf[(int64_t)ch * 144 + t];
            mf[t] = Mf[(int64_t)ch * 144 + t];
            __syncthreads();
            // T = K_c Q_c: row a (fine), column bb (merged)
            double sk = 0.0, sm = 0.0;
            for (int j = 0; j < 12; ++j) {
                sk += kf[a * 12 + j] * q[j * 12 + bb];
                sm += mf[a * 12 + j] * q[j * 12 + bb];
            }
            tk[t] = sk;
            tm[t] = sm;
            __syncthreads();
            // Q_c^T T: row a (merged), column bb (merged)
            for (int i = 0; i < 12; ++i) {
                ak += q[i * 12 + a] * tk[i * 12 + bb];
                am += q[i * 12 + a] * tm[i * 12 + bb];
            }
            __syncthreads();
        }
        Kc[E * 144 + t] = ak;
        Mc[E * 144 + t] = am;
    }
}

// Scatter the 12x12 element matrices of one element colour into a level's CSR (the
// elements of a colour share no DOF, so no two threads add into the same entry).
__global__ void mg_scatter(const int32_t *__restrict__ elist, int64_t cnt, const int32_t *__restrict__ gne,
                           const int64_t *__restrict__ rowptr, const int32_t *__restrict__ col,
                           const double *__restrict__ Ke, const double *__restrict__ Me, double *__restrict__ K,
                           double *__restrict__ M, int *__restrict__ err) {
    const int64_t nt = cnt * 144;
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < nt; u += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = elist[u / 144];
        const int t = (int)(u % 144), a = t / 12, bb = t % 12;
        const int32_t ga = gne[e * 12 + a], gb = gne[e * 12 + bb];
        if (ga <= 0 || gb <= 0) continue;
        int64_t lo = rowptr[ga - 1], hi = rowptr[ga] - 1;
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if (col[mid] < gb - 1) lo = mid + 1;
            else hi = mid;
        }
        if (col[lo] != gb - 1) {
            atomicMax(err, 1);
            continue;
        }
        K[lo] += Ke[e * 144 + t];
        M[lo] += Me[e * 144 + t];
    }
}

// ------------------------------------------------------------------ hierarchy (host)
template <class T>
static int upload_vec(Ctx *c, T **dst, const std::vector<T> &src) {
    MVF_CUDA(c, cudaMalloc((void **)dst, std::max<size_t>(src.size(), 1) * sizeof(T)));
    if (!src.empty()) MVF_CUDA(c, cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
    return 0;
}

// CSR of the triplets (row, col, val), duplicates (the same entry seen from several
// elements) collapsed to the first; and the transpose.
struct Trip {
    int32_t r, c;
    double v;
};
static void csr_of(std::vector<Trip> &t, int32_t nrow, int32_t ncol, std::vector<int64_t> &rp, std::vector<int32_t> &ci,
                   std::vector<double> &va, std::vector<int64_t> &trp, std::vector<int32_t> &tci,
                   std::vector<double> &tva) {
    std::stable_sort(t.begin(), t.end(), [](const Trip &a, const Trip &b) { return a.r != b.r ? a.r < b.r : a.c < b.c; });
    t.erase(std::unique(t.begin(), t.end(), [](const Trip &a, const Trip &b) { return a.r == b.r && a.c == b.c; }),
            t.end());
    rp.assign(nrow + 1, 0);
    ci.resize(t.size());
    va.resize(t.size());
    for (size_t k = 0; k < t.size(); ++k) {
        rp[t[k].r + 1]++;
        ci[k] = t[k].c;
        va[k] = t[k].v;
    }
    for (int32_t r = 0; r < nrow; ++r) rp[r + 1] += rp[r];
    trp.assign(ncol + 1, 0);
    for (const Trip &x : t) trp[x.c + 1]++;
    for (int32_t r = 0; r < ncol; ++r) trp[r + 1] += trp[r];
    tci.resize(t.size());
    tva.resize(t.size());
    std::vector<int64_t> fill(trp.begin(), trp.end() - 1);
    for (const Trip &x : t) {
        tci[fill[x.c]] = x.r;
        tva[fill[x.c]++] = x.v;
    }
}

static std::vector<int> merge_axis(int n) {
    std::vector<int> v;
    for (int I = 0; I <= (n + 1) / 2; ++I) v.push_back(std::min(2 * I, n));
    return v;
}

// upload a level's pattern, numbering, element colours and patches
static int finish_level(Ctx *c, MgLevel &L, const OrderTables &T12, bool coarsest) {
    std::vector<int64_t> rp;
    std::vector<int32_t> ci;
    pattern_from_gne(L.gne, 12, L.ne, L.n, rp, ci);
    L.nnz = rp[L.n];
    int rc;
    if ((rc = upload_vec(c, &L.rowptr, rp))) return rc;
    if ((rc = upload_vec(c, &L.col, ci))) return rc;
    if ((rc = upload_vec(c, &L.gne_d, L.gne))) return rc;
    std::vector<int32_t> el;
    L.ecolor_off.assign(9, 0);
    for (int col8 = 0; col8 < 8; ++col8) {
        L.ecolor_off[col8] = (int64_t)el.size();
        for (int ie = col8 & 1; ie < L.nx; ie += 2)
            for (int je = (col8 >> 1) & 1; je < L.ny; je += 2)
                for (int ke = (col8 >> 2) & 1; ke < L.nz; ke += 2)
                    el.push_back((int32_t)(((int64_t)ie * L.ny + je) * L.nz + ke));
    }
    L.ecolor_off[8] = (int64_t)el.size();
    if ((rc = upload_vec(c, &L.elist, el))) return rc;
    PatchHost ph;
    if (coarsest) {
        ph.ptr = {0, (int64_t)L.n};
        ph.ioff = {0, (int64_t)L.n * L.n};
        ph.dof.resize(L.n);
        std::iota(ph.dof.begin(), ph.dof.end(), 0);
        ph.color_off.assign(9, 1);
        ph.color_off[0] = 0;
        ph.pmax = L.n;
    } else {
        vertex_patches(L.nx, L.ny, L.nz, 12, L.gne, L.n, ph);
    }
    (void)T12;
    L.np = (int64_t)ph.ptr.size() - 1;
    L.pent = ph.ioff[L.np];
    L.pmax = ph.pmax;
    L.pcolor_off = ph.color_off;
    if ((rc = upload_vec(c, &L.pptr, ph.ptr))) return rc;
    if ((rc = upload_vec(c, &L.pioff, ph.ioff))) return rc;
    if ((rc = upload_vec(c, &L.pdof, ph.dof))) return rc;
    return 0;
}

int mg_setup(Ctx *c) {
    mg_release(c);
    OrderTables T12;
    build_tables(8, 0, T12);
    const bool dir = c->mesh.dirichlet != 0;
    const int o = c->T.nord - 1;
    // level-1 vertex coordinates: the corner nodes of the context's grid
    const int nvx0 = c->mesh.nx + 1, nvy0 = c->mesh.ny + 1, nvz0 = c->mesh.nz + 1;
    std::vector<double> vx(nvx0), vy(nvy0), vz((size_t)nvx0 * nvy0 * nvz0);
    for (int i = 0; i < nvx0; ++i) vx[i] = c->xp_h[(size_t)o * i];
    for (int j = 0; j < nvy0; ++j) vy[j] = c->yp_h[(size_t)o * j];
    for (int i = 0; i < nvx0; ++i)
        for (int j = 0; j < nvy0; ++j)
            for (int k = 0; k < nvz0; ++k)
                vz[((size_t)i * nvy0 + j) * nvz0 + k] =
                    c->zp_h[(((int64_t)o * i) * c->nny + (int64_t)o * j) * c->nnz_nodes + (int64_t)o * k];
    // ---- level 1: the 12-edge space on the context's cells
    {
        MgLevel L;
        L.nx = c->mesh.nx; L.ny = c->mesh.ny; L.nz = c->mesh.nz;
        L.ne = (int64_t)L.nx * L.ny * L.nz;
        L.n = number_grid(T12, L.nx, L.ny, L.nz, dir, L.gne);
        if (L.n <= 0) return fail(c, MVF_E_UNSUPPORTED, "multilevel preconditioner: no free DOF on the 12-edge level");
        // P_1: level 1 -> the context's DOFs, from p_local
        PLoc pl;
        p_local(c->T.mn, pl);
        std::vector<Trip> tr;
        const int me = c->T.me;
        tr.reserve((size_t)L.ne * 48);
        for (int64_t e = 0; e < L.ne; ++e)
            for (int a = 0; a < 12; ++a) {
                const int32_t g1 = L.gne[(size_t)e * 12 + a];
                if (g1 <= 0) continue;
                for (int k = 0; k < pl.cnt[a]; ++k) {
                    const int32_t g0 = c->gne_h[(size_t)e * me + pl.idx[a][k]];
                    if (g0 > 0) tr.push_back({g0 - 1, g1 - 1, pl.val[a][k]});
                }
            }
        std::vector<int64_t> rp, trp;
        std::vector<int32_t> ci, tci;
        std::vector<double> va, tva;
        csr_of(tr, c->nne, L.n, rp, ci, va, trp, tci, tva);
        int rc;
        if ((rc = upload_vec(c, &L.prow, rp)) || (rc = upload_vec(c, &L.pcol, ci)) || (rc = upload_vec(c, &L.pval, va)) ||
            (rc = upload_vec(c, &L.ptrow, trp)) || (rc = upload_vec(c, &L.ptcol, tci)) ||
            (rc = upload_vec(c, &L.ptval, tva)))
            return rc;
        c->mg.push_back(std::move(L));
    }
    // ---- merged levels
    while (true) {
        MgLevel &F = c->mg.back();
        const int fnvx = F.nx + 1, fnvy = F.ny + 1, fnvz = F.nz + 1;
        bool coarsest = F.n <= MG_COARSE || (F.nx <= 1 && F.ny <= 1 && F.nz <= 1);
        MgLevel L;
        if (!coarsest) {
            L.ix = merge_axis(F.nx);
            L.iy = merge_axis(F.ny);
            L.iz = merge_axis(F.nz);
            L.nx = (int)L.ix.size() - 1; L.ny = (int)L.iy.size() - 1; L.nz = (int)L.iz.size() - 1;
            L.ne = (int64_t)L.nx * L.ny * L.nz;
            L.n = number_grid(T12, L.nx, L.ny, L.nz, dir, L.gne);
            if (L.n <= 0) coarsest = true;
        }
        if (coarsest) {
            if (F.n > MG_MAXDIRECT)
                return fail(c, MVF_E_UNSUPPORTED, "multilevel preconditioner: the coarsest level is too large");
            return finish_level(c, F, T12, true);
        }
        int rc = finish_level(c, F, T12, false);
        if (rc) return rc;
        // prolongation L -> F and the local maps of the Galerkin products
        auto Z = [&](int i, int j, int k) { return vz[((size_t)i * fnvy + j) * fnvz + k]; };
        std::vector<int32_t> child((size_t)L.ne * 8, -1);
        std::vector<double> Q((size_t)L.ne * 8 * 144, 0.0);
        std::vector<Trip> tr;
        tr.reserve((size_t)F.ne * 24);
        for (int i = 0; i < F.nx; ++i)
            for (int j = 0; j < F.ny; ++j)
                for (int k = 0; k < F.nz; ++k) {
                    const int64_t ef = ((int64_t)i * F.ny + j) * F.nz + k;
                    const int I = i / 2, J = j / 2, Kk = k / 2;
                    const int64_t E = ((int64_t)I * L.ny + J) * L.nz + Kk;
                    const int cslot = (i & 1) * 4 + (j & 1) * 2 + (k & 1);
                    child[E * 8 + cslot] = (int32_t)ef;
                    const int fi[3] = {i, j, k};
                    const int ci3[3] = {I, J, Kk};
                    const std::vector<int> *cm[3] = {&L.ix, &L.iy, &L.iz};
                    for (int jf = 0; jf < 12; ++jf) {
                        const int nd = T12.edge_node[jf], d = T12.edge_dir[jf];
                        // the fine edge's two end vertices (fine vertex indices)
                        int v1[3], v2[3];
                        for (int a = 0; a < 3; ++a) {
                            const int off = (node_ref(nd, a) + 1) / 2;
                            v1[a] = fi[a] + (a == d ? 0 : off);
                            v2[a] = fi[a] + (a == d ? 1 : off);
                        }
                        auto coord = [&](const int *v, int a) {
                            return a == 0 ? vx[v[0]] : a == 1 ? vy[v[1]] : Z(v[0], v[1], v[2]);
                        };
                        // merged-cell reference coordinates of the fine edge across its direction
                        double cref[3] = {0, 0, 0};
                        for (int a = 0; a < 3; ++a) {
                            if (a == d) continue;
                            const double X = 0.5 * (coord(v1, a) + coord(v2, a));
                            int w1[3] = {v1[0], v1[1], v1[2]}, w2[3] = {v1[0], v1[1], v1[2]};
                            int u1[3] = {v2[0], v2[1], v2[2]}, u2[3] = {v2[0], v2[1], v2[2]};
                            w1[a] = u1[a] = (*cm[a])[ci3[a]];
                            w2[a] = u2[a] = (*cm[a])[ci3[a] + 1];
                            const double X0 = 0.5 * (coord(w1, a) + coord(u1, a));
                            const double X1 = 0.5 * (coord(w2, a) + coord(u2, a));
                            cref[a] = -1.0 + 2.0 * (X - X0) / (X1 - X0);
                        }
                        // length ratio along the direction
                        int w1[3] = {v1[0], v1[1], v1[2]}, w2[3] = {v1[0], v1[1], v1[2]};
                        w1[d] = (*cm[d])[ci3[d]];
                        w2[d] = (*cm[d])[ci3[d] + 1];
                        const double ratio = (coord(v2, d) - coord(v1, d)) / (coord(w2, d) - coord(w1, d));
                        const int32_t gf = F.gne[(size_t)ef * 12 + jf];
                        for (int jc = 0; jc < 12; ++jc) {
                            if (T12.edge_dir[jc] != d) continue;
                            double v = ratio;
                            for (int a = 0; a < 3; ++a)
                                if (a != d) v *= lin1h(node_ref(T12.edge_node[jc], a), cref[a]);
                            if (std::fabs(v) < 1e-14) continue;
                            Q[((size_t)E * 8 + cslot) * 144 + jf * 12 + jc] = v;
                            const int32_t gc = L.gne[(size_t)E * 12 + jc];
                            if (gf > 0 && gc > 0) tr.push_back({gf - 1, gc - 1, v});
                        }
                    }
                }
        std::vector<int64_t> rp, trp;
        std::vector<int32_t> ci, tci;
        std::vector<double> va, tva;
        csr_of(tr, F.n, L.n, rp, ci, va, trp, tci, tva);
        if ((rc = upload_vec(c, &L.prow, rp)) || (rc = upload_vec(c, &L.pcol, ci)) || (rc = upload_vec(c, &L.pval, va)) ||
            (rc = upload_vec(c, &L.ptrow, trp)) || (rc = upload_vec(c, &L.ptcol, tci)) ||
            (rc = upload_vec(c, &L.ptval, tva)) || (rc = upload_vec(c, &L.child, child)) ||
            (rc = upload_vec(c, &L.Q, Q)))
            return rc;
        // the merged level's vertex z: the finer level's at the kept indices
        std::vector<double> nvxv(L.ix.size()), nvyv(L.iy.size()), nvzv(L.ix.size() * L.iy.size() * L.iz.size());
        for (size_t a = 0; a < L.ix.size(); ++a) nvxv[a] = vx[L.ix[a]];
        for (size_t a = 0; a < L.iy.size(); ++a) nvyv[a] = vy[L.iy[a]];
        for (size_t a = 0; a < L.ix.size(); ++a)
            for (size_t b = 0; b < L.iy.size(); ++b)
                for (size_t q = 0; q < L.iz.size(); ++q)
                    nvzv[(a * L.iy.size() + b) * L.iz.size() + q] = Z(L.ix[a], L.iy[b], L.iz[q]);
        vx.swap(nvxv);
        vy.swap(nvyv);
        vz.swap(nvzv);
        c->mg.push_back(std::move(L));
    }
}

void mg_release(Ctx *c) {
    for (MgLevel &L : c->mg) {
        void *p[] = {L.rowptr, L.col, L.gne_d, L.prow, L.ptrow, L.pcol, L.ptcol, L.pval, L.ptval, L.child, L.Q, L.elist,
                     L.pptr, L.pioff, L.pdof};
        for (void *q : p)
            if (q) cudaFree(q);
    }
    c->mg.clear();
}

// ------------------------------------------------------------------ numeric state
struct MgWork {
    int R = 0, npol = 1, nf = 1;
    const MatrixSet *S = nullptr;
    std::vector<double *> K, M, Ke, Me;  // per level (index 0: unused)
    std::vector<double2 *> inv;          // per level, [nf][patch entries]
    std::vector<double2 *> b, x, t;      // per level, [n][R] (level 0: b, x are the caller's)
    double *wq = nullptr;                // [R] angular frequency of each right-hand side
    bool ff = false;                     // level 0 in float-float (mixed mode)
    float2 *Kff = nullptr, *Mff = nullptr;  // level-0 K and Mp as FP32 halves
    float2 *wff = nullptr;                  // [R] angular frequencies as FP32 halves
    float4 *bff = nullptr, *xff = nullptr;  // level-0 right-hand side and iterate, [n][R]
    SurfJob *sj = nullptr;                  // surface gradient correction after each cycle
};

// patch-inverse workspace rows of one level: blocks x pmax x 2 pmax complex
static int64_t ws_need(int64_t np, int pmax) { return std::min<int64_t>(np, 152 * 8) * pmax * pmax * 2; }

static unsigned grid_n(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 32)); }

void mg_free(Ctx *c, MgWork *W) {
    if (!W) return;
    (void)c;
    std::vector<void *> p;
    for (size_t l = 0; l < W->K.size(); ++l) {
        p.push_back(W->K[l]);
        p.push_back(W->M[l]);
        if (l >= 2) {
            p.push_back(W->Ke[l]);
            p.push_back(W->Me[l]);
        }
        p.push_back(W->inv[l]);
        if (l >= 1) {
            p.push_back(W->b[l]);
            p.push_back(W->x[l]);
        }
        p.push_back(W->t[l]);
    }
    p.push_back(W->wq);
    p.push_back(W->Kff);
    p.push_back(W->Mff);
    p.push_back(W->wff);
    p.push_back(W->bff);
    p.push_back(W->xff);
    for (void *q : p)
        if (q) cudaFree(q);
    surf_free(W->sj);
    W->sj = nullptr;
    delete W;
}

int mg_numeric(Ctx *c, const MatrixSet &S, const double *w, int nf, int R, int npol, MgWork **out) {
    *out = nullptr;
    if (c->mg.empty()) return fail(c, MVF_E_STATE, "multilevel preconditioner not set up");
    if (!S.K1e || !S.Mp64) return fail(c, MVF_E_STATE, "assemble after selecting the multilevel preconditioner");
    MgWork *W = new MgWork();
    W->R = R;
    W->npol = npol;
    W->nf = nf;
    W->S = &S;
    const int nl = (int)c->mg.size() + 1;
    W->K.assign(nl, nullptr); W->M.assign(nl, nullptr); W->Ke.assign(nl, nullptr); W->Me.assign(nl, nullptr);
    W->inv.assign(nl, nullptr); W->b.assign(nl, nullptr); W->x.assign(nl, nullptr); W->t.assign(nl, nullptr);
    int *err = nullptr;
    double2 *ws = nullptr;
    auto bail = [&](int rc) {
        if (err) cudaFree(err);
        if (ws) cudaFree(ws);
        mg_free(c, W);
        return rc;
    };
#define MG_CUDA(call)                                              \
    do {                                                           \
        cudaError_t _e = (call);                                   \
        if (_e != cudaSuccess) return bail(cuda_fail(c, _e, #call)); \
    } while (0)
    MG_CUDA(cudaMalloc((void **)&err, sizeof(int)));
    MG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), c->stream));
    MG_CUDA(cudaMalloc((void **)&W->t[0], (size_t)c->nne * R * sizeof(double2)));
    // operators of levels 1.. : Galerkin element matrices scattered into each pattern
    for (int l = 1; l < nl; ++l) {
        const MgLevel &L = c->mg[l - 1];
        MG_CUDA(cudaMalloc((void **)&W->K[l], std::max<int64_t>(L.nnz, 1) * sizeof(double)));
        MG_CUDA(cudaMalloc((void **)&W->M[l], std::max<int64_t>(L.nnz, 1) * sizeof(double)));
        MG_CUDA(cudaMemsetAsync(W->K[l], 0, L.nnz * sizeof(double), c->stream));
        MG_CUDA(cudaMemsetAsync(W->M[l], 0, L.nnz * sizeof(double), c->stream));
        const double *Ke = S.K1e, *Me = S.M1e;
        if (l >= 2) {
            MG_CUDA(cudaMalloc((void **)&W->Ke[l], (size_t)L.ne * 144 * sizeof(double)));
            MG_CUDA(cudaMalloc((void **)&W->Me[l], (size_t)L.ne * 144 * sizeof(double)));
            const double *Kf = l == 2 ? S.K1e : W->Ke[l - 1], *Mf = l == 2 ? S.M1e : W->Me[l - 1];
            count_launch();
            mg_galerkin<<<(unsigned)std::min<int64_t>(L.ne, 152 * 16), 144, 0, c->stream>>>(L.ne, L.child, L.Q, Kf, Mf,
                                                                                            W->Ke[l], W->Me[l]);
            Ke = W->Ke[l];
            Me = W->Me[l];
        }
        for (int col8 = 0; col8 < 8; ++col8) {
            const int64_t a = L.ecolor_off[col8], cnt = L.ecolor_off[col8 + 1] - a;
            if (cnt <= 0) continue;
            count_launch();
            mg_scatter<<<grid_n(cnt * 144), 256, 0, c->stream>>>(L.elist + a, cnt, L.gne_d, L.rowptr, L.col, Ke, Me,
                                                                 W->K[l], W->M[l], err);
        }
        MG_CUDA(cudaGetLastError());
        MG_CUDA(cudaMalloc((void **)&W->b[l], (size_t)L.n * R * sizeof(double2)));
        MG_CUDA(cudaMalloc((void **)&W->x[l], (size_t)L.n * R * sizeof(double2)));
        MG_CUDA(cudaMalloc((void **)&W->t[l], (size_t)L.n * R * sizeof(double2)));
    }
    // patch inverses of every level, per frequency
    int64_t wsn = ws_need(c->npatch, c->patch_max);
    for (const MgLevel &L : c->mg) wsn = std::max(wsn, ws_need(L.np, L.pmax));
    const int grid = 152 * 8;
    MG_CUDA(cudaMalloc((void **)&ws, (size_t)wsn * sizeof(double2)));
    MG_CUDA(cudaFuncSetAttribute(mg_smooth, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024));
    for (int l = 0; l < nl; ++l) {
        const int64_t ent = l == 0 ? c->patch_entries : c->mg[l - 1].pent;
        MG_CUDA(cudaMalloc((void **)&W->inv[l], std::max<int64_t>(ent * nf, 1) * sizeof(double2)));
        for (int f = 0; f < nf; ++f) {
            if (l == 0)
                launch_patch_invert(c->stream, (int)std::min<int64_t>(c->npatch, grid), c->npatch, c->d.patch_ptr,
                                    c->d.patch_dof, c->d.patch_ioff, c->d.rowptr, c->d.col, S.K64, S.Mp64, w[f],
                                    0.0, c->patch_max, ws, W->inv[l] + (int64_t)f * ent, err);
            else {
                const MgLevel &L = c->mg[l - 1];
                launch_patch_invert(c->stream, (int)std::min<int64_t>(L.np, grid), L.np, L.pptr, L.pdof, L.pioff,
                                    L.rowptr, L.col, W->K[l], W->M[l], w[f], 0.0, L.pmax, ws,
                                    W->inv[l] + (int64_t)f * ent, err);
            }
        }
    }
    MG_CUDA(cudaGetLastError());
    // the mixed mode sweeps level 0 in float-float: K, Mp and the inverses split
    W->ff = c->solve_mode == 0;
    if (W->ff) {
        MG_CUDA(cudaMalloc((void **)&W->Kff, c->nnz * sizeof(float2)));
        MG_CUDA(cudaMalloc((void **)&W->Mff, c->nnz * sizeof(float2)));
        count_launch();
        mg_split<<<grid_n(c->nnz), 256, 0, c->stream>>>(c->nnz, S.K64, W->Kff);
        count_launch();
        mg_split<<<grid_n(c->nnz), 256, 0, c->stream>>>(c->nnz, S.Mp64, W->Mff);
        count_launch();
        mg_split_inv<<<grid_n(c->patch_entries * nf), 256, 0, c->stream>>>(c->patch_entries * nf, W->inv[0]);
        MG_CUDA(cudaGetLastError());
        MG_CUDA(cudaFuncSetAttribute(mg_smooth_ff, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024));
    }
    // angular frequency per right-hand side, as the inverses were formed
    std::vector<double> wq(R);
    for (int q = 0; q < R; ++q) wq[q] = w[std::min(q / npol, nf - 1)];
    MG_CUDA(cudaMalloc((void **)&W->wq, R * sizeof(double)));
    MG_CUDA(cudaMemcpyAsync(W->wq, wq.data(), R * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    if (W->ff) {
        std::vector<float2> wf(R);
        for (int q = 0; q < R; ++q) {
            const float h = (float)wq[q];
            wf[q] = make_float2(h, (float)(wq[q] - (double)h));
        }
        MG_CUDA(cudaMalloc((void **)&W->wff, R * sizeof(float2)));
        MG_CUDA(cudaMemcpyAsync(W->wff, wf.data(), R * sizeof(float2), cudaMemcpyHostToDevice, c->stream));
        MG_CUDA(cudaMalloc((void **)&W->bff, (size_t)c->nne * R * sizeof(float4)));
        MG_CUDA(cudaMalloc((void **)&W->xff, (size_t)c->nne * R * sizeof(float4)));
    }
    int herr = 0;
    MG_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MG_CUDA(cudaStreamSynchronize(c->stream));
#undef MG_CUDA
    cudaFree(err);
    err = nullptr;
    cudaFree(ws);
    ws = nullptr;
    if (herr) {
        mg_free(c, W);
        return fail(c, MVF_E_SINGULAR, "multilevel preconditioner: zero pivot or missing pattern entry");
    }
    if (c->surf_on) {
        if (int rc = surf_numeric(c, S, wq.data(), R, &W->sj)) {
            mg_free(c, W);
            return rc;
        }
    }
    *out = W;
    return 0;
}

// One V-cycle on level l: x_l ~ A_l^-1 b_l (x_l starts at zero).
static void vcycle(Ctx *c, MgWork *W, int l) {
    const int R = W->R;
    const int nl = (int)W->K.size();
    const bool fine = l == 0;
    const int32_t n = fine ? c->nne : c->mg[l - 1].n;
    const int64_t *rowptr = fine ? c->d.rowptr : c->mg[l - 1].rowptr;
    const int32_t *col = fine ? c->d.col : c->mg[l - 1].col;
    const double *K = fine ? W->S->K64 : W->K[l];
    const double *M = fine ? W->S->Mp64 : W->M[l];
    const double tau = 0.0;
    const int64_t *pptr = fine ? c->d.patch_ptr : c->mg[l - 1].pptr;
    const int32_t *pdof = fine ? c->d.patch_dof : c->mg[l - 1].pdof;
    const int64_t *pioff = fine ? c->d.patch_ioff : c->mg[l - 1].pioff;
    const std::vector<int64_t> &pco = fine ? c->pcolor_off : c->mg[l - 1].pcolor_off;
    const int64_t ent = fine ? c->patch_entries : c->mg[l - 1].pent;
    const int pmax = fine ? c->patch_max : c->mg[l - 1].pmax;
    const size_t sm = (size_t)pmax * R * sizeof(double2);
    const bool ff = fine && W->ff;
    if (ff) {
        count_launch();
        mg_to_ff<<<grid_n((int64_t)n * R), 256, 0, c->stream>>>((int64_t)n * R, W->b[l], W->bff);
        cudaMemsetAsync(W->xff, 0, (size_t)n * R * sizeof(float4), c->stream);
    } else {
        cudaMemsetAsync(W->x[l], 0, (size_t)n * R * sizeof(double2), c->stream);
    }
    auto sweep = [&](int col8) {
        const int64_t a = pco[col8], b = pco[col8 + 1];
        if (b <= a) return;
        count_launch();
        const unsigned grid = (unsigned)std::min<int64_t>(b - a, 152 * 16);
        if (ff)
            mg_smooth_ff<<<grid, 128, (size_t)pmax * R * sizeof(float4), c->stream>>>(
                a, b, pptr, pdof, pioff, reinterpret_cast<const float4 *>(W->inv[l]), ent, rowptr, col, W->Kff, W->Mff,
                W->wff, R, W->npol, W->nf, W->bff, W->xff);
        else
            mg_smooth<<<grid, 128, sm, c->stream>>>(a, b, pptr, pdof, pioff, W->inv[l], ent, rowptr, col, K, M, tau,
                                                    W->wq, R, W->npol, W->nf, W->b[l], W->x[l]);
    };
    for (int col8 = 0; col8 < 8; ++col8) sweep(col8);
    if (l == nl - 1) {  // the coarsest level: one patch, solved exactly
        if (ff) {
            count_launch();
            mg_from_ff<<<grid_n((int64_t)n * R), 256, 0, c->stream>>>((int64_t)n * R, W->xff, W->x[l]);
        }
        return;
    }
    const MgLevel &C = c->mg[l];  // the next coarser level
    count_launch();
    if (ff)
        mg_resid_ff<<<grid_n((int64_t)n * R), 256, 0, c->stream>>>(n, rowptr, col, W->Kff, W->Mff, W->wff, R, W->bff,
                                                                  W->xff, W->t[l]);
    else
        mg_resid<<<grid_n((int64_t)n * R), 256, 0, c->stream>>>(n, rowptr, col, K, M, tau, W->wq, R, W->b[l], W->x[l],
                                                               W->t[l]);
    count_launch();
    mg_spmv<<<grid_n((int64_t)C.n * R), 256, 0, c->stream>>>(C.n, C.ptrow, C.ptcol, C.ptval, R, W->t[l], W->b[l + 1], 0);
    vcycle(c, W, l + 1);
    count_launch();
    if (ff)
        mg_prolong_ff<<<grid_n((int64_t)n * R), 256, 0, c->stream>>>(n, C.prow, C.pcol, C.pval, R, W->x[l + 1], W->xff);
    else
        mg_spmv<<<grid_n((int64_t)n * R), 256, 0, c->stream>>>(n, C.prow, C.pcol, C.pval, R, W->x[l + 1], W->x[l], 1);
    for (int col8 = 7; col8 >= 0; --col8) sweep(col8);
    if (ff) {
        count_launch();
        mg_from_ff<<<grid_n((int64_t)n * R), 256, 0, c->stream>>>((int64_t)n * R, W->xff, W->x[l]);
    }
}

void mg_apply(Ctx *c, MgWork *W, const double2 *r, double2 *z) {
    W->b[0] = const_cast<double2 *>(r);
    W->x[0] = z;
    vcycle(c, W, 0);
    W->b[0] = nullptr;
    W->x[0] = nullptr;
    if (W->sj) surf_apply(c, W->sj, *W->S, W->wq, r, z, W->t[0]);
}

}  // namespace mvf

using namespace mvf;

extern "C" int mvf_set_preconditioner(mvf_ctx *xc, int32_t kind, double floor_s, double tau) {
    if (!xc || kind < 0 || kind > 2) return MVF_E_ARG;
    Ctx *c = &xc->c;
    // kind 2: the multilevel method on the true conductivity (no semidefinite shift)
    c->mg_abs = kind == 2 ? 0 : 1;
    if (kind == 2) kind = 0;
    if (floor_s > 0.0) c->mg_floor = floor_s;
    if (tau >= 0.0) c->mg_tau = tau;
    c->precond = kind;
    if (kind == 0 && c->use_patches && c->mg.empty()) return mg_setup(c);
    return 0;
}

extern "C" int mvf_mg_levels(const mvf_ctx *xc, int32_t *nlevels, int32_t *ndofs, int32_t cap) {
    if (!xc || !nlevels) return MVF_E_ARG;
    const Ctx &c = xc->c;
    const int nl = c.use_patches && c.precond == 0 ? (int)c.mg.size() + 1 : 0;
    *nlevels = nl;
    if (ndofs)
        for (int l = 0; l < nl && l < cap; ++l) ndofs[l] = l == 0 ? c.nne : c.mg[l - 1].n;
    return 0;
}

// One V-cycle of the multilevel preconditioner for frequency f on R host right-hand
// sides [n][R] complex (test hook: the same cycle FGMRES applies).
extern "C" int mvf_mg_apply_once(mvf_ctx *xc, int32_t f, int32_t R, const double *r, double *z) {
    if (!xc || !r || !z || R < 1 || R > 32) return MVF_E_ARG;
    Ctx *c = &xc->c;
    if (!c->assembled) return fail(c, MVF_E_STATE, "assemble first");
    if (!c->use_patches || c->precond != 0) return fail(c, MVF_E_UNSUPPORTED, "multilevel preconditioner not in use");
    if (f < 0 || f >= c->nfreq) return fail(c, MVF_E_ARG, "bad frequency");
    const MatrixSet *S = nullptr;
    for (const MatrixSet &s : c->sets)
        if (f >= s.first_freq && f < s.first_freq + s.nfreq) S = &s;
    const double w = (c->mesh.quirks & MVF_Q_FP32_CONST) ? (double)(float)c->omega[f] : c->omega[f];
    MgWork *W = nullptr;
    // FP64 throughout, the arithmetic of the plain mode
    const int mode = c->solve_mode;
    c->solve_mode = 1;
    const int rc0 = mg_numeric(c, *S, &w, 1, R, R, &W);
    c->solve_mode = mode;
    if (rc0) return rc0;
    const size_t vb = (size_t)c->nne * R * sizeof(double2);
    double2 *dr = nullptr, *dz = nullptr;
    cudaError_t e = cudaMalloc((void **)&dr, vb);
    if (e == cudaSuccess) e = cudaMalloc((void **)&dz, vb);
    if (e == cudaSuccess) e = cudaMemcpy(dr, r, vb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        mg_apply(c, W, dr, dz);
        e = cudaStreamSynchronize(c->stream);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(z, dz, vb, cudaMemcpyDeviceToHost);
    cudaFree(dr);
    cudaFree(dz);
    mg_free(c, W);
    if (e != cudaSuccess) return cuda_fail(c, e, "multilevel apply");
    return 0;
}

// Measurement hook: one level-0 smoothing sweep (8 colour launches) of the multilevel
// preconditioner over every assembled frequency and both polarisations, in the mixed
// mode's arithmetic, timed with CUDA events on the library's stream.  Algorithmic bytes
// per sweep: every patch inverse of every frequency (16 B an entry), the CSR rows of
// the patch DOFs (column index, K and Mp halves: 20 B a nonzero) and the patch DOFs'
// right-hand side read, iterate read and write (16 B each per right-hand side).
extern "C" int mvf_profile_mg(mvf_ctx *xc, int32_t reps, double *sec_per_sweep, int64_t *bytes) {
    if (!xc || !sec_per_sweep || reps < 1) return MVF_E_ARG;
    Ctx *c = &xc->c;
    if (!c->assembled) return fail(c, MVF_E_STATE, "assemble first");
    if (!c->use_patches || c->precond != 0) return fail(c, MVF_E_UNSUPPORTED, "multilevel preconditioner not in use");
    const MatrixSet &S = c->sets[0];
    const int nf = S.nfreq, npol = 2;
    int R = 1;
    while (R < nf * npol) R <<= 1;
    std::vector<double> w(nf);
    for (int f = 0; f < nf; ++f)
        w[f] = (c->mesh.quirks & MVF_Q_FP32_CONST) ? (double)(float)c->omega[S.first_freq + f] : c->omega[S.first_freq + f];
    const int mode = c->solve_mode;
    c->solve_mode = 0;
    MgWork *W = nullptr;
    const int rc0 = mg_numeric(c, S, w.data(), nf, R, npol, &W);
    c->solve_mode = mode;
    if (rc0) return rc0;
    const size_t vb = (size_t)c->nne * R * sizeof(double2);
    double2 *b = nullptr, *x = nullptr;
    cudaError_t e = cudaMalloc((void **)&b, vb);
    if (e == cudaSuccess) e = cudaMalloc((void **)&x, vb);
    if (e == cudaSuccess) e = cudaMemsetAsync(b, 0, vb, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(x, 0, vb, c->stream);
    float ms = 0.f;
    if (e == cudaSuccess) {
        auto sweep = [&]() {
            for (int col8 = 0; col8 < 8; ++col8) {
                const int64_t a = c->pcolor_off[col8], bb = c->pcolor_off[col8 + 1];
                if (bb <= a) continue;
                count_launch();
                mg_smooth_ff<<<(unsigned)std::min<int64_t>(bb - a, 152 * 16), 128,
                               (size_t)c->patch_max * R * sizeof(float4), c->stream>>>(
                    a, bb, c->d.patch_ptr, c->d.patch_dof, c->d.patch_ioff, reinterpret_cast<const float4 *>(W->inv[0]),
                    c->patch_entries, c->d.rowptr, c->d.col, W->Kff, W->Mff, W->wff, R, npol, nf,
                    reinterpret_cast<const float4 *>(b), reinterpret_cast<float4 *>(x));
            }
        };
        sweep();
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, c->stream);
        for (int i = 0; i < reps; ++i) sweep();
        cudaEventRecord(e1, c->stream);
        e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    cudaFree(b);
    cudaFree(x);
    mg_free(c, W);
    if (e != cudaSuccess) return cuda_fail(c, e, "multilevel profile");
    *sec_per_sweep = ms * 1e-3 / reps;
    if (bytes) {
        // rows of the patch DOFs, counted on the host from the pattern
        std::vector<int64_t> rp(c->nne + 1), pp(c->npatch + 1);
        std::vector<int32_t> pd(c->patch_dofs);
        cudaMemcpy(rp.data(), c->d.rowptr, rp.size() * sizeof(int64_t), cudaMemcpyDeviceToHost);
        cudaMemcpy(pd.data(), c->d.patch_dof, pd.size() * sizeof(int32_t), cudaMemcpyDeviceToHost);
        int64_t rows = 0;
        for (int32_t g : pd) rows += rp[g + 1] - rp[g];
        *bytes = (int64_t)nf * c->patch_entries * 16 + rows * 20 + c->patch_dofs * (int64_t)(nf * npol) * 16 * 3;
    }
    return 0;
}
