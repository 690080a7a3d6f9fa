// mvf_solve.cu -- the replacement of the MUMPS solve (zmumps job=6,
// MoVFEM_3DMT.f90:113-115): right-preconditioned flexible GMRES on the GPU.
//
// Right-hand sides that share a matrix set are solved together: vectors are stored
// [row][rhs] so one pass over K and M (A_r = K + i w_r M, integration.f90:76-86)
// serves every right-hand side.  Preconditioner: z = D^-1 r + G Dphi^-1 G^T r, where D
// is the diagonal of A_r, G the discrete gradient of the edge space and Dphi the
// diagonal of G^T A_r G (the curl-curl operator vanishes on gradients, so Jacobi alone
// stalls on them; nodes whose Dphi vanishes -- air, where Re(sigma)=0 -- are left out).
// Mode 0 runs the Krylov method in complex FP32 with FP64 reductions and an FP64
// Hessenberg least-squares problem inside FP64 iterative refinement (true residual
// b - A x in FP64).  Mode 1 is the plain FP64 method, one right-hand side at a time.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <vector>

#include "mvf_internal.cuh"

namespace mvf {

template <class T>
struct C2;
template <>
struct C2<float> {
    using V = float2;
};
template <>
struct C2<double> {
    using V = double2;
};

constexpr int MAXR = 32;  // right-hand sides per batch

// angular frequency of every right-hand side of a batch, exact and FP32-rounded; one
// copy per context in device memory (solves on different contexts may overlap)
struct SolveParams {
    double omega[MAXR];
    double w32[MAXR];
};

// y = A x (b == nullptr) or y = b - A x for R right-hand sides sharing K, M.
// One warp per row.  The warp loads 32 consecutive nonzeros (K, M, column) with
// coalesced loads, then broadcasts them by shuffle: lane l works on right-hand side
// l % R for the nonzeros j = l / R, l / R + 32/R, ... of the chunk, reading
// x[col][r] as one contiguous run of R complex values per nonzero.
template <class T, class TV, int R>
__global__ void __launch_bounds__(256) spmm_km(int32_t n, const int64_t *__restrict__ rowptr,
                                                const int32_t *__restrict__ col, const T *__restrict__ K,
                                                const T *__restrict__ M, const TV *__restrict__ x,
                                                const TV *__restrict__ b, TV *__restrict__ y, int use_w32,
                                                const SolveParams *__restrict__ sp) {
    constexpr int SL = 32 / R;
    const int lane = threadIdx.x & 31;
    const int r = lane % R, s = lane / R;
    const T w = use_w32 ? (T)sp->w32[r] : (T)sp->omega[r];
    for (int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; row < n;
         row += ((int64_t)gridDim.x * blockDim.x) >> 5) {
        const int64_t k0 = rowptr[row], k1 = rowptr[row + 1];
        T ar = 0, ai = 0, br = 0, bi = 0;
        for (int64_t kc = k0; kc < k1; kc += 32) {
            const int cnt = (int)min((int64_t)32, k1 - kc);
            const bool have = lane < cnt;
            const T kl = have ? K[kc + lane] : T(0);
            const T ml = have ? M[kc + lane] : T(0);
            const int cl = have ? col[kc + lane] : 0;
#pragma unroll
            for (int jb = 0; jb < 32; jb += SL) {
                const int j = jb + s;
                const T kv = __shfl_sync(0xffffffffu, kl, j);
                const T mv = __shfl_sync(0xffffffffu, ml, j);
                const int c = __shfl_sync(0xffffffffu, cl, j);
                if (j < cnt) {
                    const TV xv = x[(int64_t)c * R + r];
                    // (K + i w M)(xr + i xi)
                    ar += kv * xv.x;
                    ai += kv * xv.y;
                    br += mv * xv.x;
                    bi += mv * xv.y;
                }
            }
        }
        T yr = ar - w * bi, yi = ai + w * br;
#pragma unroll
        for (int o = 16; o >= R; o >>= 1) {
            yr += __shfl_down_sync(0xffffffffu, yr, o);
            yi += __shfl_down_sync(0xffffffffu, yi, o);
        }
        if (s == 0) {
            TV out;
            if (b) {
                const TV bv = b[row * R + r];
                out.x = bv.x - yr;
                out.y = bv.y - yi;
            } else {
                out.x = yr;
                out.y = yi;
            }
            y[row * R + r] = out;
        }
    }
}

// Variant for R <= 4 right-hand sides: lanes stride directly over the row's nonzeros
// (32/R consecutive nonzeros per step, loads coalesced across the lanes of one rhs),
// two steps in flight per iteration.
template <class T, class TV, int R>
__global__ void __launch_bounds__(256) spmm_km_direct(int32_t n, const int64_t *__restrict__ rowptr,
                                                       const int32_t *__restrict__ col, const T *__restrict__ K,
                                                       const T *__restrict__ M, const TV *__restrict__ x,
                                                       const TV *__restrict__ b, TV *__restrict__ y, int use_w32,
                                                const SolveParams *__restrict__ sp) {
    constexpr int SL = 32 / R;
    const int lane = threadIdx.x & 31;
    const int r = lane % R, s = lane / R;
    const T w = use_w32 ? (T)sp->w32[r] : (T)sp->omega[r];
    for (int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; row < n;
         row += ((int64_t)gridDim.x * blockDim.x) >> 5) {
        const int64_t k0 = rowptr[row], k1 = rowptr[row + 1];
        T ar = 0, ai = 0, br = 0, bi = 0;
        int64_t k = k0 + s;
        for (; k + SL < k1; k += 2 * SL) {
            const T kv0 = __ldg(K + k), mv0 = __ldg(M + k), kv1 = __ldg(K + k + SL), mv1 = __ldg(M + k + SL);
            const int c0 = __ldg(col + k), c1 = __ldg(col + k + SL);
            const TV x0 = x[(int64_t)c0 * R + r], x1 = x[(int64_t)c1 * R + r];
            ar += kv0 * x0.x + kv1 * x1.x;
            ai += kv0 * x0.y + kv1 * x1.y;
            br += mv0 * x0.x + mv1 * x1.x;
            bi += mv0 * x0.y + mv1 * x1.y;
        }
        if (k < k1) {
            const T kv = __ldg(K + k), mv = __ldg(M + k);
            const TV xv = x[(int64_t)__ldg(col + k) * R + r];
            ar += kv * xv.x;
            ai += kv * xv.y;
            br += mv * xv.x;
            bi += mv * xv.y;
        }
        T yr = ar - w * bi, yi = ai + w * br;
#pragma unroll
        for (int o = 16; o >= R; o >>= 1) {
            yr += __shfl_down_sync(0xffffffffu, yr, o);
            yi += __shfl_down_sync(0xffffffffu, yi, o);
        }
        if (s == 0) {
            TV out;
            if (b) {
                const TV bv = b[row * R + r];
                out.x = bv.x - yr;
                out.y = bv.y - yi;
            } else {
                out.x = yr;
                out.y = yi;
            }
            y[row * R + r] = out;
        }
    }
}

// R consecutive complex values x[0..R) into registers with the widest aligned loads
// (16-byte runs: two complex64 or one complex128 per load).
template <class T, class TV, int R>
__device__ __forceinline__ void load_run(const TV *__restrict__ p, TV (&v)[R]) {
    if constexpr (sizeof(TV) == 8 && R % 2 == 0) {
        const float4 *q = reinterpret_cast<const float4 *>(p);
#pragma unroll
        for (int i = 0; i < R / 2; ++i) {
            const float4 t = __ldg(q + i);
            v[2 * i].x = t.x;
            v[2 * i].y = t.y;
            v[2 * i + 1].x = t.z;
            v[2 * i + 1].y = t.w;
        }
    } else {
#pragma unroll
        for (int i = 0; i < R; ++i) v[i] = p[i];
    }
}

// G lanes per row, 32/G rows per warp, every lane carrying all R right-hand sides:
// each nonzero costs one column index, one K and one M value, and one contiguous
// R-complex run of x -- against R copies of the index and values when lanes are split
// over the right-hand sides.  The group's partial sums meet by xor-shuffles; lane j of
// the group writes right-hand sides j, j+G, ...
template <class T, class TV, int R, int G>
__global__ void __launch_bounds__(256) spmm_km_vec(int32_t n, const int64_t *__restrict__ rowptr,
                                                    const int32_t *__restrict__ col, const T *__restrict__ K,
                                                    const T *__restrict__ M, const TV *__restrict__ x,
                                                    const TV *__restrict__ b, TV *__restrict__ y, int use_w32,
                                                const SolveParams *__restrict__ sp) {
    constexpr int RPW = 32 / G;
    const int lane = threadIdx.x & 31, g = lane / G, j = lane % G;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t base = warp * RPW; base < n; base += nwarps * RPW) {
        const int64_t row = base + g;
        int64_t k0 = 0, k1 = 0;
        if (row < n) {
            k0 = __ldg(rowptr + row);
            k1 = __ldg(rowptr + row + 1);
        }
        T kr[R], ki[R], mr[R], mi[R];
#pragma unroll
        for (int r = 0; r < R; ++r) kr[r] = ki[r] = mr[r] = mi[r] = T(0);
        int64_t k = k0 + j;
        for (; k + G < k1; k += 2 * G) {
            const int c0 = __ldg(col + k), c1 = __ldg(col + k + G);
            const T kv0 = __ldg(K + k), mv0 = __ldg(M + k), kv1 = __ldg(K + k + G), mv1 = __ldg(M + k + G);
            TV x0[R], x1[R];
            load_run<T, TV, R>(x + (int64_t)c0 * R, x0);
            load_run<T, TV, R>(x + (int64_t)c1 * R, x1);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                kr[r] += kv0 * x0[r].x + kv1 * x1[r].x;
                ki[r] += kv0 * x0[r].y + kv1 * x1[r].y;
                mr[r] += mv0 * x0[r].x + mv1 * x1[r].x;
                mi[r] += mv0 * x0[r].y + mv1 * x1[r].y;
            }
        }
        if (k < k1) {
            const int c0 = __ldg(col + k);
            const T kv0 = __ldg(K + k), mv0 = __ldg(M + k);
            TV x0[R];
            load_run<T, TV, R>(x + (int64_t)c0 * R, x0);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                kr[r] += kv0 * x0[r].x;
                ki[r] += kv0 * x0[r].y;
                mr[r] += mv0 * x0[r].x;
                mi[r] += mv0 * x0[r].y;
            }
        }
        // (K + i w M) x: fold w in before the reduction
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const T w = use_w32 ? (T)sp->w32[r] : (T)sp->omega[r];
            kr[r] -= w * mi[r];
            ki[r] += w * mr[r];
        }
#pragma unroll
        for (int o = G / 2; o >= 1; o >>= 1)
#pragma unroll
            for (int r = 0; r < R; ++r) {
                kr[r] += __shfl_xor_sync(0xffffffffu, kr[r], o);
                ki[r] += __shfl_xor_sync(0xffffffffu, ki[r], o);
            }
        if (row < n) {
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (r % G != j) continue;
                TV out;
                if (b) {
                    const TV bv = b[row * R + r];
                    out.x = bv.x - kr[r];
                    out.y = bv.y - ki[r];
                } else {
                    out.x = kr[r];
                    out.y = ki[r];
                }
                y[row * R + r] = out;
            }
        }
    }
}

// ---- float-float K/M SpMM for the FP64 Krylov vectors of the 36/54-DOF systems -------
// The FP64 SpMM is bound by GB300's FP64 pipe.  Here K and M are held as hi + lo FP32
// halves (8 bytes a value, as FP64), the Krylov vector is split the same way once per
// product, and the products and sums run in float-float arithmetic on the FP32 pipe
// (FMA-exact products, TwoSum), about 44 significant bits.  Only the inner Krylov
// operator uses it; every true residual stays in FP64.

__device__ __forceinline__ void ffm(float &sh, float &sl, float ah, float al, float bh, float bl) {
    const float p = ah * bh;
    float e = fmaf(ah, bh, -p);
    e = fmaf(ah, bl, fmaf(al, bh, e));
    const float t = sh + p;
    const float bb = t - sh;
    const float err = (sh - (t - bb)) + (p - bb);
    const float lo = sl + e + err;
    sh = t + lo;
    sl = lo - (sh - t);
}

__device__ __forceinline__ void ffadd(float &sh, float &sl, float bh, float bl) {
    const float t = sh + bh;
    const float bb = t - sh;
    const float err = (sh - (t - bb)) + (bh - bb);
    const float lo = sl + bl + err;
    sh = t + lo;
    sl = lo - (sh - t);
}

__global__ void split_values(int64_t n, const double *__restrict__ a, float2 *__restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = a[i];
        const float h = __double2float_rn(v);
        out[i] = make_float2(h, __double2float_rn(v - (double)h));
    }
}

__global__ void split_vector(int64_t n, const double2 *__restrict__ x, float4 *__restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double2 v = x[i];
        const float xh = __double2float_rn(v.x), yh = __double2float_rn(v.y);
        out[i] = make_float4(xh, yh, __double2float_rn(v.x - (double)xh), __double2float_rn(v.y - (double)yh));
    }
}

// y = (K + i w M) x for R right-hand sides r0 .. r0+R-1 of vectors holding RS per row,
// G lanes per row, each lane all R; the group's float-float partial sums meet by
// xor-shuffles with TwoSum.
template <int R, int G>
__global__ void __launch_bounds__(256) spmm_ff(int32_t n, const int64_t *__restrict__ rowptr,
                                               const int32_t *__restrict__ col, const float2 *__restrict__ K,
                                               const float2 *__restrict__ M, const float4 *__restrict__ x,
                                               double2 *__restrict__ y, const SolveParams *__restrict__ sp, int RS,
                                               int r0) {
    constexpr int RPW = 32 / G;
    const int lane = threadIdx.x & 31, g = lane / G, j = lane % G;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t base = warp * RPW; base < n; base += nwarps * RPW) {
        const int64_t row = base + g;
        int64_t k0 = 0, k1 = 0;
        if (row < n) {
            k0 = __ldg(rowptr + row);
            k1 = __ldg(rowptr + row + 1);
        }
        // [r][0..7]: K x re (hi, lo), K x im, M x re, M x im
        float acc[R][8];
#pragma unroll
        for (int r = 0; r < R; ++r)
#pragma unroll
            for (int q = 0; q < 8; ++q) acc[r][q] = 0.f;
        for (int64_t k = k0 + j; k < k1; k += G) {
            const int c = __ldg(col + k);
            const float2 kv = __ldg(K + k), mv = __ldg(M + k);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const float4 xv = __ldg(x + (int64_t)c * RS + r0 + r);
                ffm(acc[r][0], acc[r][1], kv.x, kv.y, xv.x, xv.z);
                ffm(acc[r][2], acc[r][3], kv.x, kv.y, xv.y, xv.w);
                ffm(acc[r][4], acc[r][5], mv.x, mv.y, xv.x, xv.z);
                ffm(acc[r][6], acc[r][7], mv.x, mv.y, xv.y, xv.w);
            }
        }
#pragma unroll
        for (int o = G / 2; o >= 1; o >>= 1)
#pragma unroll
            for (int r = 0; r < R; ++r)
#pragma unroll
                for (int q = 0; q < 8; q += 2) {
                    const float bh = __shfl_xor_sync(0xffffffffu, acc[r][q], o);
                    const float bl = __shfl_xor_sync(0xffffffffu, acc[r][q + 1], o);
                    ffadd(acc[r][q], acc[r][q + 1], bh, bl);
                }
        if (row < n) {
#pragma unroll
            for (int r = 0; r < R; ++r) {
                if (r % G != j) continue;
                const double w = sp->w32[r0 + r];
                const double kr = (double)acc[r][0] + acc[r][1], ki = (double)acc[r][2] + acc[r][3];
                const double mr = (double)acc[r][4] + acc[r][5], mi = (double)acc[r][6] + acc[r][7];
                y[row * RS + r0 + r] = make_double2(kr - w * mi, ki + w * mr);
            }
        }
    }
}

// diagonal entries of K and M
__global__ void extract_diag(int32_t n, const int64_t *__restrict__ rowptr, const int32_t *__restrict__ col,
                             const double *__restrict__ K, const double *__restrict__ M, double *__restrict__ kd,
                             double *__restrict__ md) {
    for (int32_t r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
        double a = 0, b = 0;
        for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
            if (col[k] == r) { a = K[k]; b = M[k]; }
        kd[r] = a;
        md[r] = b;
    }
}

// inverse diagonals of the preconditioner for each rhs: dinv [n][R], pinv [ngn][R]
__global__ void build_inverse_diag(int32_t n, int32_t ngn, int R, const double *__restrict__ kd,
                                   const double *__restrict__ md, const double *__restrict__ kphi,
                                   const double *__restrict__ mphi, const double *__restrict__ mabs,
                                   double2 *__restrict__ dinv, double2 *__restrict__ pinv,
                                   const SolveParams *__restrict__ sp) {
    const int64_t tot = ((int64_t)n + ngn) * R;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < tot; t += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(t % R);
        const int64_t i = t / R;
        const double w = sp->w32[r];
        if (i < n) {
            const double a = kd[i], b = w * md[i];
            const double s = a * a + b * b;
            dinv[i * R + r] = s > 0 ? make_double2(a / s, -b / s) : make_double2(0.0, 0.0);
        } else {
            const int64_t j = i - n;
            const double a = kphi[j], b = w * mphi[j];
            const double scale = fabs(kphi[j]) + w * mabs[j];
            const double s = a * a + b * b;
            // keep a gradient node only where the mass part is a real fraction of its scale
            const bool keep = scale > 0 && w * fabs(mphi[j]) > 1e-8 * scale && s > 0;
            pinv[j * R + r] = keep ? make_double2(a / s, -b / s) : make_double2(0.0, 0.0);
        }
    }
}

// t = Pinv .* (G^T r)   (gradient nodes)
template <class TV>
__global__ void grad_t(int32_t ngn, int R, const int64_t *__restrict__ gtrow, const int32_t *__restrict__ gtcol,
                       const float *__restrict__ gtval, const TV *__restrict__ r, const double2 *__restrict__ pinv,
                       TV *__restrict__ t) {
    const int64_t tot = (int64_t)ngn * R;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < tot; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = q / R;
        const int rr = (int)(q % R);
        double sr = 0, si = 0;
        for (int64_t k = gtrow[j]; k < gtrow[j + 1]; ++k) {
            const TV v = r[(int64_t)gtcol[k] * R + rr];
            sr += gtval[k] * (double)v.x;
            si += gtval[k] * (double)v.y;
        }
        const double2 p = pinv[q];
        TV o;
        o.x = (decltype(o.x))(p.x * sr - p.y * si);
        o.y = (decltype(o.y))(p.x * si + p.y * sr);
        t[q] = o;
    }
}

// z = Dinv .* r + G t
template <class TV>
__global__ void apply_prec(int32_t n, int R, const int64_t *__restrict__ grow, const int32_t *__restrict__ gcol,
                           const float *__restrict__ gval, const TV *__restrict__ r, const double2 *__restrict__ dinv,
                           const TV *__restrict__ t, TV *__restrict__ z) {
    const int64_t tot = (int64_t)n * R;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < tot; q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = q / R;
        const int rr = (int)(q % R);
        const TV v = r[q];
        const double2 d = dinv[q];
        double zr = d.x * v.x - d.y * v.y, zi = d.x * v.y + d.y * v.x;
        for (int64_t k = grow[i]; k < grow[i + 1]; ++k) {
            const TV tv = t[(int64_t)gcol[k] * R + rr];
            zr += gval[k] * (double)tv.x;
            zi += gval[k] * (double)tv.y;
        }
        TV o;
        o.x = (decltype(o.x))zr;
        o.y = (decltype(o.y))zi;
        z[q] = o;
    }
}

// Partial sums of conj(V_j) . w for j < k and all rhs (FP64 accumulation), one row
// of partial[block][j][r] per block.  Threads keep 8 projections in registers while
// streaming w once per group of 8 basis vectors; lanes with the same rhs are combined
// with shuffles, warps through shared-memory atomics ([k][R] doubles).
template <class TV>
__global__ void __launch_bounds__(256) multidot(int32_t n, int R, int k, const TV *__restrict__ V, int64_t vstride,
                                                 const TV *__restrict__ w, double2 *__restrict__ partial) {
    extern __shared__ double red[];  // [k*R][2]
    constexpr int JC = 8;
    const int lane = threadIdx.x & 31;
    const int kr = k * R;
    for (int t = threadIdx.x; t < 2 * kr; t += blockDim.x) red[t] = 0.0;
    __syncthreads();
    const int r = threadIdx.x % R;  // R divides 32 and blockDim, so fixed per thread
    const int64_t tot = (int64_t)n * R;
    for (int j0 = 0; j0 < k; j0 += JC) {
        const int jn = min(JC, k - j0);
        double sr[JC], si[JC];
#pragma unroll
        for (int q = 0; q < JC; ++q) sr[q] = si[q] = 0.0;
        if constexpr (sizeof(TV) == 8) {
            // complex64 vectors: products and runs of up to 4 terms in FP32, every run
            // added into the FP64 sums (FP64 arithmetic is scarce on GB300; the FP32
            // products carry the same relative error as the complex64 entries)
            float fr[JC], fi[JC];
            int run = 0;
#pragma unroll
            for (int q = 0; q < JC; ++q) fr[q] = fi[q] = 0.f;
            for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < tot;
                 q += (int64_t)gridDim.x * blockDim.x) {
                const TV b = w[q];
#pragma unroll
                for (int jj = 0; jj < JC; ++jj) {
                    if (jj < jn) {
                        const TV a = V[(int64_t)(j0 + jj) * vstride + q];
                        fr[jj] = fmaf(a.x, b.x, fmaf(a.y, b.y, fr[jj]));
                        fi[jj] = fmaf(a.x, b.y, fmaf(-a.y, b.x, fi[jj]));
                    }
                }
                if (++run == 4) {
#pragma unroll
                    for (int jj = 0; jj < JC; ++jj) {
                        sr[jj] += fr[jj];
                        si[jj] += fi[jj];
                        fr[jj] = fi[jj] = 0.f;
                    }
                    run = 0;
                }
            }
#pragma unroll
            for (int jj = 0; jj < JC; ++jj) {
                sr[jj] += fr[jj];
                si[jj] += fi[jj];
            }
        } else {
            for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < tot;
                 q += (int64_t)gridDim.x * blockDim.x) {
                const TV b = w[q];
#pragma unroll
                for (int jj = 0; jj < JC; ++jj) {
                    if (jj < jn) {
                        const TV a = V[(int64_t)(j0 + jj) * vstride + q];
                        sr[jj] += (double)a.x * b.x + (double)a.y * b.y;
                        si[jj] += (double)a.x * b.y - (double)a.y * b.x;
                    }
                }
            }
        }
#pragma unroll
        for (int jj = 0; jj < JC; ++jj) {
            double xr = sr[jj], xi = si[jj];
            for (int o = 16; o >= R; o >>= 1) {
                xr += __shfl_down_sync(0xffffffffu, xr, o);
                xi += __shfl_down_sync(0xffffffffu, xi, o);
            }
            if (jj < jn && lane < R) {
                atomicAdd(&red[2 * ((j0 + jj) * R + r)], xr);
                atomicAdd(&red[2 * ((j0 + jj) * R + r) + 1], xi);
            }
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < kr; t += blockDim.x)
        partial[(int64_t)blockIdx.x * kr + t] = make_double2(red[2 * t], red[2 * t + 1]);
}

// sum the block partials: h[t] (+)= sum_b partial[b][t]
__global__ void reduce_partials(int nblocks, int kr, const double2 *__restrict__ partial, double2 *__restrict__ h,
                                int accumulate) {
    const int t = blockIdx.x;
    double sr = 0, si = 0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
        sr += partial[(int64_t)b * kr + t].x;
        si += partial[(int64_t)b * kr + t].y;
    }
    __shared__ double2 s[256];
    s[threadIdx.x] = make_double2(sr, si);
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            s[threadIdx.x].x += s[threadIdx.x + o].x;
            s[threadIdx.x].y += s[threadIdx.x + o].y;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        if (accumulate) {
            h[t].x += s[0].x;
            h[t].y += s[0].y;
        } else {
            h[t] = s[0];
        }
    }
}

// w -= sum_j c[j][r] V_j  (c is the last projection, FP64)
template <class TV>
__global__ void axpy_multi(int32_t n, int R, int k, const TV *__restrict__ V, int64_t vstride,
                           const double2 *__restrict__ c, TV *__restrict__ w) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < (int64_t)n * R;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(q % R);
        TV o = w[q];
        double orr = o.x, oi = o.y;
        for (int j = 0; j < k; ++j) {
            const TV v = V[(int64_t)j * vstride + q];
            const double2 h = c[j * R + r];
            orr -= h.x * v.x - h.y * v.y;
            oi -= h.x * v.y + h.y * v.x;
        }
        o.x = (decltype(o.x))orr;
        o.y = (decltype(o.y))oi;
        w[q] = o;
    }
}

// v = w / nrm[r]  (nrm from a 1-vector multidot of w with itself)
template <class TV>
__global__ void scale_into(int32_t n, int R, const TV *__restrict__ w, const double2 *__restrict__ nrm2,
                           TV *__restrict__ v) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < (int64_t)n * R;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(q % R);
        const double nr = sqrt(fmax(nrm2[r].x, 0.0));
        const double s = nr > 0 ? 1.0 / nr : 0.0;
        TV o = w[q];
        o.x = (decltype(o.x))(o.x * s);
        o.y = (decltype(o.y))(o.y * s);
        v[q] = o;
    }
}

// Hessenberg column k for each rhs: h[0..k] from the two CGS passes (hc), h[k+1] =
// ||w||; apply the previous Givens rotations, form the new one, update g.
constexpr int MAXM = 256;  // longest FGMRES cycle (restart length)
struct Hess {
    double2 H[MAXM][MAXM + 1];  // H[row][col], (m+1) x m
    double2 cs[MAXM];           // cos (real) packed in .x; sin complex
    double2 sn[MAXM];
    double2 g[MAXM + 1];
    double beta;
    int active;
};

// The new column k runs through the k previous rotations, a chain of dependent
// updates: it is held in shared memory (one column per right-hand side, lane r) so
// the chain waits on shared-memory latency, and the rotations are read up front.
__global__ void hessenberg_step(int R, int k, const double2 *__restrict__ hc, const double2 *__restrict__ wn2, Hess *hs) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R || k >= MAXM) return;
    Hess &S = hs[r];
    // previous rotations [c s; -conj(s) c] (c real) applied down the new column: rotation
    // i mixes entries i and i+1; entry i is then final, entry i+1 carries on.  The loads
    // of hc and the rotations do not depend on the chain, which is arithmetic only.
    double2 carry = hc[r];
    for (int i = 0; i < k; ++i) {
        const double c = S.cs[i].x;
        const double2 s = S.sn[i];
        const double2 a = carry, b = hc[(i + 1) * R + r];
        double2 t1, t2;
        t1.x = c * a.x + (s.x * b.x - s.y * b.y);
        t1.y = c * a.y + (s.x * b.y + s.y * b.x);
        t2.x = -(s.x * a.x + s.y * a.y) + c * b.x;
        t2.y = -(s.x * a.y - s.y * a.x) + c * b.y;
        S.H[i][k] = t1;
        carry = t2;
    }
    const double2 a = carry;
    const double bb = sqrt(fmax(wn2[r].x, 0.0));  // ||w||, real and >= 0
    const double na = hypot(a.x, a.y);
    double c;
    double2 s;
    if (bb == 0.0) { c = 1.0; s = make_double2(0.0, 0.0); }
    else if (na == 0.0) { c = 0.0; s = make_double2(1.0, 0.0); }
    else {
        const double nrm = hypot(na, bb);
        c = na / nrm;
        // s = (a/|a|) * conj(b) / nrm  with b real
        s = make_double2(a.x / na * bb / nrm, a.y / na * bb / nrm);
    }
    S.cs[k] = make_double2(c, 0.0);
    S.sn[k] = s;
    // H[k][k] = c a + s b
    S.H[k][k] = make_double2(c * a.x + s.x * bb, c * a.y + s.y * bb);
    S.H[k + 1][k] = make_double2(0.0, 0.0);
    const double2 gk = S.g[k];
    S.g[k] = make_double2(c * gk.x, c * gk.y);
    // g[k+1] = -conj(s) g[k]
    S.g[k + 1] = make_double2(-(s.x * gk.x + s.y * gk.y), -(s.x * gk.y - s.y * gk.x));
}

// residual estimate |g[k]| / beta of every right-hand side after k steps
__global__ void hessenberg_est(int R, int k, const Hess *hs, double *__restrict__ est) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    const Hess &S = hs[r];
    est[r] = S.beta > 0 ? hypot(S.g[k].x, S.g[k].y) / S.beta : 0.0;
}

__global__ void hessenberg_init(int R, const double2 *__restrict__ rn2, Hess *hs) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= R) return;
    const double b = sqrt(fmax(rn2[r].x, 0.0));
    hs[r].beta = b;
    hs[r].g[0] = make_double2(b, 0.0);
    for (int i = 1; i < MAXM + 1; ++i) hs[r].g[i] = make_double2(0.0, 0.0);
}

// back substitution: y = H(0:k,0:k)^-1 g(0:k), stored in yout[j][r].  One warp per
// right-hand side (block r): for each row the lanes form the products with the known
// y_j (j = lane, lane + 32) and a shuffle sum, so the row chain waits on one
// reduction instead of k dependent loads.
__global__ void hessenberg_solve(int R, int k, Hess *hs, double2 *__restrict__ yout) {
    __shared__ double2 y[MAXM];
    const int r = blockIdx.x, lane = threadIdx.x;
    if (r >= R || k > MAXM) return;
    Hess &S = hs[r];
    for (int i = k - 1; i >= 0; --i) {
        double tr = 0.0, ti = 0.0;
        for (int j = i + 1 + lane; j < k; j += 32) {
            const double2 h = S.H[i][j], v = y[j];
            tr += h.x * v.x - h.y * v.y;
            ti += h.x * v.y + h.y * v.x;
        }
        for (int o = 16; o > 0; o >>= 1) {
            tr += __shfl_xor_sync(0xffffffffu, tr, o);
            ti += __shfl_xor_sync(0xffffffffu, ti, o);
        }
        if (lane == 0) {
            const double2 g = S.g[i], d = S.H[i][i];
            const double t_r = g.x - tr, t_i = g.y - ti;
            const double dd = d.x * d.x + d.y * d.y;
            y[i] = dd > 0 ? make_double2((t_r * d.x + t_i * d.y) / dd, (t_i * d.x - t_r * d.y) / dd)
                          : make_double2(0, 0);
        }
        __syncwarp();
    }
    for (int i = lane; i < k; i += 32) yout[i * R + r] = y[i];
}

// x += sum_j y[j][r] Z_j   (x in FP64; Z in the Krylov precision)
template <class TV, class XV>
__global__ void update_x(int32_t n, int R, int k, const TV *__restrict__ Z, int64_t zstride,
                         const double2 *__restrict__ y, XV *__restrict__ x, int xstride_r, int xoff) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < (int64_t)n * R;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(q % R);
        double sr = 0, si = 0;
        for (int j = 0; j < k; ++j) {
            const TV z = Z[(int64_t)j * zstride + q];
            const double2 c = y[j * R + r];
            sr += c.x * z.x - c.y * z.y;
            si += c.x * z.y + c.y * z.x;
        }
        const int64_t i = q / R;
        XV &o = x[i * xstride_r + xoff + r];
        o.x += sr;
        o.y += si;
    }
}

template <class TV>
__global__ void cast_vec(int64_t n, const double2 *__restrict__ a, TV *__restrict__ b, double scale) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
        TV o;
        o.x = (decltype(o.x))(a[q].x * scale);
        o.y = (decltype(o.y))(a[q].y * scale);
        b[q] = o;
    }
}

// gather rhs [f][p][n] -> [n][R] and scatter back
// (padding right-hand sides r >= Rreal read as zero and are not written back)
__global__ void gather_rhs(int32_t n, int R, int Rreal, int f0, const double2 *__restrict__ src,
                           double2 *__restrict__ dst) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < (int64_t)n * R;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(q % R);
        const int64_t i = q / R;
        dst[q] = r < Rreal ? src[((int64_t)(f0 * 2 + r)) * n + i] : make_double2(0.0, 0.0);
    }
}
__global__ void scatter_sol(int32_t n, int R, int Rreal, int f0, const double2 *__restrict__ src,
                            double2 *__restrict__ dst) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < (int64_t)n * R;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(q % R);
        const int64_t i = q / R;
        if (r < Rreal) dst[((int64_t)(f0 * 2 + r)) * n + i] = src[q];
    }
}

// ------------------------------------------------------------------------ host side
struct Work {
    int R = 0, m = 0;
    int passes = 2;  // Gram-Schmidt passes per iteration
    int32_t n = 0;
    int nblocks = 0;
    void *V = nullptr, *Z = nullptr, *w = nullptr, *t = nullptr;  // Krylov precision
    double2 *x64 = nullptr, *b64 = nullptr, *r64 = nullptr;       // [n][R]
    double2 *dinv = nullptr, *pinv = nullptr;
    double2 *partial = nullptr, *hc = nullptr, *htmp = nullptr, *nrm = nullptr, *y = nullptr;
    double *kd = nullptr, *md = nullptr;
    Hess *hs = nullptr;
    double *est = nullptr;  // [R] residual estimates of the running cycle
    size_t vb = 0;
    double2 *pinvs = nullptr;  // vertex-patch inverses, one set per frequency
    double2 *xbest = nullptr;  // iterate with the lowest true residual so far
    float4 *xf = nullptr;      // float-float copy of the SpMM input (float-float operator)
    MgWork *mg = nullptr;      // multilevel preconditioner of the 36/54-DOF systems
    int npol = 2, nfi = 1;
    // captured blocks of Arnoldi steps (see fgmres_cycle)
    static constexpr int GCH = 10, MAXB = 8;
    cudaGraphExec_t blocks[MAXB] = {};
    int64_t block_launches[MAXB] = {};
    int cycles = 0;
};

// Work buffers come from the stream-ordered allocator: no device-wide synchronisation
// when they are freed, so solves on different contexts can overlap (mvf_solve_many).
static void free_work(Ctx *c, Work &W) {
    for (cudaGraphExec_t &g : W.blocks)
        if (g) cudaGraphExecDestroy(g);
    void *p[] = {W.V, W.Z, W.w, W.t, W.x64, W.b64, W.r64, W.dinv, W.pinv, W.partial, W.hc, W.htmp, W.nrm, W.y, W.kd, W.md, W.hs,
                 W.xbest, W.xf, W.est};
    for (void *q : p)
        if (q) cudaFreeAsync(q, c->stream);
    if (W.pinvs) cudaFree(W.pinvs);
    if (W.mg) mg_free(c, W.mg);
    W = Work{};
}

template <class T>
static int alloc_work(Ctx *c, Work &W, int R, int m) {
    using TV = typename C2<T>::V;
    W.R = R;
    W.m = m;
    W.n = c->nne;
    // reduction blocks: at least 2 vector entries per thread, at most 4 blocks per SM.
    // The projections are FP64 arithmetic, which GB300 runs at a small fraction of
    // its FP32 rate, so small systems must still spread over every SM.
    W.nblocks = (int)std::max<int64_t>(1, std::min<int64_t>(152 * 4, ((int64_t)c->nne * R + 511) / 512));
    const size_t nv = (size_t)W.n * R;
    W.vb = nv * sizeof(TV);
    MVF_CUDA(c, cudaMallocAsync(&W.V, W.vb * (m + 1), c->stream));
    MVF_CUDA(c, cudaMallocAsync(&W.Z, W.vb * m, c->stream));
    MVF_CUDA(c, cudaMallocAsync(&W.w, W.vb, c->stream));
    MVF_CUDA(c, cudaMallocAsync(&W.t, (size_t)std::max(c->ngn, 1) * R * sizeof(TV), c->stream));
    MVF_CUDA(c, cudaMallocAsync((void **)&W.x64, nv * sizeof(double2), c->stream));
    MVF_CUDA(c, cudaMallocAsync((void **)&W.b64, nv * sizeof(double2), c->stream));
    MVF_CUDA(c, cudaMallocAsync((void **)&W.r64, nv * sizeof(double2), c->stream));
    MVF_CUDA(c, cudaMallocAsync((void **)&W.dinv, nv * sizeof(double2), c->stream));
    MVF_CUDA(c, cudaMallocAsync((void **)&W.pinv, (size_t)std::max(c->ngn, 1) * R * sizeof(double2), c->stream));
    MVF_CUDA(c, cudaMallocAsync((void **)&W.partial, (size_t)W.nblocks * (m + 1) * R * sizeof(double2), c->stream));
    MVF_CUDA(c, cudaMallocAsync((void **)&W.hc, (size_t)(m + 1) * R * sizeof(double2), c->stream));
    MVF_CUDA(c, cudaMallocAsync((void **)&W.htmp, (size_t)(m + 1) * R * sizeof(double2), c->stream));
    MVF_CUDA(c, cudaMallocAsync((void **)&W.nrm, (size_t)R * sizeof(double2), c->stream));
    MVF_CUDA(c, cudaMallocAsync((void **)&W.y, (size_t)(m + 1) * R * sizeof(double2), c->stream));
    MVF_CUDA(c, cudaMallocAsync((void **)&W.kd, (size_t)W.n * sizeof(double), c->stream));
    MVF_CUDA(c, cudaMallocAsync((void **)&W.md, (size_t)W.n * sizeof(double), c->stream));
    MVF_CUDA(c, cudaMallocAsync((void **)&W.hs, (size_t)R * sizeof(Hess), c->stream));
    MVF_CUDA(c, cudaMallocAsync((void **)&W.est, (size_t)R * sizeof(double), c->stream));
    // the projections of a long cycle need more than the default 48 KB of shared memory
    MVF_CUDA(c, cudaFuncSetAttribute(multidot<TV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)std::max<size_t>(48 * 1024, (size_t)(m + 1) * R * sizeof(double2))));
    return 0;
}

// SpMM variants: 0 chunked (spmm_km), 1 direct (R <= 4), 2..5 vec with G = 4, 8, 16,
// 32 lanes per row (R <= 16).
constexpr int SPMM_VARIANTS = 6;
static const char *const spmm_names[SPMM_VARIANTS] = {"chunked", "direct", "vec/G=4", "vec/G=8", "vec/G=16",
                                                      "vec/G=32"};

static bool spmm_ok(int v, int R) { return v == 0 || (v == 1 && R <= 4) || (v >= 2 && R <= 16); }

template <class T, class TV, int R>
static void spmm_variant(Ctx *c, int v, const T *K, const T *M, const TV *x, const TV *b, TV *y, int use_w32) {
    const int threads = 256;
    const int G = v >= 2 ? (4 << (v - 2)) : 32;
    const int64_t rows_per_block = (threads / 32) * (32 / G);
    const unsigned grid = (unsigned)std::min<int64_t>((c->nne + rows_per_block - 1) / rows_per_block, 152 * 64);
    count_launch();
#define MVF_SPMM_ARGS \
    <<<grid, threads, 0, c->stream>>>(c->nne, c->d.rowptr, c->d.col, K, M, x, b, y, use_w32, (const SolveParams *)c->d.wsp)
    switch (v) {
        case 1:
            if constexpr (R <= 4) spmm_km_direct<T, TV, R> MVF_SPMM_ARGS;
            break;
        case 2:
            if constexpr (R <= 16) spmm_km_vec<T, TV, R, 4> MVF_SPMM_ARGS;
            break;
        case 3:
            if constexpr (R <= 16) spmm_km_vec<T, TV, R, 8> MVF_SPMM_ARGS;
            break;
        case 4:
            if constexpr (R <= 16) spmm_km_vec<T, TV, R, 16> MVF_SPMM_ARGS;
            break;
        case 5:
            if constexpr (R <= 16) spmm_km_vec<T, TV, R, 32> MVF_SPMM_ARGS;
            break;
        default: spmm_km<T, TV, R> MVF_SPMM_ARGS; break;
    }
#undef MVF_SPMM_ARGS
}

template <class T, class TV>
static void spmm_dispatch(Ctx *c, int v, int R, const T *K, const T *M, const TV *x, const TV *b, TV *y,
                          int use_w32) {
    switch (R) {
        case 1: spmm_variant<T, TV, 1>(c, v, K, M, x, b, y, use_w32); break;
        case 2: spmm_variant<T, TV, 2>(c, v, K, M, x, b, y, use_w32); break;
        case 4: spmm_variant<T, TV, 4>(c, v, K, M, x, b, y, use_w32); break;
        case 8: spmm_variant<T, TV, 8>(c, v, K, M, x, b, y, use_w32); break;
        case 16: spmm_variant<T, TV, 16>(c, v, K, M, x, b, y, use_w32); break;
        default: spmm_variant<T, TV, 32>(c, v, K, M, x, b, y, use_w32); break;
    }
}

// y = A x or b - A x.  The first product of a given precision and batch width on a
// context times every applicable variant on the real operands (one warm-up and three
// timed launches each, CUDA events on the context's stream) and keeps the fastest;
// y is simply rewritten by each trial (x and b are never aliased with y).  Inside a
// stream capture nothing is timed: the untuned default runs and the choice stays open.
template <class T, class TV>
static void launch_spmm(Ctx *c, int R, const T *K, const T *M, const TV *x, const TV *b, TV *y, int use_w32) {
    int li = 0;
    while ((1 << li) < R && li < 5) ++li;
    const int fp64 = sizeof(T) == 8;
    int &pick = c->spmm_pick[fp64][li];
    if (pick < 0) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        cudaStreamIsCapturing(c->stream, &cs);
        if (cs != cudaStreamCaptureStatusNone) {
            spmm_dispatch<T, TV>(c, R <= 4 ? 1 : 0, R, K, M, x, b, y, use_w32);
            return;
        }
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        int best = R <= 4 ? 1 : 0;
        float best_ms = 1e30f;
        char line[96];
        std::snprintf(line, sizeof line, "%s R=%d:", fp64 ? "fp64" : "fp32", R);
        c->spmm_note += line;
        if (cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess) {
            for (int v = 0; v < SPMM_VARIANTS; ++v) {
                if (!spmm_ok(v, R)) continue;
                spmm_dispatch<T, TV>(c, v, R, K, M, x, b, y, use_w32);
                cudaEventRecord(e0, c->stream);
                for (int t = 0; t < 3; ++t) spmm_dispatch<T, TV>(c, v, R, K, M, x, b, y, use_w32);
                cudaEventRecord(e1, c->stream);
                float ms = 0;
                if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) break;
                std::snprintf(line, sizeof line, " %s %.1f us,", spmm_names[v], (double)ms * 1e3 / 3);
                c->spmm_note += line;
                if (ms < best_ms) {
                    best_ms = ms;
                    best = v;
                }
            }
        }
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        pick = best;
        c->spmm_us[fp64][li] = best_ms * 1e3f / 3;
        std::snprintf(line, sizeof line, " pick %s; ", spmm_names[best]);
        c->spmm_note += line;
    }
    spmm_dispatch<T, TV>(c, pick, R, K, M, x, b, y, use_w32);
}

static unsigned grid_for(int64_t n) { return (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 32); }

// float-float operator of the FP64 Krylov path: split x, then y = (K + i w M) x
static void launch_spmm_ff(Ctx *c, const MatrixSet &S, int R, const double2 *x, double2 *y, float4 *xf) {
    const int64_t nv = (int64_t)c->nne * R;
    count_launch();
    split_vector<<<grid_for(nv), 256, 0, c->stream>>>(nv, x, xf);
    constexpr int G = 16;
    const int64_t rows_per_block = 8 * (32 / G);
    const unsigned grid = (unsigned)std::min<int64_t>((c->nne + rows_per_block - 1) / rows_per_block, 152 * 64);
    const SolveParams *sp = (const SolveParams *)c->d.wsp;
    count_launch();
    switch (R) {
        case 1: spmm_ff<1, G><<<grid, 256, 0, c->stream>>>(c->nne, c->d.rowptr, c->d.col, S.Kff, S.Mff, xf, y, sp, 1, 0); break;
        case 2: spmm_ff<2, G><<<grid, 256, 0, c->stream>>>(c->nne, c->d.rowptr, c->d.col, S.Kff, S.Mff, xf, y, sp, 2, 0); break;
        case 4: spmm_ff<4, G><<<grid, 256, 0, c->stream>>>(c->nne, c->d.rowptr, c->d.col, S.Kff, S.Mff, xf, y, sp, 4, 0); break;
        default:
            // R = 8, 16, 32: passes of 8 right-hand sides
            for (int r0 = 0; r0 < R; r0 += 8) {
                if (r0) count_launch();
                spmm_ff<8, G><<<grid, 256, 0, c->stream>>>(c->nne, c->d.rowptr, c->d.col, S.Kff, S.Mff, xf, y, sp, R, r0);
            }
            break;
    }
}

// K, M as FP32 halves for the float-float operator (once per matrix set)
static int ensure_split(Ctx *c, MatrixSet &S) {
    if (S.Kff) return 0;
    MVF_CUDA(c, cudaMalloc((void **)&S.Kff, c->nnz * sizeof(float2)));
    MVF_CUDA(c, cudaMalloc((void **)&S.Mff, c->nnz * sizeof(float2)));
    count_launch();
    split_values<<<grid_for(c->nnz), 256, 0, c->stream>>>(c->nnz, S.K64, S.Kff);
    count_launch();
    split_values<<<grid_for(c->nnz), 256, 0, c->stream>>>(c->nnz, S.M64, S.Mff);
    MVF_CUDA(c, cudaGetLastError());
    return 0;
}

// Orthogonalise w against V_0..V_{k-1} with W.passes classical Gram-Schmidt passes
// (FP64 projections), write the projections to W.hc[0..k) and ||w||^2 to W.nrm.
template <class TV>
static int cgs2(Ctx *c, Work &W, int k) {
    const int R = W.R;
    const TV *V = (const TV *)W.V;
    TV *w = (TV *)W.w;
    const int64_t vs = (int64_t)W.n * R;
    for (int pass = 0; pass < W.passes; ++pass) {
        const size_t sm = (size_t)k * R * sizeof(double2);
        count_launch();
        multidot<TV><<<W.nblocks, 256, sm, c->stream>>>(W.n, R, k, V, vs, w, W.partial);
        count_launch();
        reduce_partials<<<k * R, 256, 0, c->stream>>>(W.nblocks, k * R, W.partial, pass == 0 ? W.hc : W.htmp, 0);
        count_launch();
        axpy_multi<TV><<<grid_for(vs), 256, 0, c->stream>>>(W.n, R, k, V, vs, pass == 0 ? W.hc : W.htmp, w);
        if (pass == 1) {
            // hc += htmp
            count_launch();
            reduce_partials<<<k * R, 256, 0, c->stream>>>(1, k * R, W.htmp, W.hc, 1);
        }
    }
    count_launch();
    multidot<TV><<<W.nblocks, 256, (size_t)R * sizeof(double2), c->stream>>>(W.n, R, 1, w, vs, w, W.partial);
    count_launch();
    reduce_partials<<<R, 256, 0, c->stream>>>(W.nblocks, R, W.partial, W.nrm, 0);
    MVF_CUDA(c, cudaGetLastError());
    return 0;
}

template <class TV>
static void precondition(Ctx *c, Work &W, const TV *r, TV *z) {
    const int R = W.R;
    if constexpr (std::is_same<TV, double2>::value) {
        if (W.mg) {
            mg_apply(c, W.mg, r, z);
            return;
        }
    }
    if (W.pinvs) {
        patch_apply(c, W.pinvs, R, W.npol, W.nfi, r, z);
        return;
    }
    count_launch();
    grad_t<TV><<<grid_for((int64_t)c->ngn * R), 256, 0, c->stream>>>(c->ngn, R, c->d.gtrow, c->d.gtcol, c->d.gtval, r,
                                                                    W.pinv, (TV *)W.t);
    count_launch();
    apply_prec<TV><<<grid_for((int64_t)W.n * R), 256, 0, c->stream>>>(W.n, R, c->d.grow, c->d.gcol, c->d.gval, r,
                                                                     W.dinv, (const TV *)W.t, z);
}

// One FGMRES cycle (at most m iterations) on A d = rhs (Krylov precision TV) with
// initial guess 0, adding the correction to x (FP64, [n][R]).  Returns iterations.
template <class T>
static int fgmres_cycle(Ctx *c, Work &W, const MatrixSet &S, const typename C2<T>::V *rhs, double2 *x, double tol_abs_rel,
                        int &iters, std::vector<double> &est) {
    using TV = typename C2<T>::V;
    const int R = W.R, m = W.m;
    const int64_t vs = (int64_t)W.n * R;
    TV *V = (TV *)W.V, *Z = (TV *)W.Z, *w = (TV *)W.w;
    const T *K = std::is_same<T, float>::value ? (const T *)S.K32 : (const T *)S.K64;
    const T *M = std::is_same<T, float>::value ? (const T *)S.M32 : (const T *)S.M64;
    const int use_w32 = 1;
    // V0 = rhs / ||rhs||
    MVF_CUDA(c, cudaMemcpyAsync(w, rhs, W.vb, cudaMemcpyDeviceToDevice, c->stream));
    count_launch();
    multidot<TV><<<W.nblocks, 256, (size_t)R * sizeof(double2), c->stream>>>(W.n, R, 1, w, vs, w, W.partial);
    count_launch();
    reduce_partials<<<R, 256, 0, c->stream>>>(W.nblocks, R, W.partial, W.nrm, 0);
    count_launch();
    hessenberg_init<<<1, 32, 0, c->stream>>>(R, W.nrm, W.hs);
    count_launch();
    scale_into<TV><<<grid_for(vs), 256, 0, c->stream>>>(W.n, R, w, W.nrm, V);
    // one Arnoldi step: z_k = P v_k, w = A z_k, orthogonalise, v_{k+1} = w / ||w||
    auto step = [&](int k) -> int {
        precondition<TV>(c, W, V + k * vs, Z + k * vs);
        bool ff = false;
        if constexpr (std::is_same<T, double>::value) {
            if (W.xf) {
                launch_spmm_ff(c, S, R, Z + k * vs, w, W.xf);
                ff = true;
            }
        }
        if (!ff) launch_spmm<T, TV>(c, R, K, M, Z + k * vs, (const TV *)nullptr, w, use_w32);
        int rc = cgs2<TV>(c, W, k + 1);
        if (rc) return rc;
        count_launch();
        hessenberg_step<<<1, 32, 0, c->stream>>>(R, k, W.hc, W.nrm, W.hs);
        count_launch();
        scale_into<TV><<<grid_for(vs), 256, 0, c->stream>>>(W.n, R, w, W.nrm, V + (k + 1) * vs);
        return 0;
    };
    int k = 0;
    // blocks of GCH steps between residual checks; from the second cycle of a solve on
    // (the SpMM is tuned by then and every pointer is fixed) each block is captured
    // once as a CUDA graph and replayed, one launch instead of ~10 per step
    while (k < m) {
        const int k1 = std::min(k + Work::GCH, m), kb = k / Work::GCH;
        bool done = false;
        if (W.cycles > 0 && kb < Work::MAXB && k % Work::GCH == 0) {
            if (!W.blocks[kb]) {
                int64_t nk = 0;
                cudaGraph_t g = nullptr;
                if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
                    int rc = 0;
                    capture_tally() = &nk;  // counted at each replay instead
                    for (int kk = k; kk < k1 && !rc; ++kk) rc = step(kk);
                    capture_tally() = nullptr;
                    const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
                    if (e == cudaSuccess && !rc && g && cudaGraphInstantiate(&W.blocks[kb], g, 0) == cudaSuccess)
                        W.block_launches[kb] = nk;
                    else
                        W.blocks[kb] = nullptr;
                    if (g) cudaGraphDestroy(g);
                    cudaGetLastError();
                }
            }
            if (W.blocks[kb] && cudaGraphLaunch(W.blocks[kb], c->stream) == cudaSuccess) {
                launch_counter().fetch_add(W.block_launches[kb]);
                done = true;
            }
        }
        if (!done)
            for (int kk = k; kk < k1; ++kk)
                if (int rc = step(kk)) return rc;
        k = k1;
        // residual estimate after the block
        count_launch();
        hessenberg_est<<<1, 32, 0, c->stream>>>(R, k, W.hs, W.est);
        MVF_CUDA(c, cudaMemcpyAsync(est.data(), W.est, sizeof(double) * R, cudaMemcpyDeviceToHost, c->stream));
        MVF_CUDA(c, cudaStreamSynchronize(c->stream));
        bool all = true;
        for (int r = 0; r < R; ++r)
            if (est[r] > tol_abs_rel) all = false;
        if (all) break;
    }
    ++W.cycles;
    count_launch();
    hessenberg_solve<<<R, 32, 0, c->stream>>>(R, k, W.hs, W.y);
    count_launch();
    update_x<TV, double2><<<grid_for(vs), 256, 0, c->stream>>>(W.n, R, k, Z, vs, W.y, x, R, 0);
    MVF_CUDA(c, cudaGetLastError());
    iters += k;
    return 0;
}

static int residual_norms(Ctx *c, Work &W, const MatrixSet &S, std::vector<double> &rel, std::vector<double> &bn) {
    const int R = W.R;
    const int64_t vs = (int64_t)W.n * R;
    launch_spmm<double, double2>(c, R, S.K64, S.M64, W.x64, W.b64, W.r64, 1);
    count_launch();
    multidot<double2><<<W.nblocks, 256, (size_t)R * sizeof(double2), c->stream>>>(W.n, R, 1, W.r64, vs, W.r64, W.partial);
    count_launch();
    reduce_partials<<<R, 256, 0, c->stream>>>(W.nblocks, R, W.partial, W.nrm, 0);
    std::vector<double2> h(R);
    MVF_CUDA(c, cudaMemcpyAsync(h.data(), W.nrm, R * sizeof(double2), cudaMemcpyDeviceToHost, c->stream));
    MVF_CUDA(c, cudaStreamSynchronize(c->stream));
    for (int r = 0; r < R; ++r) rel[r] = bn[r] > 0 ? std::sqrt(std::max(h[r].x, 0.0)) / bn[r] : 0.0;
    return 0;
}

// Solve the R = 2*nf right-hand sides of one matrix set.
template <class T>
static int solve_set(Ctx *c, const MatrixSet &S, int f0, int nfs, int pol0, int npol, double tol, int max_iters,
                     mvf_stats *st, int m) {
    using TV = typename C2<T>::V;
    // the kernels map right-hand sides onto warp lanes: pad to a power of two with
    // zero right-hand sides (their Krylov sequences stay zero)
    const int Rreal = nfs * npol;
    int R = 1;
    while (R < Rreal) R <<= 1;
    Work W;
    int rc = alloc_work<T>(c, W, R, m);
    if (rc) { free_work(c, W); return rc; }
    // the FP32 inner solve sits inside FP64 refinement, which absorbs the loss of
    // orthogonality of a single pass; the plain FP64 method keeps two passes
    W.passes = std::is_same<T, float>::value ? c->mixed_passes : 2;
    W.npol = npol;
    W.nfi = nfs;
    if (c->use_patches) {
        std::vector<double> wl(nfs);
        for (int f = 0; f < nfs; ++f)
            wl[f] = (c->mesh.quirks & MVF_Q_FP32_CONST) ? (double)(float)c->omega[f0 + f] : c->omega[f0 + f];
        if (c->precond == 0)
            rc = mg_numeric(c, S, wl.data(), nfs, R, npol, &W.mg);
        else
            rc = patch_invert(c, S, wl.data(), nfs, &W.pinvs);
        if (rc) { free_work(c, W); return rc; }
        if (std::is_same<T, double>::value && c->solve_mode == 0 && c->patch_precision == 2) {
            MVF_CUDA(c, cudaMallocAsync((void **)&W.xf, (size_t)W.n * R * sizeof(float4), c->stream));
            if ((rc = ensure_split(c, const_cast<MatrixSet &>(S)))) { free_work(c, W); return rc; }
        }
    }
    SolveParams sp{};
    for (int r = 0; r < R; ++r) {
        const int f = f0 + std::min(r, Rreal - 1) / npol;
        sp.omega[r] = c->omega[f];
        sp.w32[r] = (c->mesh.quirks & MVF_Q_FP32_CONST) ? (double)(float)c->omega[f] : c->omega[f];
    }
    MVF_CUDA(c, cudaMemcpyAsync(c->d.wsp, &sp, sizeof sp, cudaMemcpyHostToDevice, c->stream));
    count_launch();
    extract_diag<<<grid_for(c->nne), 256, 0, c->stream>>>(c->nne, c->d.rowptr, c->d.col, S.K64, S.M64, W.kd, W.md);
    count_launch();
    build_inverse_diag<<<grid_for(((int64_t)c->nne + c->ngn) * R), 256, 0, c->stream>>>(
        c->nne, c->ngn, R, W.kd, W.md, S.kphi, S.mphi, S.mabs, W.dinv, W.pinv, (const SolveParams *)c->d.wsp);
    // gather right-hand sides [f][p][n] -> [n][R]
    if (npol == 2) {
        count_launch();
        gather_rhs<<<grid_for((int64_t)W.n * R), 256, 0, c->stream>>>(W.n, R, Rreal, f0, (const double2 *)c->d.rhs, W.b64);
    } else {
        // single rhs (f0, pol0)
        MVF_CUDA(c, cudaMemcpyAsync(W.b64, (const double2 *)c->d.rhs + ((int64_t)f0 * 2 + pol0) * W.n,
                                    (size_t)W.n * sizeof(double2), cudaMemcpyDeviceToDevice, c->stream));
    }
    MVF_CUDA(c, cudaMemsetAsync(W.x64, 0, (size_t)W.n * R * sizeof(double2), c->stream));
    if (c->d.guess && c->guess_nfreq == c->nfreq) {
        // initial guess (e.g. the learned warm start): refinement starts from b - A x0
        if (npol == 2) {
            count_launch();
            gather_rhs<<<grid_for((int64_t)W.n * R), 256, 0, c->stream>>>(W.n, R, Rreal, f0, (const double2 *)c->d.guess,
                                                                         W.x64);
        } else {
            MVF_CUDA(c, cudaMemcpyAsync(W.x64, (const double2 *)c->d.guess + ((int64_t)f0 * 2 + pol0) * W.n,
                                        (size_t)W.n * sizeof(double2), cudaMemcpyDeviceToDevice, c->stream));
        }
    }
    std::vector<double> bn(R, 1.0), rel(R, 0.0), est(R, 0.0);
    {
        const int64_t vs = (int64_t)W.n * R;
        count_launch();
        multidot<double2><<<W.nblocks, 256, (size_t)R * sizeof(double2), c->stream>>>(W.n, R, 1, W.b64, vs, W.b64, W.partial);
        count_launch();
        reduce_partials<<<R, 256, 0, c->stream>>>(W.nblocks, R, W.partial, W.nrm, 0);
        std::vector<double2> h(R);
        MVF_CUDA(c, cudaMemcpyAsync(h.data(), W.nrm, R * sizeof(double2), cudaMemcpyDeviceToHost, c->stream));
        MVF_CUDA(c, cudaStreamSynchronize(c->stream));
        for (int r = 0; r < R; ++r) bn[r] = std::sqrt(std::max(h[r].x, 0.0));
    }
    int iters = 0, outer = 0;
    const bool mixed = std::is_same<T, float>::value;
    double worst = 1.0;
    bool stagnated = false, have_best = false;
    double best = HUGE_VAL;
    std::vector<double> hist;
    std::vector<int> hist_it;  // inner iterations done at each entry of hist
    while (true) {
        if ((rc = residual_norms(c, W, S, rel, bn))) break;
        worst = 0;
        for (int r = 0; r < Rreal; ++r) worst = std::max(worst, rel[r]);
        hist.push_back(worst);
        hist_it.push_back(iters);
        // keep the best iterate; a refinement step that raises the true residual
        // tenfold above it means the inner solves have stopped helping (near-singular
        // air block): return the best iterate instead
        const size_t xb = (size_t)W.n * R * sizeof(double2);
        if (worst < best) {
            best = worst;
            if (worst > tol && iters < max_iters) {
                if (!W.xbest) MVF_CUDA(c, cudaMallocAsync((void **)&W.xbest, xb, c->stream));
                MVF_CUDA(c, cudaMemcpyAsync(W.xbest, W.x64, xb, cudaMemcpyDeviceToDevice, c->stream));
                have_best = true;
            }
        } else if (have_best && worst > 10.0 * best) {
            break;
        }
        if (worst <= tol || iters >= max_iters) break;
        // Residual floor: without a Dirichlet constraint on them, gradients of nodal
        // functions inside the air (Re(sigma) = 0) are in the kernel of A, and the
        // right-hand side carries a component there whenever the nodal sigma's
        // imaginary part differs from i*eps*omega (update_sigma refreshes only part of
        // the nodes, geometry.f90:144-153).  No solver reduces that component; the rest
        // of the residual, and the surface fields, converge.  Stop once 80 inner
        // iterations (at least two refinement steps) have not halved the true residual.
        if (worst < 1e-5 && hist.size() >= 3) {
            int j = -1;
            for (int q = (int)hist.size() - 3; q >= 0; --q)
                if (hist_it[q] <= iters - 80) { j = q; break; }
            if (j >= 0 && worst > 0.5 * hist[j]) {
                stagnated = true;
                break;
            }
        }
        ++outer;
        // inner solve on the residual in the Krylov precision, staged in V_m (the cycle
        // reads it into V_0 before V_m is overwritten)
        TV *stage = (TV *)W.V + (int64_t)W.m * W.n * R;
        count_launch();
        cast_vec<TV><<<grid_for((int64_t)W.n * R), 256, 0, c->stream>>>((int64_t)W.n * R, W.r64, stage, 1.0);
        const double inner_tol = mixed ? std::max(tol / std::max(worst, 1e-300), 2e-5) : tol / std::max(worst, 1e-300);
        if ((rc = fgmres_cycle<T>(c, W, S, stage, W.x64, inner_tol, iters, est))) break;
    }
    if (!rc && have_best && worst > best) {
        // the last refinement steps made things worse: hand back the best iterate
        MVF_CUDA(c, cudaMemcpyAsync(W.x64, W.xbest, (size_t)W.n * R * sizeof(double2), cudaMemcpyDeviceToDevice,
                                    c->stream));
        worst = best;
    }
    if (!rc) {
        if (npol == 2) {
            count_launch();
            scatter_sol<<<grid_for((int64_t)W.n * R), 256, 0, c->stream>>>(W.n, R, Rreal, f0, W.x64, (double2 *)c->d.x);
        } else
            MVF_CUDA(c, cudaMemcpyAsync((double2 *)c->d.x + ((int64_t)f0 * 2 + pol0) * W.n, W.x64,
                                        (size_t)W.n * sizeof(double2), cudaMemcpyDeviceToDevice, c->stream));
        MVF_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    if (st) {
        st->outer_iters = std::max(st->outer_iters, outer);
        st->inner_iters = std::max(st->inner_iters, iters);
        st->rel_residual = std::max(st->rel_residual, worst);
        if (stagnated) st->stagnated = 1;
    }
    free_work(c, W);
    if (!rc && worst > tol && !stagnated) return MVF_E_NOCONV;
    return rc;
}

}  // namespace mvf

using namespace mvf;

extern "C" int mvf_solve(mvf_ctx *xc, double *rhs_inout, double tol, int32_t mode, int32_t max_iters, mvf_stats *st) {
    if (!xc) return MVF_E_ARG;
    Ctx *c = &xc->c;
    if (!c->assembled) return fail(c, MVF_E_STATE, "assemble before solve");
    if (!(tol > 0) || max_iters < 1) return fail(c, MVF_E_ARG, "tol > 0 and max_iters >= 1 required");
    if (st) *st = mvf_stats{};
    c->solve_mode = mode;  // the plain FP64 mode keeps the patch preconditioner in FP64 too
    const size_t vb = (size_t)c->nfreq * 2 * c->nne * 2 * sizeof(double);
    if (rhs_inout) MVF_CUDA(c, cudaMemcpy(c->d.rhs, rhs_inout, vb, cudaMemcpyHostToDevice));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, c->stream);
    int rc = 0, noconv = 0;
    for (const MatrixSet &S : c->sets) {
        if (mode == 0) {
            // all frequencies of the set and both polarisations in one batch (or one
            // frequency per batch); complex FP32 Krylov vectors, except with the
            // preconditioners of the 36/54-DOF elements, which need FP64 vectors
            const int step = c->freq_batch == 1 ? 1 : S.nfreq;
            for (int f0 = S.first_freq; f0 < S.first_freq + S.nfreq && !rc; f0 += step) {
                const int nfs = std::min(step, S.first_freq + S.nfreq - f0);
                int r = c->use_patches ? solve_set<double>(c, S, f0, nfs, 0, 2, tol, max_iters, st, c->restart)
                                       : solve_set<float>(c, S, f0, nfs, 0, 2, tol, max_iters, st, c->restart);
                if (r == MVF_E_NOCONV) noconv = 1;
                else if (r) rc = r;
            }
            if (rc) break;
        } else {
            for (int f = S.first_freq; f < S.first_freq + S.nfreq && !rc; ++f)
                for (int p = 0; p < 2 && !rc; ++p) {
                    int r = solve_set<double>(c, S, f, 1, p, 1, tol, max_iters, st, c->restart);
                    if (r == MVF_E_NOCONV) noconv = 1;
                    else if (r) rc = r;
                }
        }
    }
    cudaEventRecord(e1, c->stream);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) st->seconds = ms * 1e-3;
    if (rc) return rc;
    if (rhs_inout) MVF_CUDA(c, cudaMemcpy(rhs_inout, c->d.x, vb, cudaMemcpyDeviceToHost));
    c->solved = true;
    if (noconv) return fail(c, MVF_E_NOCONV, "solver stopped at its iteration cap above tolerance");
    return 0;
}

// Many independent models at once: host threads take contexts from a queue (largest
// systems first) and run mvf_solve on each context's own stream, so the small solves
// of uneven models overlap on the GPU.  Work buffers are stream-ordered allocations
// and the solver keeps no state outside the context, so the solves do not serialise.
extern "C" int mvf_solve_many(mvf_ctx **ctx, int32_t n, double tol, int32_t mode, int32_t max_iters, mvf_stats *st,
                              int32_t nthreads) {
    if (!ctx || n < 1 || nthreads < 1) return MVF_E_ARG;
    for (int i = 0; i < n; ++i)
        if (!ctx[i]) return MVF_E_ARG;
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::sort(order.begin(), order.end(), [&](int a, int b) {
        return (int64_t)ctx[a]->c.nne * ctx[a]->c.nfreq > (int64_t)ctx[b]->c.nne * ctx[b]->c.nfreq;
    });
    std::vector<int> rc(n, 0);
    std::atomic<int> next{0};
#pragma omp parallel num_threads(nthreads)
    {
        for (;;) {
            const int k = next.fetch_add(1);
            if (k >= n) break;
            const int i = order[k];
            if (cudaSetDevice(ctx[i]->c.device) != cudaSuccess) {
                rc[i] = MVF_E_CUDA;
                continue;
            }
            rc[i] = mvf_solve(ctx[i], nullptr, tol, mode, max_iters, st ? &st[i] : nullptr);
        }
    }
    int noconv = 0;
    for (int i = 0; i < n; ++i) {
        if (rc[i] == MVF_E_NOCONV) noconv = 1;
        else if (rc[i]) return rc[i];
    }
    return noconv ? MVF_E_NOCONV : 0;
}

extern "C" int mvf_set_solver(mvf_ctx *xc, int32_t restart, int32_t mixed_passes, int32_t patch_precision) {
    if (!xc) return MVF_E_ARG;
    Ctx *c = &xc->c;
    if (restart != 0 && (restart < 2 || restart > MAXM)) return fail(c, MVF_E_ARG, "restart must be 2..256");
    if (mixed_passes != 0 && (mixed_passes < 1 || mixed_passes > 2)) return fail(c, MVF_E_ARG, "passes must be 1 or 2");
    if (patch_precision != 0 && patch_precision != 1 && patch_precision != 2)
        return fail(c, MVF_E_ARG, "patch precision must be 1 (FP64) or 2 (float-float)");
    if (restart) c->restart = restart;
    if (mixed_passes) c->mixed_passes = mixed_passes;
    if (patch_precision) c->patch_precision = patch_precision;
    return 0;
}

extern "C" int64_t mvf_kernel_launches(void) { return launch_counter().load(); }

extern "C" int mvf_set_batching(mvf_ctx *xc, int32_t per_frequency) {
    if (!xc || per_frequency < 0 || per_frequency > 1) return MVF_E_ARG;
    xc->c.freq_batch = per_frequency;
    return 0;
}

extern "C" int mvf_set_guess(mvf_ctx *xc, const double *x0) {
    if (!xc) return MVF_E_ARG;
    Ctx *c = &xc->c;
    if (!x0) {
        if (c->d.guess) cudaFree(c->d.guess);
        c->d.guess = nullptr;
        c->guess_nfreq = 0;
        return 0;
    }
    if (!c->assembled) return fail(c, MVF_E_STATE, "assemble before setting an initial guess");
    const size_t vb = (size_t)c->nfreq * 2 * c->nne * sizeof(double2);
    if (c->d.guess && c->guess_nfreq != c->nfreq) {
        cudaFree(c->d.guess);
        c->d.guess = nullptr;
    }
    if (!c->d.guess) MVF_CUDA(c, cudaMalloc((void **)&c->d.guess, vb));
    MVF_CUDA(c, cudaMemcpyAsync(c->d.guess, x0, vb, cudaMemcpyHostToDevice, c->stream));
    MVF_CUDA(c, cudaStreamSynchronize(c->stream));
    c->guess_nfreq = c->nfreq;
    return 0;
}

extern "C" const char *mvf_spmm_tuning(mvf_ctx *xc) { return xc ? xc->c.spmm_note.c_str() : ""; }

extern "C" int mvf_spmm_variant(mvf_ctx *xc, int32_t f, int32_t variant, int32_t fp64, int32_t R, const double *x,
                                double *y) {
    if (!xc || !x || !y) return MVF_E_ARG;
    Ctx *c = &xc->c;
    if (!c->assembled) return fail(c, MVF_E_STATE, "assemble first");
    if (f < 0 || f >= c->nfreq) return fail(c, MVF_E_ARG, "bad frequency");
    const bool ffv = variant == SPMM_VARIANTS;  // the float-float operator (FP64 vectors)
    if (R < 1 || R > MAXR || (R & (R - 1)) || variant < 0 || variant > SPMM_VARIANTS ||
        (!ffv && !spmm_ok(variant, R)) || (ffv && !fp64))
        return fail(c, MVF_E_ARG, "bad variant / right-hand-side count");
    const MatrixSet *S = nullptr;
    for (const MatrixSet &s : c->sets)
        if (f >= s.first_freq && f < s.first_freq + s.nfreq) S = &s;
    SolveParams sp{};
    for (int r = 0; r < R; ++r) {
        sp.omega[r] = c->omega[f];
        sp.w32[r] = (c->mesh.quirks & MVF_Q_FP32_CONST) ? (double)(float)c->omega[f] : c->omega[f];
    }
    MVF_CUDA(c, cudaMemcpyAsync(c->d.wsp, &sp, sizeof sp, cudaMemcpyHostToDevice, c->stream));
    const size_t nv = (size_t)c->nne * R;
    if (fp64) {
        double2 *dx, *dy;
        MVF_CUDA(c, cudaMalloc((void **)&dx, nv * sizeof(double2)));
        MVF_CUDA(c, cudaMalloc((void **)&dy, nv * sizeof(double2)));
        MVF_CUDA(c, cudaMemcpyAsync(dx, x, nv * sizeof(double2), cudaMemcpyHostToDevice, c->stream));
        if (ffv) {
            float4 *xf;
            if (int rc = ensure_split(c, const_cast<MatrixSet &>(*S))) return rc;
            MVF_CUDA(c, cudaMalloc((void **)&xf, nv * sizeof(float4)));
            launch_spmm_ff(c, *S, R, dx, dy, xf);
            MVF_CUDA(c, cudaStreamSynchronize(c->stream));
            cudaFree(xf);
        } else {
            spmm_dispatch<double, double2>(c, variant, R, S->K64, S->M64, dx, nullptr, dy, 1);
        }
        MVF_CUDA(c, cudaMemcpyAsync(y, dy, nv * sizeof(double2), cudaMemcpyDeviceToHost, c->stream));
        MVF_CUDA(c, cudaStreamSynchronize(c->stream));
        cudaFree(dx);
        cudaFree(dy);
    } else {
        std::vector<float2> hx(nv), hy(nv);
        for (size_t i = 0; i < nv; ++i) hx[i] = make_float2((float)x[2 * i], (float)x[2 * i + 1]);
        float2 *dx, *dy;
        MVF_CUDA(c, cudaMalloc((void **)&dx, nv * sizeof(float2)));
        MVF_CUDA(c, cudaMalloc((void **)&dy, nv * sizeof(float2)));
        MVF_CUDA(c, cudaMemcpyAsync(dx, hx.data(), nv * sizeof(float2), cudaMemcpyHostToDevice, c->stream));
        spmm_dispatch<float, float2>(c, variant, R, S->K32, S->M32, dx, nullptr, dy, 1);
        MVF_CUDA(c, cudaMemcpyAsync(hy.data(), dy, nv * sizeof(float2), cudaMemcpyDeviceToHost, c->stream));
        MVF_CUDA(c, cudaStreamSynchronize(c->stream));
        cudaFree(dx);
        cudaFree(dy);
        for (size_t i = 0; i < nv; ++i) {
            y[2 * i] = hy[i].x;
            y[2 * i + 1] = hy[i].y;
        }
    }
    MVF_CUDA(c, cudaGetLastError());
    return 0;
}

extern "C" int mvf_profile_spmm(mvf_ctx *xc, int32_t f, int32_t reps, double *sec_per_launch, int64_t *bytes) {
    if (!xc || !sec_per_launch || reps < 1) return MVF_E_ARG;
    Ctx *c = &xc->c;
    if (!c->assembled) return fail(c, MVF_E_STATE, "assemble first");
    if (f < 0 || f >= c->nfreq) return fail(c, MVF_E_ARG, "bad frequency");
    const MatrixSet *S = nullptr;
    for (const MatrixSet &s : c->sets)
        if (f >= s.first_freq && f < s.first_freq + s.nfreq) S = &s;
    int R = 1;
    while (R < 2 * S->nfreq) R <<= 1;
    SolveParams sp{};
    for (int r = 0; r < R; ++r) {
        const int ff = S->first_freq + std::min(r, 2 * S->nfreq - 1) / 2;
        sp.omega[r] = c->omega[ff];
        sp.w32[r] = (double)(float)c->omega[ff];
    }
    MVF_CUDA(c, cudaMemcpyAsync(c->d.wsp, &sp, sizeof sp, cudaMemcpyHostToDevice, c->stream));
    float2 *x, *y;
    const size_t nb = (size_t)c->nne * R * sizeof(float2);
    MVF_CUDA(c, cudaMalloc((void **)&x, nb));
    MVF_CUDA(c, cudaMalloc((void **)&y, nb));
    MVF_CUDA(c, cudaMemsetAsync(x, 0, nb, c->stream));
    launch_spmm<float, float2>(c, R, S->K32, S->M32, x, (const float2 *)nullptr, y, 1);  // warm
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, c->stream);
    for (int i = 0; i < reps; ++i) launch_spmm<float, float2>(c, R, S->K32, S->M32, x, (const float2 *)nullptr, y, 1);
    cudaEventRecord(e1, c->stream);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(x);
    cudaFree(y);
    MVF_CUDA(c, cudaGetLastError());
    *sec_per_launch = ms * 1e-3 / reps;
    // algorithmic bytes: K, M (FP32) and column index per nonzero, row pointers (int64),
    // x gathered once and y written once per right-hand side (complex64)
    if (bytes) *bytes = c->nnz * 12 + 8 * ((int64_t)c->nne + 1) + 2 * (int64_t)R * c->nne * 8;
    return 0;
}

extern "C" int mvf_spmv(mvf_ctx *xc, int32_t f, const double *x, double *y) {
    if (!xc || !x || !y) return MVF_E_ARG;
    Ctx *c = &xc->c;
    if (!c->assembled) return fail(c, MVF_E_STATE, "assemble first");
    if (f < 0 || f >= c->nfreq) return fail(c, MVF_E_ARG, "bad frequency");
    const MatrixSet *S = nullptr;
    for (const MatrixSet &s : c->sets)
        if (f >= s.first_freq && f < s.first_freq + s.nfreq) S = &s;
    SolveParams sp{};
    sp.omega[0] = sp.omega[1] = c->omega[f];
    sp.w32[0] = sp.w32[1] = (c->mesh.quirks & MVF_Q_FP32_CONST) ? (double)(float)c->omega[f] : c->omega[f];
    MVF_CUDA(c, cudaMemcpyAsync(c->d.wsp, &sp, sizeof sp, cudaMemcpyHostToDevice, c->stream));
    double2 *dx, *dy, *tx, *ty;
    const size_t nb = (size_t)c->nne * 2 * sizeof(double2);
    MVF_CUDA(c, cudaMalloc((void **)&dx, nb));
    MVF_CUDA(c, cudaMalloc((void **)&dy, nb));
    MVF_CUDA(c, cudaMalloc((void **)&tx, nb));
    MVF_CUDA(c, cudaMalloc((void **)&ty, nb));
    MVF_CUDA(c, cudaMemcpyAsync(dx, x, nb, cudaMemcpyHostToDevice, c->stream));
    count_launch();
    gather_rhs<<<grid_for((int64_t)c->nne * 2), 256, 0, c->stream>>>(c->nne, 2, 2, 0, dx, tx);
    launch_spmm<double, double2>(c, 2, S->K64, S->M64, tx, (const double2 *)nullptr, ty, 1);
    count_launch();
    scatter_sol<<<grid_for((int64_t)c->nne * 2), 256, 0, c->stream>>>(c->nne, 2, 2, 0, ty, dy);
    MVF_CUDA(c, cudaMemcpyAsync(y, dy, nb, cudaMemcpyDeviceToHost, c->stream));
    MVF_CUDA(c, cudaStreamSynchronize(c->stream));
    cudaFree(dx); cudaFree(dy); cudaFree(tx); cudaFree(ty);
    return 0;
}

extern "C" int mvf_export_rhs(const mvf_ctx *xc, int32_t f, double *rhs) {
    if (!xc || !rhs) return MVF_E_ARG;
    Ctx *c = const_cast<Ctx *>(&xc->c);
    if (!c->assembled) return fail(c, MVF_E_STATE, "assemble first");
    if (f < 0 || f >= c->nfreq) return fail(c, MVF_E_ARG, "bad frequency");
    MVF_CUDA(c, cudaMemcpy(rhs, c->d.rhs + (int64_t)f * 2 * c->nne * 2, (size_t)2 * c->nne * 2 * sizeof(double),
                           cudaMemcpyDeviceToHost));
    return 0;
}

// Lower-triangle COO of frequency f in row-major order (global_vfem's arrays before
// ga_sort_sparse).  drop: leave out the entries whose complex value is exactly zero and
// count them, as find_zeros / rem_zeros do before the MUMPS call
// (global_assembly.f90:123-150, MoVFEM_3DMT.f90:85-97); -0.0 counts as zero there too.
static int export_coo(Ctx *c, int32_t f, int32_t *ia, int32_t *ja, double *a, int64_t *nnz, int64_t *nzero,
                      bool drop) {
    if (!c->assembled) return fail(c, MVF_E_STATE, "assemble first");
    if (f < 0 || f >= c->nfreq) return fail(c, MVF_E_ARG, "bad frequency");
    const bool want = ia || ja || a;
    if (want && (!ia || !ja || !a)) return fail(c, MVF_E_ARG, "ia, ja and a must all be given");
    if (!drop && !want) {
        *nnz = c->nnz_lower;
        return 0;
    }
    const MatrixSet *S = nullptr;
    for (const MatrixSet &s : c->sets)
        if (f >= s.first_freq && f < s.first_freq + s.nfreq) S = &s;
    if (!S) return fail(c, MVF_E_STATE, "no matrix set holds this frequency");
    std::vector<int64_t> rp(c->nne + 1);
    std::vector<int32_t> cl(c->nnz);
    std::vector<double> K(c->nnz), M(c->nnz);
    MVF_CUDA(c, cudaMemcpy(rp.data(), c->d.rowptr, rp.size() * sizeof(int64_t), cudaMemcpyDeviceToHost));
    MVF_CUDA(c, cudaMemcpy(cl.data(), c->d.col, cl.size() * sizeof(int32_t), cudaMemcpyDeviceToHost));
    MVF_CUDA(c, cudaMemcpy(K.data(), S->K64, K.size() * sizeof(double), cudaMemcpyDeviceToHost));
    MVF_CUDA(c, cudaMemcpy(M.data(), S->M64, M.size() * sizeof(double), cudaMemcpyDeviceToHost));
    const double w32 = (c->mesh.quirks & MVF_Q_FP32_CONST) ? (double)(float)c->omega[f] : c->omega[f];
    int64_t q = 0, zeros = 0;
    for (int32_t r = 0; r < c->nne; ++r)
        for (int64_t k = rp[r]; k < rp[r + 1]; ++k) {
            if (cl[k] > r) continue;
            const double re = K[k], im = w32 * M[k];
            if (drop && re == 0.0 && im == 0.0) {
                ++zeros;
                continue;
            }
            if (want) {
                ia[q] = r + 1;
                ja[q] = cl[k] + 1;
                a[2 * q] = re;
                a[2 * q + 1] = im;
            }
            ++q;
        }
    *nnz = q;
    if (nzero) *nzero = zeros;
    return 0;
}

extern "C" int mvf_export_coo(const mvf_ctx *xc, int32_t f, int32_t *ia, int32_t *ja, double *a, int64_t *nnz) {
    if (!xc || !nnz) return MVF_E_ARG;
    return export_coo(const_cast<Ctx *>(&xc->c), f, ia, ja, a, nnz, nullptr, false);
}

extern "C" int mvf_export_coo_nz(const mvf_ctx *xc, int32_t f, int32_t *ia, int32_t *ja, double *a, int64_t *nnz,
                                 int64_t *nzero) {
    if (!xc || !nnz || !nzero) return MVF_E_ARG;
    return export_coo(const_cast<Ctx *>(&xc->c), f, ia, ja, a, nnz, nzero, true);
}
