// mvf_patch.cu -- vertex-patch additive Schwarz preconditioner for the 36- and 54-DOF
// elements.
//
// Point Jacobi (with or without a gradient correction) barely reduces the residual
// of the mixed-order quadratic and Lagrangian edge systems.  The preconditioner here
// is z = sum_v R_v^T A_v^-1 R_v r over the vertices v of the element grid, where R_v
// restricts to the DOFs whose elements all lie in the 2x2x2 block of elements around
// v (the Arnold-Falk-Winther patches for H(curl)); each block contains the local
// gradient modes, so the curl-curl kernel is handled inside the local solves.
// A_v depends on the frequency (A = K + i w M): the inverses are formed per frequency
// by Gauss-Jordan elimination with partial pivoting in FP64 (a relative shift of 1e-10
// of the largest diagonal entry keeps the patches that lie entirely in the air, where
// A_v is singular, invertible) and stored in complex FP64: those inverses carry large
// components along the air gradients, which complex64 cannot hold next to the rest.  Patches of one vertex-parity
// colour share no DOF, so the 8 colour launches accumulate z without atomics.
#include <algorithm>
#include <climits>
#include <cmath>
#include <vector>

#include "mvf_internal.cuh"

namespace mvf {

// Vertex patches of an element grid with numbering gne ([ne][me], 1-based, <= 0 for
// eliminated DOFs): a DOF lies in the patch of vertex v when every element that holds it
// lies in the 2x2x2 block of elements around v.  Patches are ordered by vertex-parity
// colour; empty ones are dropped.
void vertex_patches(int nx, int ny, int nz, int me, const std::vector<int32_t> &gne, int32_t n, PatchHost &out) {
    std::vector<int32_t> lo(3 * (size_t)n, INT32_MAX), hi(3 * (size_t)n, -1);
    for (int ie = 0; ie < nx; ++ie)
        for (int je = 0; je < ny; ++je)
            for (int ke = 0; ke < nz; ++ke) {
                const int64_t e = ((int64_t)ie * ny + je) * nz + ke;
                const int idx[3] = {ie, je, ke};
                for (int j = 0; j < me; ++j) {
                    const int32_t g = gne[(size_t)e * me + j];
                    if (g <= 0) continue;
                    for (int a = 0; a < 3; ++a) {
                        lo[3 * (size_t)(g - 1) + a] = std::min(lo[3 * (size_t)(g - 1) + a], idx[a]);
                        hi[3 * (size_t)(g - 1) + a] = std::max(hi[3 * (size_t)(g - 1) + a], idx[a]);
                    }
                }
            }
    // a DOF lies in the patch of vertex v when v-1 <= lo and hi <= v on every axis
    const int64_t nvx = nx + 1, nvy = ny + 1, nvz = nz + 1, nv = nvx * nvy * nvz;
    std::vector<int32_t> cnt(nv, 0);
    auto for_patches = [&](int32_t g, auto &&fn) {
        int a0[3], a1[3];
        for (int a = 0; a < 3; ++a) {
            a0[a] = hi[3 * (size_t)g + a];
            a1[a] = lo[3 * (size_t)g + a] + 1;
        }
        for (int vi = a0[0]; vi <= a1[0]; ++vi)
            for (int vj = a0[1]; vj <= a1[1]; ++vj)
                for (int vk = a0[2]; vk <= a1[2]; ++vk) fn(((int64_t)vi * nvy + vj) * nvz + vk);
    };
    for (int32_t g = 0; g < n; ++g) for_patches(g, [&](int64_t v) { cnt[v]++; });
    std::vector<int64_t> order;
    order.reserve(nv);
    out.color_off.assign(9, 0);
    for (int col = 0; col < 8; ++col) {
        out.color_off[col] = (int64_t)order.size();
        for (int64_t vi = col & 1; vi < nvx; vi += 2)
            for (int64_t vj = (col >> 1) & 1; vj < nvy; vj += 2)
                for (int64_t vk = (col >> 2) & 1; vk < nvz; vk += 2) {
                    const int64_t v = (vi * nvy + vj) * nvz + vk;
                    if (cnt[v] > 0) order.push_back(v);
                }
    }
    out.color_off[8] = (int64_t)order.size();
    const int64_t np = (int64_t)order.size();
    std::vector<int64_t> slot(nv, -1);
    for (int64_t p = 0; p < np; ++p) slot[order[p]] = p;
    out.ptr.assign(np + 1, 0);
    for (int64_t p = 0; p < np; ++p) out.ptr[p + 1] = out.ptr[p] + cnt[order[p]];
    out.dof.assign(out.ptr[np], 0);
    std::vector<int64_t> fill(out.ptr.begin(), out.ptr.end() - 1);
    for (int32_t g = 0; g < n; ++g) for_patches(g, [&](int64_t v) { out.dof[fill[slot[v]]++] = g; });
    out.pmax = 0;
    out.ioff.assign(np + 1, 0);
    for (int64_t p = 0; p < np; ++p) {
        const int sz = (int)(out.ptr[p + 1] - out.ptr[p]);
        out.pmax = std::max(out.pmax, sz);
        out.ioff[p + 1] = out.ioff[p] + (int64_t)sz * sz;
    }
}

// Build the patch lists of the context's own grid (host, once per context).
int patch_setup(Ctx *c) {
    PatchHost h;
    vertex_patches(c->mesh.nx, c->mesh.ny, c->mesh.nz, c->T.me, c->gne_h, c->nne, h);
    const int64_t np = (int64_t)h.ptr.size() - 1;
    c->pcolor_off = h.color_off;
    c->npatch = np;
    c->patch_max = h.pmax;
    c->patch_entries = h.ioff[np];
    c->patch_dofs = h.ptr[np];
    MVF_CUDA(c, cudaMalloc((void **)&c->d.patch_ptr, (np + 1) * sizeof(int64_t)));
    MVF_CUDA(c, cudaMalloc((void **)&c->d.patch_dof, std::max<int64_t>(h.ptr[np], 1) * sizeof(int32_t)));
    MVF_CUDA(c, cudaMalloc((void **)&c->d.patch_ioff, (np + 1) * sizeof(int64_t)));
    MVF_CUDA(c, cudaMemcpy(c->d.patch_ptr, h.ptr.data(), (np + 1) * sizeof(int64_t), cudaMemcpyHostToDevice));
    MVF_CUDA(c, cudaMemcpy(c->d.patch_dof, h.dof.data(), h.ptr[np] * sizeof(int32_t), cudaMemcpyHostToDevice));
    MVF_CUDA(c, cudaMemcpy(c->d.patch_ioff, h.ioff.data(), (np + 1) * sizeof(int64_t), cudaMemcpyHostToDevice));
    return 0;
}

// Gather A_v = K + i w M over the patch DOFs into ws (complex FP64, P x P row-major),
// invert it in place by Gauss-Jordan with partial pivoting and store the inverse as
// complex64.  One CTA per patch (grid-stride); ws is a per-CTA workspace.
__global__ void __launch_bounds__(256) patch_invert_kernel(
    int64_t np, const int64_t *__restrict__ pptr, const int32_t *__restrict__ pdof, const int64_t *__restrict__ ioff,
    const int64_t *__restrict__ rowptr, const int32_t *__restrict__ col, const double *__restrict__ K,
    const double *__restrict__ M, double w, double tau, int pmax, double2 *__restrict__ ws_all,
    double2 *__restrict__ inv, int *__restrict__ err) {
    __shared__ int piv_row;
    __shared__ double red_v[256];
    __shared__ int red_i[256];
    double2 *ws = ws_all + (size_t)blockIdx.x * pmax * pmax * 2;  // [P][2P]: A | I
    for (int64_t p = blockIdx.x; p < np; p += gridDim.x) {
        const int64_t b0 = pptr[p];
        const int P = (int)(pptr[p + 1] - b0);
        const int W2 = 2 * P;
        // gather
        for (int t = threadIdx.x; t < P * P; t += blockDim.x) {
            const int i = t / P, j = t % P;
            const int32_t gi = pdof[b0 + i], gj = pdof[b0 + j];
            int64_t lo = rowptr[gi], hi = rowptr[gi + 1] - 1;
            while (lo < hi) {
                const int64_t mid = (lo + hi) >> 1;
                if (col[mid] < gj) lo = mid + 1;
                else hi = mid;
            }
            double2 a = make_double2(0.0, 0.0);
            if (col[lo] == gj) a = make_double2(K[lo], w * M[lo]);
            ws[i * W2 + j] = a;
            ws[i * W2 + P + j] = make_double2(i == j ? 1.0 : 0.0, 0.0);
        }
        __syncthreads();
        // tau > 0: the regularised operator K + i w (M + tau diag K) of the multilevel
        // preconditioner; tau == 0: the operator as it is; tau < 0: a real shift of
        // 1e-10 of the largest diagonal modulus (the one-level preconditioner)
        if (tau > 0.0) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) ws[i * W2 + i].y += w * tau * ws[i * W2 + i].x;
        } else if (tau < 0.0 && threadIdx.x == 0) {
            double dmax = 0.0;
            for (int i = 0; i < P; ++i) dmax = fmax(dmax, hypot(ws[i * W2 + i].x, ws[i * W2 + i].y));
            const double s = 1e-10 * dmax;
            for (int i = 0; i < P; ++i) ws[i * W2 + i].x += s;
        }
        __syncthreads();
        for (int k = 0; k < P; ++k) {
            // pivot search over rows k..P-1 of column k
            double best = -1.0;
            int bi = k;
            for (int i = k + threadIdx.x; i < P; i += blockDim.x) {
                const double v = hypot(ws[i * W2 + k].x, ws[i * W2 + k].y);
                if (v > best) { best = v; bi = i; }
            }
            red_v[threadIdx.x] = best;
            red_i[threadIdx.x] = bi;
            __syncthreads();
            for (int o = blockDim.x / 2; o > 0; o >>= 1) {
                if (threadIdx.x < o && red_v[threadIdx.x + o] > red_v[threadIdx.x]) {
                    red_v[threadIdx.x] = red_v[threadIdx.x + o];
                    red_i[threadIdx.x] = red_i[threadIdx.x + o];
                }
                __syncthreads();
            }
            if (threadIdx.x == 0) {
                piv_row = red_i[0];
                if (!(red_v[0] > 0.0)) atomicExch(err, 1);
            }
            __syncthreads();
            const int pr = piv_row;
            if (pr != k)
                for (int j = threadIdx.x; j < W2; j += blockDim.x) {
                    const double2 t = ws[k * W2 + j];
                    ws[k * W2 + j] = ws[pr * W2 + j];
                    ws[pr * W2 + j] = t;
                }
            __syncthreads();
            // scale row k by 1/pivot
            const double2 pv = ws[k * W2 + k];
            const double s2 = pv.x * pv.x + pv.y * pv.y;
            const double2 ip = s2 > 0 ? make_double2(pv.x / s2, -pv.y / s2) : make_double2(0.0, 0.0);
            __syncthreads();
            for (int j = threadIdx.x; j < W2; j += blockDim.x) {
                const double2 a = ws[k * W2 + j];
                ws[k * W2 + j] = make_double2(a.x * ip.x - a.y * ip.y, a.x * ip.y + a.y * ip.x);
            }
            __syncthreads();
            // eliminate column k from every other row
            for (int t = threadIdx.x; t < P * W2; t += blockDim.x) {
                const int i = t / W2, j = t % W2;
                if (i == k || j == k) continue;
                const double2 f = ws[i * W2 + k];
                const double2 r = ws[k * W2 + j];
                ws[i * W2 + j].x -= f.x * r.x - f.y * r.y;
                ws[i * W2 + j].y -= f.x * r.y + f.y * r.x;
            }
            __syncthreads();
            for (int i = threadIdx.x; i < P; i += blockDim.x)
                if (i != k) ws[i * W2 + k] = make_double2(0.0, 0.0);
            __syncthreads();
        }
        double2 *out = inv + ioff[p];
        for (int t = threadIdx.x; t < P * P; t += blockDim.x) {
            const int i = t / P, j = t % P;
            out[t] = ws[i * W2 + P + j];
        }
        __syncthreads();
    }
}

// Inverses of the patches of one grid level for one frequency (see the kernel above).
void launch_patch_invert(cudaStream_t st, int grid, int64_t np, const int64_t *pptr, const int32_t *pdof,
                         const int64_t *ioff, const int64_t *rowptr, const int32_t *col, const double *K,
                         const double *M, double w, double tau, int pmax, double2 *ws, double2 *inv, int *err) {
    count_launch();
    patch_invert_kernel<<<grid, 256, 0, st>>>(np, pptr, pdof, ioff, rowptr, col, K, M, w, tau, pmax, ws, inv, err);
}

// z[dof][r] += A_v^-1 r[dof][r] for the patches [p0, p1) (one colour); the inverse of
// right-hand side r's frequency is inv + (r / npol) * entries.
template <class TV>
__global__ void __launch_bounds__(128) patch_apply_kernel(int64_t p0, int64_t p1, const int64_t *__restrict__ pptr,
                                                          const int32_t *__restrict__ pdof,
                                                          const int64_t *__restrict__ ioff,
                                                          const double2 *__restrict__ inv, int64_t fstride, int R,
                                                          int npol, int nfi, const TV *__restrict__ r,
                                                          TV *__restrict__ z) {
    extern __shared__ double2 rs[];  // [P][R]
    for (int64_t p = p0 + blockIdx.x; p < p1; p += gridDim.x) {
        const int64_t b0 = pptr[p];
        const int P = (int)(pptr[p + 1] - b0);
        for (int t = threadIdx.x; t < P * R; t += blockDim.x) {
            const int i = t / R, q = t % R;
            const TV v = r[(int64_t)pdof[b0 + i] * R + q];
            rs[t] = make_double2(v.x, v.y);
        }
        __syncthreads();
        const double2 *A = inv + ioff[p];
        for (int t = threadIdx.x; t < P * R; t += blockDim.x) {
            const int i = t / R, q = t % R;
            const double2 *Ai = A + (int64_t)min(q / npol, nfi - 1) * fstride + (int64_t)i * P;
            double sr = 0.0, si = 0.0;
            for (int j = 0; j < P; ++j) {
                const double2 a = Ai[j];
                const double2 x = rs[j * R + q];
                sr += a.x * x.x - a.y * x.y;
                si += a.x * x.y + a.y * x.x;
            }
            TV &o = z[(int64_t)pdof[b0 + i] * R + q];
            o.x += (decltype(o.x))sr;
            o.y += (decltype(o.y))si;
        }
        __syncthreads();
    }
}

// ---- float-float application ---------------------------------------------------
// GB300 runs FP64 at a small fraction of its FP32 rate, and the FP64 application above
// is bound by the FP64 pipe.  Here every inverse entry is held as an unevaluated sum
// hi + lo of two FP32 numbers (same 16 bytes per complex entry), the right-hand sides
// likewise, and the products and sums run on the FP32 pipe with error-free
// transformations (Dekker/Knuth: a product's rounding error by FMA, a sum's by TwoSum),
// accumulated as a compensated dot product: about as accurate as a sum in twice FP32's
// precision, against 24 bits for plain FP32 -- enough for inverses whose air-gradient
// components dwarf the rest.

// The inverses span many orders of magnitude (air patches, PML stretch), beyond what
// FP32 halves can hold.  Each patch's inverse is therefore stored scaled symmetrically,
// S = D^-1 A_v^-1 D^-1 with d_i = sqrt|A_v^-1_ii| (1 where that vanishes), and the
// application computes z_i = d_i sum_j S_ij (d_j r_j) with d in FP64.  *bad is set when
// a scaled entry is too large for FP32 halves (then the FP64 application is used).
__device__ __forceinline__ double patch_scale(const double2 *A, int P, int i) {
    const double2 v = A[(int64_t)i * P + i];
    const double m = sqrt(hypot(v.x, v.y));
    return m > 0.0 && m < 1e150 ? m : 1.0;
}

// one block per (patch, frequency), grid-stride over the patches
__global__ void scale_check(int64_t np, int nf, const int64_t *__restrict__ pptr, const int64_t *__restrict__ ioff,
                            int64_t ent, const double2 *__restrict__ inv, int *__restrict__ bad) {
    for (int64_t pf = blockIdx.x; pf < np * nf; pf += gridDim.x) {
        const int64_t p = pf % np, f = pf / np;
        const int P = (int)(pptr[p + 1] - pptr[p]);
        const double2 *A = inv + f * ent + ioff[p];
        for (int t = threadIdx.x; t < P * P; t += blockDim.x) {
            const int i = t / P, j = t % P;
            const double sc = patch_scale(A, P, i) * patch_scale(A, P, j);
            const double2 v = A[t];
            const double m = fmax(fabs(v.x), fabs(v.y)) / sc;
            if (!(m < 1e30)) atomicOr(bad, 1);
        }
    }
}

// in place: A_ij (double2) -> S_ij as float4 (re_hi, im_hi, re_lo, im_lo), same 16
// bytes; d into scale[f][patch dof].  The scales are read from the diagonal before any
// thread of the block overwrites it.
__global__ void scale_split(int64_t np, int nf, const int64_t *__restrict__ pptr, const int64_t *__restrict__ ioff,
                            int64_t ent, int64_t ndof, double2 *__restrict__ inv, double *__restrict__ scale) {
    extern __shared__ double dsc[];  // [P]
    for (int64_t pf = blockIdx.x; pf < np * nf; pf += gridDim.x) {
        const int64_t p = pf % np, f = pf / np;
        const int64_t b0 = pptr[p];
        const int P = (int)(pptr[p + 1] - b0);
        double2 *A = inv + f * ent + ioff[p];
        for (int i = threadIdx.x; i < P; i += blockDim.x) {
            dsc[i] = patch_scale(A, P, i);
            scale[f * ndof + b0 + i] = dsc[i];
        }
        __syncthreads();
        for (int t = threadIdx.x; t < P * P; t += blockDim.x) {
            const int i = t / P, j = t % P;
            const double sc = dsc[i] * dsc[j];
            const double2 v = A[t];
            // scaled entries below 1e-30 (the diagonal is 1) are dropped: FP32 halves
            // cannot hold them, and a preconditioner that differs by such terms only
            // changes FGMRES iteration counts -- the FP64 true residual decides
            double x = v.x / sc, y = v.y / sc;
            if (fabs(x) < 1e-30) x = 0.0;
            if (fabs(y) < 1e-30) y = 0.0;
            const float xh = __double2float_rn(x), yh = __double2float_rn(y);
            const float xl = __double2float_rn(x - (double)xh), yl = __double2float_rn(y - (double)yh);
            reinterpret_cast<float4 *>(A)[t] = make_float4(xh, yh, xl, yl);
        }
        __syncthreads();
    }
}

template <class TV>
__global__ void __launch_bounds__(128) patch_apply_ff_kernel(int64_t p0, int64_t p1, const int64_t *__restrict__ pptr,
                                                             const int32_t *__restrict__ pdof,
                                                             const int64_t *__restrict__ ioff,
                                                             const float4 *__restrict__ inv, int64_t fstride, int R,
                                                             int npol, int nfi, const double *__restrict__ scale,
                                                             int64_t ndof, const TV *__restrict__ r,
                                                             TV *__restrict__ z) {
    extern __shared__ float4 rsf[];  // [P][R]: (re_hi, im_hi, re_lo, im_lo) of d_j r_j
    for (int64_t p = p0 + blockIdx.x; p < p1; p += gridDim.x) {
        const int64_t b0 = pptr[p];
        const int P = (int)(pptr[p + 1] - b0);
        for (int t = threadIdx.x; t < P * R; t += blockDim.x) {
            const int i = t / R, q = t % R;
            const TV v = r[(int64_t)pdof[b0 + i] * R + q];
            const double d = scale[(int64_t)min(q / npol, nfi - 1) * ndof + b0 + i];
            const double vx = d * v.x, vy = d * v.y;
            const float xh = __double2float_rn(vx), yh = __double2float_rn(vy);
            rsf[t] = make_float4(xh, yh, __double2float_rn(vx - (double)xh), __double2float_rn(vy - (double)yh));
        }
        __syncthreads();
        const float4 *A = inv + ioff[p];
        for (int t = threadIdx.x; t < P * R; t += blockDim.x) {
            const int i = t / R, q = t % R;
            const float4 *Ai = A + (int64_t)min(q / npol, nfi - 1) * fstride + (int64_t)i * P;
            float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
            for (int j = 0; j < P; ++j) {
                const float4 a = Ai[j];
                const float4 x = rsf[j * R + q];
                // (a.re + i a.im)(x.re + i x.im)
                dot2_mac(rh, rl, a.x, a.z, x.x, x.z);
                dot2_mac(rh, rl, -a.y, -a.w, x.y, x.w);
                dot2_mac(ih, il, a.x, a.z, x.y, x.w);
                dot2_mac(ih, il, a.y, a.w, x.x, x.z);
            }
            const double d = scale[(int64_t)min(q / npol, nfi - 1) * ndof + b0 + i];
            TV &o = z[(int64_t)pdof[b0 + i] * R + q];
            o.x += (decltype(o.x))(d * ((double)rh + (double)rl));
            o.y += (decltype(o.y))(d * ((double)ih + (double)il));
        }
        __syncthreads();
    }
}

// Inverses for the frequencies w[0..nf) of matrix set S: inv[f][entries].
int patch_invert(Ctx *c, const MatrixSet &S, const double *w, int nf, double2 **inv_out) {
    double2 *inv = nullptr;
    const int64_t ent = c->patch_entries;
    // inverses [nf][entries], then room for the float-float scales [nf][patch dofs]
    MVF_CUDA(c, cudaMalloc((void **)&inv, std::max<int64_t>(ent * nf, 1) * sizeof(double2) +
                                              (size_t)nf * c->patch_dofs * sizeof(double)));
    const int grid = (int)std::min<int64_t>(c->npatch, 152 * 8);
    double2 *ws = nullptr;
    int *err = nullptr;
    MVF_CUDA(c, cudaMalloc((void **)&ws, (size_t)grid * c->patch_max * c->patch_max * 2 * sizeof(double2)));
    MVF_CUDA(c, cudaMalloc((void **)&err, sizeof(int)));
    MVF_CUDA(c, cudaMemsetAsync(err, 0, sizeof(int), c->stream));
    for (int f = 0; f < nf; ++f) {
        count_launch();
        patch_invert_kernel<<<grid, 256, 0, c->stream>>>(c->npatch, c->d.patch_ptr, c->d.patch_dof, c->d.patch_ioff,
                                                          c->d.rowptr, c->d.col, S.K64, S.M64, w[f], -1.0, c->patch_max, ws,
                                                          inv + (int64_t)f * ent, err);
    }
    MVF_CUDA(c, cudaGetLastError());
    int herr = 0;
    MVF_CUDA(c, cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MVF_CUDA(c, cudaStreamSynchronize(c->stream));
    cudaFree(ws);
    if (herr) {
        cudaFree(err);
        cudaFree(inv);
        return fail(c, MVF_E_SINGULAR, "zero pivot in a patch inverse");
    }
    c->patch_inv_split = 0;
    if (c->patch_precision == 2 && c->solve_mode == 0) {
        const unsigned g = (unsigned)std::min<int64_t>(c->npatch * nf, 152 * 16);
        int bad = 0;
        MVF_CUDA(c, cudaMemsetAsync(err, 0, sizeof(int), c->stream));
        count_launch();
        scale_check<<<g, 256, 0, c->stream>>>(c->npatch, nf, c->d.patch_ptr, c->d.patch_ioff, ent, inv, err);
        MVF_CUDA(c, cudaMemcpyAsync(&bad, err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        MVF_CUDA(c, cudaStreamSynchronize(c->stream));
        if (!bad) {
            count_launch();
            scale_split<<<g, 256, (size_t)c->patch_max * sizeof(double), c->stream>>>(
                c->npatch, nf, c->d.patch_ptr, c->d.patch_ioff, ent, c->patch_dofs, inv,
                reinterpret_cast<double *>(inv + ent * nf));
            MVF_CUDA(c, cudaGetLastError());
            c->patch_inv_split = 1;
        }
    }
    cudaFree(err);
    *inv_out = inv;
    return 0;
}

template <class TV>
static void apply_impl(Ctx *c, const double2 *inv, int R, int npol, int nfi, const TV *r, TV *z) {
    cudaMemsetAsync(z, 0, (size_t)c->nne * R * sizeof(TV), c->stream);
    const size_t sm = (size_t)c->patch_max * R * 16;  // double2 or float4 per (dof, rhs)
    const bool ff = c->patch_inv_split != 0;
    if (ff)
        cudaFuncSetAttribute(patch_apply_ff_kernel<TV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    else
        cudaFuncSetAttribute(patch_apply_kernel<TV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    for (int col = 0; col < 8; ++col) {
        const int64_t a = c->pcolor_off[col], b = c->pcolor_off[col + 1];
        if (b <= a) continue;
        const unsigned grid = (unsigned)std::min<int64_t>(b - a, 152 * 16);
        count_launch();
        if (ff)
            patch_apply_ff_kernel<TV><<<grid, 128, sm, c->stream>>>(
                a, b, c->d.patch_ptr, c->d.patch_dof, c->d.patch_ioff, reinterpret_cast<const float4 *>(inv),
                c->patch_entries, R, npol, nfi,
                reinterpret_cast<const double *>(inv + (int64_t)nfi * c->patch_entries), c->patch_dofs, r, z);
        else
            patch_apply_kernel<TV><<<grid, 128, sm, c->stream>>>(a, b, c->d.patch_ptr, c->d.patch_dof, c->d.patch_ioff,
                                                                 inv, c->patch_entries, R, npol, nfi, r, z);
    }
}

void patch_apply(Ctx *c, const double2 *inv, int R, int npol, int nfi, const float2 *r, float2 *z) {
    apply_impl<float2>(c, inv, R, npol, nfi, r, z);
}
void patch_apply(Ctx *c, const double2 *inv, int R, int npol, int nfi, const double2 *r, double2 *z) {
    apply_impl<double2>(c, inv, R, npol, nfi, r, z);
}

}  // namespace mvf

using namespace mvf;

// Measurement hook: one preconditioner application (memset + 8 colour launches) of
// frequency f's patch inverses on 2 right-hand sides in complex FP64, timed with CUDA
// events on the library's stream.  Algorithmic bytes per application: the inverses
// (16 B per entry), each patch's gather of r and scatter of z, and the zeroing of z.
extern "C" int mvf_profile_patch(mvf_ctx *xc, int32_t f, int32_t reps, double *sec_per_apply, int64_t *bytes) {
    if (!xc || !sec_per_apply || reps < 1) return MVF_E_ARG;
    Ctx *c = &xc->c;
    if (!c->assembled) return fail(c, MVF_E_STATE, "assemble first");
    if (!c->use_patches) return fail(c, MVF_E_UNSUPPORTED, "vertex patches serve the 36/54-DOF elements only");
    if (f < 0 || f >= c->nfreq) return fail(c, MVF_E_ARG, "bad frequency");
    const MatrixSet *S = nullptr;
    for (const MatrixSet &s : c->sets)
        if (f >= s.first_freq && f < s.first_freq + s.nfreq) S = &s;
    const double w = (c->mesh.quirks & MVF_Q_FP32_CONST) ? (double)(float)c->omega[f] : c->omega[f];
    double2 *inv = nullptr;
    c->solve_mode = 0;  // the arithmetic of the mixed mode's application
    if (int rc = patch_invert(c, *S, &w, 1, &inv)) return rc;
    const int R = 2;
    const size_t vb = (size_t)c->nne * R * sizeof(double2);
    double2 *r = nullptr, *z = nullptr;
    cudaError_t e = cudaMalloc((void **)&r, vb);
    if (e == cudaSuccess) e = cudaMalloc((void **)&z, vb);
    if (e == cudaSuccess) e = cudaMemsetAsync(r, 0, vb, c->stream);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float ms = 0.f;
    if (e == cudaSuccess) {
        patch_apply(c, inv, R, 2, 1, r, z);  // warm
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, c->stream);
        for (int i = 0; i < reps; ++i) patch_apply(c, inv, R, 2, 1, r, z);
        cudaEventRecord(e1, c->stream);
        e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    cudaFree(r);
    cudaFree(z);
    cudaFree(inv);
    if (e != cudaSuccess) return cuda_fail(c, e, "patch profile");
    *sec_per_apply = ms * 1e-3 / reps;
    if (bytes) *bytes = c->patch_entries * 16 + 2 * c->patch_dofs * R * 16 + (int64_t)c->nne * R * 16;
    return 0;
}

extern "C" int32_t mvf_patch_arithmetic(const mvf_ctx *xc) {
    if (!xc || !xc->c.use_patches) return 0;
    return xc->c.patch_inv_split ? 2 : 1;
}
