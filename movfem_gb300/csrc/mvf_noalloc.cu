// mvf_noalloc.cu -- y = A_f x without any device allocation.
//
// mvf_spmv (the parity hook) stages the two polarisations in an interleaved
// [row][polarisation] layout in buffers it allocates on every call.  Some callers
// cannot let a library allocate: a host that has handed the whole device-memory
// budget to its own pool allocator (a Fortran or C++ solver framework that owns the
// device), where a cudaMalloc from inside the library would fail or fragment that
// pool.  mvf_spmv_noalloc does the same product with the staging buffers in a fixed,
// file-scope device array instead.
//
// Limits and sharing rules:
//  * at most MVF_NOALLOC_MAX_DOF free DOFs (the array holds two [nne][2] complex
//    FP64 vectors: 16 MiB, resident on every device that loads the library);
//  * all calls share the array; each call writes every word it reads before reading
//    it, so nothing carries over from the previous call, but two calls whose kernels
//    overlap on the GPU (different streams or contexts on one device) race on it;
//  * the kernels run on the library's own stream: the caller must have finished
//    writing x_dev (synchronise the stream or event that produced it) before the
//    call, and the call synchronises the library's stream before it returns, so y_dev
//    is complete when it does;
//  * the first call on a device looks up the array's device address (once per device,
//    with that device current) and caches it; a cudaDeviceReset after that first call
//    invalidates the cached address, so no device reset may follow it in the process.
#include <cstdio>
#include <mutex>

#include "mvf_internal.cuh"

#define MVF_NOALLOC_MAX_DOF (1 << 18)

namespace mvf {

static __device__ __align__(256) double2 g_noalloc_scratch[2 * 2 * MVF_NOALLOC_MAX_DOF];

// x [2][n] -> t [n][2]
__global__ void na_gather(int32_t n, const double2 *__restrict__ x, double2 *__restrict__ t) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < 2 * (int64_t)n;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = q >> 1;
        const int p = (int)(q & 1);
        t[q] = x[(int64_t)p * n + i];
    }
}

// u[row][p] = sum_k (K_k + i w M_k) t[col_k][p]; one warp per row, lanes split into
// two polarisation halves over the row's nonzeros
__global__ void __launch_bounds__(256) na_spmm(int32_t n, const int64_t *__restrict__ rowptr,
                                                const int32_t *__restrict__ col, const double *__restrict__ K,
                                                const double *__restrict__ M, double w,
                                                const double2 *__restrict__ t, double2 *__restrict__ u) {
    const int lane = threadIdx.x & 31, p = lane & 1, s = lane >> 1;
    for (int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; row < n;
         row += ((int64_t)gridDim.x * blockDim.x) >> 5) {
        double ar = 0, ai = 0, br = 0, bi = 0;
        for (int64_t k = rowptr[row] + s; k < rowptr[row + 1]; k += 16) {
            const double kv = K[k], mv = M[k];
            const double2 xv = t[(int64_t)col[k] * 2 + p];
            ar += kv * xv.x;
            ai += kv * xv.y;
            br += mv * xv.x;
            bi += mv * xv.y;
        }
        double yr = ar - w * bi, yi = ai + w * br;
        for (int o = 16; o >= 2; o >>= 1) {
            yr += __shfl_down_sync(0xffffffffu, yr, o);
            yi += __shfl_down_sync(0xffffffffu, yi, o);
        }
        if (s == 0) u[row * 2 + p] = make_double2(yr, yi);
    }
}

// u [n][2] -> y [2][n]
__global__ void na_scatter(int32_t n, const double2 *__restrict__ u, double2 *__restrict__ y) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < 2 * (int64_t)n;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = q >> 1;
        const int p = (int)(q & 1);
        y[(int64_t)p * n + i] = u[q];
    }
}

// device address of the scratch array, looked up once per device
static std::mutex g_na_mu;
static double2 *g_na_addr[64] = {nullptr};

static int scratch_for(Ctx *c, double2 **out) {
    if (c->device < 0 || c->device >= 64) return fail(c, MVF_E_ARG, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (!g_na_addr[c->device]) {
        int cur = 0;
        MVF_CUDA(c, cudaGetDevice(&cur));
        if (cur != c->device) MVF_CUDA(c, cudaSetDevice(c->device));
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (cur != c->device) cudaSetDevice(cur);
        if (e != cudaSuccess) return cuda_fail(c, e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_na_addr[c->device] = (double2 *)p;
    }
    *out = g_na_addr[c->device];
    return 0;
}

}  // namespace mvf

using namespace mvf;

extern "C" int mvf_spmv_noalloc(mvf_ctx *xc, int32_t f, const double *x_dev, double *y_dev) {
    if (!xc || !x_dev || !y_dev) return MVF_E_ARG;
    Ctx *c = &xc->c;
    if (!c->assembled) return fail(c, MVF_E_STATE, "assemble first");
    if (f < 0 || f >= c->nfreq) return fail(c, MVF_E_ARG, "bad frequency");
    if (c->nne > MVF_NOALLOC_MAX_DOF)
        return fail(c, MVF_E_ARG, "mvf_spmv_noalloc handles at most 262144 free DOFs; this model has " +
                                      std::to_string(c->nne));
    const MatrixSet *S = nullptr;
    for (const MatrixSet &s : c->sets)
        if (f >= s.first_freq && f < s.first_freq + s.nfreq) S = &s;
    if (!S) return fail(c, MVF_E_STATE, "no assembled matrix set holds this frequency");
    if (c->nne == 0) return 0;
    double2 *scratch = nullptr;
    int rc = scratch_for(c, &scratch);
    if (rc) return rc;
    double2 *t = scratch, *u = scratch + 2 * (size_t)MVF_NOALLOC_MAX_DOF;
    const double w = (c->mesh.quirks & MVF_Q_FP32_CONST) ? (double)(float)c->omega[f] : c->omega[f];
    const unsigned g1 = (unsigned)std::min<int64_t>((2 * (int64_t)c->nne + 255) / 256, 152 * 32);
    const unsigned g2 = (unsigned)std::min<int64_t>(((int64_t)c->nne + 7) / 8, 152 * 64);
    count_launch();
    na_gather<<<g1, 256, 0, c->stream>>>(c->nne, (const double2 *)x_dev, t);
    count_launch();
    na_spmm<<<g2, 256, 0, c->stream>>>(c->nne, c->d.rowptr, c->d.col, S->K64, S->M64, w, t, u);
    count_launch();
    na_scatter<<<g1, 256, 0, c->stream>>>(c->nne, u, (double2 *)y_dev);
    MVF_CUDA(c, cudaGetLastError());
    MVF_CUDA(c, cudaStreamSynchronize(c->stream));
    return 0;
}
