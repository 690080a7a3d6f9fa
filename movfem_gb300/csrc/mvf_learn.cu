// mvf_learn.cu -- the learned warm start: a small dilated 3-D convolutional operator
// on the cell grid of a model.  Input channels per cell describe the conductivity,
// the air, the depth and the frequency; output channels are the secondary field on
// the cell's edges (both polarisations, real and imaginary parts), from which the
// host averages a warm start for the Krylov solve.  No counterpart in the reference.
//
// Storage is BF16 for weights and activations, accumulation FP32; training keeps
// FP32 master weights and Adam moments and refreshes the BF16 copy after each
// update.  Activations are channels-last [x][y][z][c]; a KS^3 convolution with
// dilation d reads the zero-padded neighbours at offsets (t - KS/2) * d.  Every
// kernel here is deterministic: reductions run over fixed partitions in shared
// memory, never with atomics.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "mvf_internal.cuh"

namespace {

using bf16 = __nv_bfloat16;

struct Layer {
    int cin, cout, ks, dil, relu;
    int64_t woff, boff;  // offsets of the weights [ks^3][cin][cout] and the bias [cout]
};

__device__ __forceinline__ void tap_offset(int tap, int ks, int dil, int &di, int &dj, int &dk) {
    const int h = ks / 2;
    di = (tap / (ks * ks) - h) * dil;
    dj = ((tap / ks) % ks - h) * dil;
    dk = (tap % ks - h) * dil;
}

__global__ void to_bf16(int64_t n, const float *__restrict__ a, bf16 *__restrict__ b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = __float2bfloat16(a[i]);
}

// out[v][co] = bias[co] + sum_tap sum_ci in[v + off(tap)][ci] w[tap][ci][co] (ReLU optional);
// one thread per (voxel, output channel), output channels fastest (coalesced weights).
__global__ void conv_fwd(int X, int Y, int Z, int cin, int cout, int ks, int dil, const bf16 *__restrict__ in,
                         const bf16 *__restrict__ w, const float *__restrict__ bias, int relu, bf16 *__restrict__ out_bf,
                         float *__restrict__ out_f) {
    const int64_t V = (int64_t)X * Y * Z;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < V * cout;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int co = (int)(idx % cout);
        const int64_t v = idx / cout;
        const int k = (int)(v % Z), j = (int)((v / Z) % Y), i = (int)(v / ((int64_t)Z * Y));
        float acc = bias[co];
        const int nt = ks * ks * ks;
        for (int t = 0; t < nt; ++t) {
            int di, dj, dk;
            tap_offset(t, ks, dil, di, dj, dk);
            const int ii = i + di, jj = j + dj, kk = k + dk;
            if (ii < 0 || ii >= X || jj < 0 || jj >= Y || kk < 0 || kk >= Z) continue;
            const bf16 *ip = in + (((int64_t)ii * Y + jj) * Z + kk) * cin;
            const bf16 *wp = w + (int64_t)t * cin * cout + co;
            for (int ci = 0; ci < cin; ++ci) acc += __bfloat162float(ip[ci]) * __bfloat162float(wp[(int64_t)ci * cout]);
        }
        if (relu) acc = fmaxf(acc, 0.f);
        if (out_f) out_f[idx] = acc;
        if (out_bf) out_bf[idx] = __float2bfloat16(acc);
    }
}

// gin[u][ci] = sum_tap sum_co gpre[u - off(tap)][co] w[tap][ci][co], times the ReLU mask
// of the layer input (act[u][ci] > 0) when the input is a ReLU output.
__global__ void conv_bwd_data(int X, int Y, int Z, int cin, int cout, int ks, int dil, const float *__restrict__ gpre,
                              const bf16 *__restrict__ w, const bf16 *__restrict__ act, int mask, float *__restrict__ gin) {
    const int64_t V = (int64_t)X * Y * Z;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < V * cin;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int ci = (int)(idx % cin);
        const int64_t u = idx / cin;
        if (mask && !(__bfloat162float(act[idx]) > 0.f)) {
            gin[idx] = 0.f;
            continue;
        }
        const int k = (int)(u % Z), j = (int)((u / Z) % Y), i = (int)(u / ((int64_t)Z * Y));
        float acc = 0.f;
        const int nt = ks * ks * ks;
        for (int t = 0; t < nt; ++t) {
            int di, dj, dk;
            tap_offset(t, ks, dil, di, dj, dk);
            const int ii = i - di, jj = j - dj, kk = k - dk;
            if (ii < 0 || ii >= X || jj < 0 || jj >= Y || kk < 0 || kk >= Z) continue;
            const float *gp = gpre + (((int64_t)ii * Y + jj) * Z + kk) * cout;
            const bf16 *wp = w + ((int64_t)t * cin + ci) * cout;
            for (int co = 0; co < cout; ++co) acc += gp[co] * __bfloat162float(wp[co]);
        }
        gin[idx] = acc;
    }
}

// gw[tap][ci][co] = sum_v in[v + off(tap)][ci] gpre[v][co]: one block per (tap, ci);
// thread (co, part) sums voxels part, part + nparts, ... and the parts meet in shared
// memory in a fixed order.  One extra block (index nt * cin) forms the bias gradient
// sum_v gpre[v][co] the same way.
__global__ void conv_bwd_weight(int X, int Y, int Z, int cin, int cout, int ks, int dil, const bf16 *__restrict__ in,
                                const float *__restrict__ gpre, float *__restrict__ gw, float *__restrict__ gb) {
    extern __shared__ float red[];
    const int nparts = blockDim.x / cout;
    const int co = threadIdx.x % cout, part = threadIdx.x / cout;
    const int64_t V = (int64_t)X * Y * Z;
    const int nt = ks * ks * ks;
    const bool bias_block = blockIdx.x == (unsigned)(nt * cin);
    float acc = 0.f;
    if (part < nparts) {
        if (bias_block) {
            for (int64_t v = part; v < V; v += nparts) acc += gpre[v * cout + co];
        } else {
            const int t = blockIdx.x / cin, ci = blockIdx.x % cin;
            int di, dj, dk;
            tap_offset(t, ks, dil, di, dj, dk);
            for (int64_t v = part; v < V; v += nparts) {
                const int k = (int)(v % Z), j = (int)((v / Z) % Y), i = (int)(v / ((int64_t)Z * Y));
                const int ii = i + di, jj = j + dj, kk = k + dk;
                if (ii < 0 || ii >= X || jj < 0 || jj >= Y || kk < 0 || kk >= Z) continue;
                acc += __bfloat162float(in[(((int64_t)ii * Y + jj) * Z + kk) * cin + ci]) * gpre[v * cout + co];
            }
        }
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    if (part == 0) {
        float s = 0.f;
        for (int p = 0; p < nparts; ++p) s += red[p * cout + co];
        if (bias_block)
            gb[co] = s;
        else
            gw[(int64_t)blockIdx.x * cout + co] = s;
    }
}

// mean squared error over n values: per-block partial sums of (out - t)^2 and the
// gradient 2 (out - t) / n
__global__ void mse_grad(int64_t n, const float *__restrict__ out, const float *__restrict__ t, float *__restrict__ g,
                         float *__restrict__ partial) {
    __shared__ float s[256];
    float acc = 0.f;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float d = out[i] - t[i];
        acc += d * d;
        g[i] = 2.f * d / (float)n;
    }
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}

__global__ void adam_step(int64_t n, float *__restrict__ p, float *__restrict__ m, float *__restrict__ v,
                          const float *__restrict__ g, bf16 *__restrict__ pb, float lr, float b1, float b2, float c1,
                          float c2, float eps) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        p[i] = pi;
        pb[i] = __float2bfloat16(pi);
    }
}

unsigned grid1(int64_t n) { return (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 16); }

}  // namespace

struct mvf_net {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    std::vector<Layer> L;
    int cin = 0, cout = 0, maxc = 0;
    int64_t np = 0, adam_t = 0;
    float *master = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr;
    bf16 *wbf = nullptr;
    int64_t vcap = 0;
    std::vector<bf16 *> act;       // act[0] input, act[l + 1] output of layer l (BF16)
    float *out = nullptr;          // output of the last layer (FP32)
    float *g0 = nullptr, *g1 = nullptr;  // gradient ping-pong buffers [V][maxc]
    float *hin = nullptr, *target = nullptr, *partial = nullptr;
};

namespace {

int nfail(mvf_net *n, int code, const std::string &msg) {
    if (n) n->err = msg;
    return code;
}

#define NET_CUDA(n, call)                                                                        \
    do {                                                                                         \
        cudaError_t _e = (call);                                                                 \
        if (_e != cudaSuccess) return nfail((n), MVF_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)

void free_acts(mvf_net *n) {
    for (bf16 *a : n->act) cudaFree(a);
    n->act.clear();
    cudaFree(n->out);
    cudaFree(n->g0);
    cudaFree(n->g1);
    cudaFree(n->hin);
    cudaFree(n->target);
    n->out = n->g0 = n->g1 = n->hin = n->target = nullptr;
    n->vcap = 0;
}

int ensure(mvf_net *n, int64_t V) {
    if (V <= n->vcap) return 0;
    free_acts(n);
    n->act.assign(n->L.size() + 1, nullptr);
    NET_CUDA(n, cudaMalloc((void **)&n->act[0], V * n->cin * sizeof(bf16)));
    for (size_t l = 0; l < n->L.size(); ++l)
        NET_CUDA(n, cudaMalloc((void **)&n->act[l + 1], V * n->L[l].cout * sizeof(bf16)));
    NET_CUDA(n, cudaMalloc((void **)&n->out, V * n->cout * sizeof(float)));
    NET_CUDA(n, cudaMalloc((void **)&n->g0, V * n->maxc * sizeof(float)));
    NET_CUDA(n, cudaMalloc((void **)&n->g1, V * n->maxc * sizeof(float)));
    NET_CUDA(n, cudaMalloc((void **)&n->hin, V * n->cin * sizeof(float)));
    NET_CUDA(n, cudaMalloc((void **)&n->target, V * n->cout * sizeof(float)));
    n->vcap = V;
    return 0;
}

int forward(mvf_net *n, int X, int Y, int Z, const float *in_host) {
    const int64_t V = (int64_t)X * Y * Z;
    if (int rc = ensure(n, V)) return rc;
    NET_CUDA(n, cudaMemcpyAsync(n->hin, in_host, V * n->cin * sizeof(float), cudaMemcpyHostToDevice, n->stream));
    mvf::count_launch();
    to_bf16<<<grid1(V * n->cin), 256, 0, n->stream>>>(V * n->cin, n->hin, n->act[0]);
    for (size_t l = 0; l < n->L.size(); ++l) {
        const Layer &y = n->L[l];
        const bool last = l + 1 == n->L.size();
        mvf::count_launch();
        conv_fwd<<<grid1(V * y.cout), 256, 0, n->stream>>>(X, Y, Z, y.cin, y.cout, y.ks, y.dil, n->act[l], n->wbf + y.woff,
                                                           n->master + y.boff, y.relu, n->act[l + 1],
                                                           last ? n->out : nullptr);
    }
    NET_CUDA(n, cudaGetLastError());
    return 0;
}

// backward from d(loss)/d(out) in g0: parameter gradients into n->grad
int backward(mvf_net *n, int X, int Y, int Z) {
    const int64_t V = (int64_t)X * Y * Z;
    float *gpre = n->g0, *gnext = n->g1;
    for (int l = (int)n->L.size() - 1; l >= 0; --l) {
        const Layer &y = n->L[l];
        const int nt = y.ks * y.ks * y.ks;
        const int nparts = std::max(1, 256 / y.cout);
        const int threads = nparts * y.cout;
        mvf::count_launch();
        conv_bwd_weight<<<nt * y.cin + 1, threads, threads * sizeof(float), n->stream>>>(
            X, Y, Z, y.cin, y.cout, y.ks, y.dil, n->act[l], gpre, n->grad + y.woff, n->grad + y.boff);
        if (l > 0) {
            // the input of layer l is the ReLU output of layer l-1
            mvf::count_launch();
            conv_bwd_data<<<grid1(V * y.cin), 256, 0, n->stream>>>(X, Y, Z, y.cin, y.cout, y.ks, y.dil, gpre,
                                                                   n->wbf + y.woff, n->act[l], n->L[l - 1].relu, gnext);
            std::swap(gpre, gnext);
        }
    }
    NET_CUDA(n, cudaGetLastError());
    return 0;
}

int loss_grad(mvf_net *n, int64_t count, const float *target_host, float *loss) {
    NET_CUDA(n, cudaMemcpyAsync(n->target, target_host, count * sizeof(float), cudaMemcpyHostToDevice, n->stream));
    const unsigned nb = std::min<unsigned>(grid1(count), 256);
    mvf::count_launch();
    mse_grad<<<nb, 256, 0, n->stream>>>(count, n->out, n->target, n->g0, n->partial);
    std::vector<float> h(nb);
    NET_CUDA(n, cudaMemcpyAsync(h.data(), n->partial, nb * sizeof(float), cudaMemcpyDeviceToHost, n->stream));
    NET_CUDA(n, cudaStreamSynchronize(n->stream));
    double s = 0;
    for (float x : h) s += x;
    if (loss) *loss = (float)(s / (double)count);
    return 0;
}

bool dims_ok(int X, int Y, int Z) { return X > 0 && Y > 0 && Z > 0 && (int64_t)X * Y * Z <= (int64_t)1 << 26; }

}  // namespace

extern "C" {

int mvf_net_create(mvf_net **out, int32_t cin, int32_t width, int32_t cout, int32_t nconv, const int32_t *dilations,
                   uint64_t seed, int32_t device) {
    if (!out) return MVF_E_ARG;
    *out = nullptr;
    if (cin < 1 || width < 1 || cout < 1 || nconv < 1 || nconv > 16 || !dilations || width > 256 || cout > 256 ||
        cin > 256)
        return MVF_E_ARG;
    for (int l = 0; l < nconv; ++l)
        if (dilations[l] < 1 || dilations[l] > 16) return MVF_E_ARG;
    mvf_net *n = new mvf_net();
    n->device = device < 0 ? 0 : device;
    n->cin = cin;
    n->cout = cout;
    int64_t off = 0;
    int c = cin;
    for (int l = 0; l <= nconv; ++l) {
        Layer y{};
        y.cin = c;
        y.cout = l < nconv ? width : cout;
        y.ks = l < nconv ? 3 : 1;
        y.dil = l < nconv ? dilations[l] : 1;
        y.relu = l < nconv;
        y.woff = off;
        off += (int64_t)y.ks * y.ks * y.ks * y.cin * y.cout;
        y.boff = off;
        off += y.cout;
        n->L.push_back(y);
        c = y.cout;
    }
    n->np = off;
    n->maxc = std::max({cin, width, cout});
    // He-uniform weights from a splitmix64 stream, zero biases
    std::vector<float> p(off, 0.f);
    uint64_t s = seed;
    auto next = [&]() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    for (const Layer &y : n->L) {
        const double fan_in = (double)y.ks * y.ks * y.ks * y.cin;
        const double a = std::sqrt(6.0 / fan_in) * (y.relu ? 1.0 : 0.5);
        for (int64_t i = 0; i < (int64_t)y.ks * y.ks * y.ks * y.cin * y.cout; ++i)
            p[y.woff + i] = (float)((2.0 * next() - 1.0) * a);
    }
    cudaError_t e = cudaSetDevice(n->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc((void **)&n->master, off * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void **)&n->m, off * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void **)&n->v, off * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void **)&n->grad, off * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void **)&n->wbf, off * sizeof(bf16));
    if (e == cudaSuccess) e = cudaMalloc((void **)&n->partial, 256 * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(n->m, 0, off * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(n->v, 0, off * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(n->master, p.data(), off * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        to_bf16<<<grid1(off), 256, 0, n->stream>>>(off, n->master, n->wbf);
        e = cudaStreamSynchronize(n->stream);
    }
    *out = n;
    if (e != cudaSuccess) {
        n->err = std::string("network setup: ") + cudaGetErrorString(e);
        return MVF_E_CUDA;
    }
    return 0;
}

void mvf_net_destroy(mvf_net *n) {
    if (!n) return;
    cudaSetDevice(n->device);
    if (n->stream) cudaStreamSynchronize(n->stream);
    free_acts(n);
    cudaFree(n->master);
    cudaFree(n->m);
    cudaFree(n->v);
    cudaFree(n->grad);
    cudaFree(n->wbf);
    cudaFree(n->partial);
    if (n->stream) cudaStreamDestroy(n->stream);
    delete n;
}

const char *mvf_net_last_error(mvf_net *n) { return n ? n->err.c_str() : "null network"; }

int64_t mvf_net_num_params(mvf_net *n) { return n ? n->np : -1; }

int mvf_net_get_params(mvf_net *n, float *p) {
    if (!n || !p) return MVF_E_ARG;
    NET_CUDA(n, cudaSetDevice(n->device));
    NET_CUDA(n, cudaMemcpyAsync(p, n->master, n->np * sizeof(float), cudaMemcpyDeviceToHost, n->stream));
    NET_CUDA(n, cudaStreamSynchronize(n->stream));
    return 0;
}

int mvf_net_set_params(mvf_net *n, const float *p) {
    if (!n || !p) return MVF_E_ARG;
    NET_CUDA(n, cudaSetDevice(n->device));
    NET_CUDA(n, cudaMemcpyAsync(n->master, p, n->np * sizeof(float), cudaMemcpyHostToDevice, n->stream));
    to_bf16<<<grid1(n->np), 256, 0, n->stream>>>(n->np, n->master, n->wbf);
    NET_CUDA(n, cudaMemsetAsync(n->m, 0, n->np * sizeof(float), n->stream));
    NET_CUDA(n, cudaMemsetAsync(n->v, 0, n->np * sizeof(float), n->stream));
    n->adam_t = 0;
    NET_CUDA(n, cudaStreamSynchronize(n->stream));
    return 0;
}

int mvf_net_forward(mvf_net *n, int32_t X, int32_t Y, int32_t Z, const float *in, float *out) {
    if (!n || !in || !out || !dims_ok(X, Y, Z)) return nfail(n, MVF_E_ARG, "bad grid or buffers");
    NET_CUDA(n, cudaSetDevice(n->device));
    if (int rc = forward(n, X, Y, Z, in)) return rc;
    const int64_t V = (int64_t)X * Y * Z;
    NET_CUDA(n, cudaMemcpyAsync(out, n->out, V * n->cout * sizeof(float), cudaMemcpyDeviceToHost, n->stream));
    NET_CUDA(n, cudaStreamSynchronize(n->stream));
    return 0;
}

int mvf_net_gradients(mvf_net *n, int32_t X, int32_t Y, int32_t Z, const float *in, const float *target, float *loss,
                      float *grad) {
    if (!n || !in || !target || !grad || !dims_ok(X, Y, Z)) return nfail(n, MVF_E_ARG, "bad grid or buffers");
    NET_CUDA(n, cudaSetDevice(n->device));
    if (int rc = forward(n, X, Y, Z, in)) return rc;
    const int64_t V = (int64_t)X * Y * Z;
    if (int rc = loss_grad(n, V * n->cout, target, loss)) return rc;
    if (int rc = backward(n, X, Y, Z)) return rc;
    NET_CUDA(n, cudaMemcpyAsync(grad, n->grad, n->np * sizeof(float), cudaMemcpyDeviceToHost, n->stream));
    NET_CUDA(n, cudaStreamSynchronize(n->stream));
    return 0;
}

int mvf_net_train_step(mvf_net *n, int32_t X, int32_t Y, int32_t Z, const float *in, const float *target, float lr,
                       float *loss) {
    if (!n || !in || !target || !dims_ok(X, Y, Z) || !(lr > 0)) return nfail(n, MVF_E_ARG, "bad grid, buffers or lr");
    NET_CUDA(n, cudaSetDevice(n->device));
    if (int rc = forward(n, X, Y, Z, in)) return rc;
    const int64_t V = (int64_t)X * Y * Z;
    if (int rc = loss_grad(n, V * n->cout, target, loss)) return rc;
    if (int rc = backward(n, X, Y, Z)) return rc;
    const float b1 = 0.9f, b2 = 0.999f;
    ++n->adam_t;
    const float c1 = 1.f - std::pow(b1, (float)n->adam_t), c2 = 1.f - std::pow(b2, (float)n->adam_t);
    mvf::count_launch();
    adam_step<<<grid1(n->np), 256, 0, n->stream>>>(n->np, n->master, n->m, n->v, n->grad, n->wbf, lr, b1, b2, c1, c2,
                                                  1e-8f);
    NET_CUDA(n, cudaGetLastError());
    return 0;
}

}  // extern "C"
