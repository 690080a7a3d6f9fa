// mvf_surface.cu -- the surface gradient correction of the multilevel preconditioner.
//
// Just above the earth's surface the reference's quadratic interpolation of the nodal
// conductivity (problem.f90:132-149; earth value at the surface nodes, 0 in the air
// above) dips below zero: sigma(zeta) = sigma_e zeta (zeta - 1) / 2 inside the first air
// cells, down to -sigma_e / 8.  The true A = K + i w M is therefore indefinite on the
// gradients of those cells, while the multilevel method works on a positive
// semidefinite mass (mvf_mg.cu), which flips their sign: FGMRES then converges slowly
// however well the V-cycle approximates its operator.  After each V-cycle this stage
// solves those gradient modes exactly with the true operator:
//
//     z += G_s (G_s^T A G_s)^-1 G_s^T (r - A z),
//
// G_s the discrete gradients (the element table T.G) of the grid nodes from one node
// layer below the surface to the top of the first air cells.  G_s^T K G_s = 0 (the
// gradients are in the kernel of the discrete curl), so G_s^T A G_s = i w N with the
// real symmetric N = G_s^T M G_s of the matrix set: one factorisation serves every
// frequency of the set.  N is a thin, quasi-two-dimensional nodal system, indefinite
// (positive below the surface, negative above), which local or iterative solvers do not
// handle; it is factorised once per assembled matrix set as a band matrix (natural grid
// order, LU with partial pivoting) on the host CPU, and every application solves it
// there between two device stages: the device forms r - A z and G_s^T of it, the host
// solves the band system for each right-hand side (one OpenMP thread per real vector),
// the device adds G_s times the result.  The host step is a host node of the stream
// (cudaLaunchHostFunc on pinned buffers), so the stage can sit inside the captured
// Arnoldi graphs.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <memory>
#include <vector>

#include "mvf_internal.cuh"

namespace mvf {

// ------------------------------------------------------------------ band LU (host)
struct BandLU {
    int64_t n = 0;
    int kl = 0, ku = 0, ldab = 0;
    std::vector<double> ab;  // column-major band, ldab = 2 kl + ku + 1 (kl rows of fill)
    std::vector<int32_t> ipiv;

    double &at(int64_t i, int64_t j) { return ab[(size_t)j * ldab + (size_t)(kl + ku + i - j)]; }
    double at(int64_t i, int64_t j) const { return ab[(size_t)j * ldab + (size_t)(kl + ku + i - j)]; }

    void init(int64_t n_, int kl_, int ku_) {
        n = n_;
        kl = kl_;
        ku = ku_;
        ldab = 2 * kl + ku + 1;
        ab.assign((size_t)n * ldab, 0.0);
        ipiv.assign(n, 0);
    }
    // unblocked band LU with row interchanges; false on an exactly zero pivot column
    bool factor() {
        int64_t ju = 0;
        for (int64_t j = 0; j < n; ++j) {
            const int64_t km = std::min<int64_t>(kl, n - 1 - j);
            int64_t jp = 0;
            double amax = std::fabs(at(j, j));
            for (int64_t i = 1; i <= km; ++i) {
                const double v = std::fabs(at(j + i, j));
                if (v > amax) {
                    amax = v;
                    jp = i;
                }
            }
            ipiv[j] = (int32_t)(j + jp);
            if (amax == 0.0) return false;
            ju = std::max<int64_t>(ju, std::min<int64_t>(j + ku + jp, n - 1));
            if (jp != 0)
                for (int64_t c = j; c <= ju; ++c) std::swap(at(j, c), at(j + jp, c));
            const double piv = at(j, j);
            for (int64_t i = 1; i <= km; ++i) at(j + i, j) /= piv;
            const int64_t ncol = ju - j;
#pragma omp parallel for schedule(static) if (ncol * km > 32768)
            for (int64_t c = j + 1; c <= ju; ++c) {
                const double t = at(j, c);
                if (t == 0.0) continue;
                for (int64_t i = 1; i <= km; ++i) at(j + i, c) -= at(j + i, j) * t;
            }
        }
        return true;
    }
    void solve(double *b) const {
        const int64_t kv = kl + ku;
        for (int64_t j = 0; j + 1 < n; ++j) {
            const int64_t km = std::min<int64_t>(kl, n - 1 - j);
            const int64_t l = ipiv[j];
            if (l != j) std::swap(b[l], b[j]);
            const double t = b[j];
            if (t != 0.0)
                for (int64_t i = 1; i <= km; ++i) b[j + i] -= at(j + i, j) * t;
        }
        for (int64_t j = n - 1; j >= 0; --j) {
            b[j] /= at(j, j);
            const double t = b[j];
            if (t == 0.0) continue;
            for (int64_t i = std::max<int64_t>(0, j - kv); i < j; ++i) b[i] -= at(i, j) * t;
        }
    }
};

struct Surface {
    int64_t ns = 0;  // slab nodes
    // G_s: rows = free DOFs (CSR over all nne rows), columns = slab nodes; and G_s^T
    std::vector<int64_t> gptr, tptr;
    std::vector<int32_t> gcol, tcol;
    std::vector<double> gval, tval;
    int64_t *d_gptr = nullptr, *d_tptr = nullptr;
    int32_t *d_gcol = nullptr, *d_tcol = nullptr;
    double *d_gval = nullptr, *d_tval = nullptr;
    // host copy of the CSR pattern, for G_s^T M G_s
    std::vector<int64_t> rowptr;
    std::vector<int32_t> col;
    // factors per matrix set of the current assembly (heap-held: jobs keep pointers)
    struct Entry {
        const double *M64 = nullptr;
        uint64_t gen = 0;
        std::unique_ptr<BandLU> lu;
    };
    std::vector<Entry> cache;
};

struct SurfJob {
    const BandLU *lu = nullptr;
    int64_t ns = 0;
    int R = 0;
    std::vector<double> w;            // [R] angular frequency of each right-hand side
    double2 *h_in = nullptr, *h_out = nullptr;  // pinned [ns][R]
    double2 *d_ys = nullptr, *d_y = nullptr;    // device [ns][R]
};

// ------------------------------------------------------------------ kernels
// t = r - (K + i w_q M) z, the true operator (FP64)
__global__ void surf_resid(int32_t n, const int64_t *__restrict__ rowptr, const int32_t *__restrict__ col,
                           const double *__restrict__ K, const double *__restrict__ M, const double *__restrict__ wq,
                           int R, const double2 *__restrict__ r, const double2 *__restrict__ z,
                           double2 *__restrict__ t) {
    const int64_t nt = (int64_t)n * R;
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < nt; u += (int64_t)gridDim.x * blockDim.x) {
        const int32_t g = (int32_t)(u / R);
        const int q = (int)(u % R);
        const double w = wq[q];
        double2 acc = r[u];
        for (int64_t k = rowptr[g]; k < rowptr[g + 1]; ++k) {
            const double2 zv = z[(int64_t)col[k] * R + q];
            const double kv = K[k], mv = w * M[k];
            acc.x -= kv * zv.x - mv * zv.y;
            acc.y -= kv * zv.y + mv * zv.x;
        }
        t[u] = acc;
    }
}

// y[a][q] = sum over row a of G_s^T of coefficient * t[dof][q]
__global__ void surf_gather(int64_t ns, int R, const int64_t *__restrict__ tptr, const int32_t *__restrict__ tcol,
                            const double *__restrict__ tval, const double2 *__restrict__ t, double2 *__restrict__ y) {
    const int64_t nt = ns * R;
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < nt; u += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = u / R;
        const int q = (int)(u % R);
        double2 s = make_double2(0.0, 0.0);
        for (int64_t k = tptr[a]; k < tptr[a + 1]; ++k) {
            const double2 v = t[(int64_t)tcol[k] * R + q];
            s.x += tval[k] * v.x;
            s.y += tval[k] * v.y;
        }
        y[u] = s;
    }
}

// z[i][q] += sum over row i of G_s of coefficient * s[node][q]
__global__ void surf_scatter(int32_t n, int R, const int64_t *__restrict__ gptr, const int32_t *__restrict__ gcol,
                             const double *__restrict__ gval, const double2 *__restrict__ s, double2 *__restrict__ z) {
    const int64_t nt = (int64_t)n * R;
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < nt; u += (int64_t)gridDim.x * blockDim.x) {
        const int32_t i = (int32_t)(u / R);
        const int q = (int)(u % R);
        const int64_t k0 = gptr[i], k1 = gptr[i + 1];
        if (k0 == k1) continue;
        double2 acc = z[u];
        for (int64_t k = k0; k < k1; ++k) {
            const double2 v = s[(int64_t)gcol[k] * R + q];
            acc.x += gval[k] * v.x;
            acc.y += gval[k] * v.y;
        }
        z[u] = acc;
    }
}

static unsigned grid_of(int64_t n) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 32));
}

// the host step: for every right-hand side q, (i w_q N) s = y, i.e. s = -i N^-1 y / w_q;
// with u = N^-1 y: Re s = Im u / w_q, Im s = -Re u / w_q
static void CUDART_CB surf_host(void *p) {
    SurfJob *J = (SurfJob *)p;
    const int64_t n = J->ns;
    const int R = J->R;
#pragma omp parallel for schedule(dynamic, 1)
    for (int v = 0; v < 2 * R; ++v) {
        const int q = v >> 1, part = v & 1;
        std::vector<double> b(n);
        for (int64_t a = 0; a < n; ++a) b[a] = part ? J->h_in[a * R + q].y : J->h_in[a * R + q].x;
        J->lu->solve(b.data());
        const double w = J->w[q];
        if (part)
            for (int64_t a = 0; a < n; ++a) J->h_out[a * R + q].x = b[a] / w;
        else
            for (int64_t a = 0; a < n; ++a) J->h_out[a * R + q].y = -b[a] / w;
    }
}

// ------------------------------------------------------------------ setup
int surf_setup(Ctx *c) {
    if (c->surf) return 0;
    const OrderTables &T = c->T;
    const int me = T.me, mn = T.mn, o = T.nord - 1;
    const int64_t ksurf = (int64_t)o * (c->mesh.nz - c->mesh.nzl_air - c->mesh.nzl_top);
    if (ksurf - 1 < 0 || ksurf + o > c->nnz_nodes - 1)
        return fail(c, MVF_E_ARG, "surface correction: no earth surface inside the grid (nzl_air, nzl_top)");
    auto in_slab = [&](int64_t id) {
        const int64_t i = id / (c->nny * c->nnz_nodes), j = (id / c->nnz_nodes) % c->nny, k = id % c->nnz_nodes;
        if (k < ksurf - 1 || k > ksurf + o) return false;
        if (c->mesh.dirichlet && (i == 0 || j == 0 || k == 0 || i == c->nnx - 1 || j == c->nny - 1 ||
                                  k == c->nnz_nodes - 1))
            return false;
        return true;
    };
    // entries (row, grid node, coefficient), each DOF row taken from its first element
    std::vector<char> row_done(c->nne, 0);
    std::vector<std::vector<std::pair<int64_t, double>>> rows(c->nne);
    std::vector<char> used(c->npt, 0);
    for (int ie = 0; ie < c->mesh.nx; ++ie)
        for (int je = 0; je < c->mesh.ny; ++je)
            for (int ke = 0; ke < c->mesh.nz; ++ke) {
                const int64_t e = ((int64_t)ie * c->mesh.ny + je) * c->mesh.nz + ke;
                int64_t nodes[MVF_MAX_NODES];
                for (int l = 0; l < mn; ++l) nodes[l] = element_node(*c, ie, je, ke, l);
                for (int j = 0; j < me; ++j) {
                    const int32_t g = c->gne_h[(size_t)e * me + j];
                    if (g <= 0 || row_done[g - 1]) continue;
                    row_done[g - 1] = 1;
                    for (int l = 0; l < mn; ++l) {
                        if (T.G[j][l] == 0.0 || !in_slab(nodes[l])) continue;
                        used[nodes[l]] = 1;
                        rows[g - 1].push_back({nodes[l], T.G[j][l]});
                    }
                }
            }
    // slab nodes numbered in grid order (the band ordering)
    std::vector<int64_t> sidx(c->npt, -1);
    int64_t ns = 0;
    for (int64_t id = 0; id < c->npt; ++id)
        if (used[id]) sidx[id] = ns++;
    if (ns == 0) return fail(c, MVF_E_ARG, "surface correction: no gradient nodes in the surface layers");
    Surface *S = new Surface();
    S->ns = ns;
    S->gptr.assign(c->nne + 1, 0);
    S->tptr.assign(ns + 1, 0);
    for (int32_t r = 0; r < c->nne; ++r) S->gptr[r + 1] = S->gptr[r] + (int64_t)rows[r].size();
    S->gcol.resize(S->gptr[c->nne]);
    S->gval.resize(S->gptr[c->nne]);
    for (int32_t r = 0; r < c->nne; ++r) {
        for (auto &pr : rows[r]) pr.first = sidx[pr.first];
        std::sort(rows[r].begin(), rows[r].end());
        for (size_t k = 0; k < rows[r].size(); ++k) {
            S->gcol[S->gptr[r] + k] = (int32_t)rows[r][k].first;
            S->gval[S->gptr[r] + k] = rows[r][k].second;
            S->tptr[rows[r][k].first + 1]++;
        }
    }
    for (int64_t a = 0; a < ns; ++a) S->tptr[a + 1] += S->tptr[a];
    S->tcol.resize(S->tptr[ns]);
    S->tval.resize(S->tptr[ns]);
    {
        std::vector<int64_t> fill(S->tptr.begin(), S->tptr.end() - 1);
        for (int32_t r = 0; r < c->nne; ++r)
            for (int64_t k = S->gptr[r]; k < S->gptr[r + 1]; ++k) {
                const int64_t a = S->gcol[k];
                S->tcol[fill[a]] = r;
                S->tval[fill[a]++] = S->gval[k];
            }
    }
    auto up = [&](void **d, const void *h, size_t bytes) -> int {
        cudaError_t e = cudaMalloc(d, std::max<size_t>(bytes, 8));
        if (e == cudaSuccess && bytes) e = cudaMemcpy(*d, h, bytes, cudaMemcpyHostToDevice);
        return e == cudaSuccess ? 0 : cuda_fail(c, e, "surface correction upload");
    };
    int rc = up((void **)&S->d_gptr, S->gptr.data(), S->gptr.size() * sizeof(int64_t));
    if (!rc) rc = up((void **)&S->d_gcol, S->gcol.data(), S->gcol.size() * sizeof(int32_t));
    if (!rc) rc = up((void **)&S->d_gval, S->gval.data(), S->gval.size() * sizeof(double));
    if (!rc) rc = up((void **)&S->d_tptr, S->tptr.data(), S->tptr.size() * sizeof(int64_t));
    if (!rc) rc = up((void **)&S->d_tcol, S->tcol.data(), S->tcol.size() * sizeof(int32_t));
    if (!rc) rc = up((void **)&S->d_tval, S->tval.data(), S->tval.size() * sizeof(double));
    if (!rc) {
        S->rowptr.resize(c->nne + 1);
        S->col.resize(c->nnz);
        cudaError_t e = cudaMemcpy(S->rowptr.data(), c->d.rowptr, S->rowptr.size() * sizeof(int64_t),
                                   cudaMemcpyDeviceToHost);
        if (e == cudaSuccess)
            e = cudaMemcpy(S->col.data(), c->d.col, S->col.size() * sizeof(int32_t), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) rc = cuda_fail(c, e, "surface correction pattern copy");
    }
    c->surf = S;
    if (rc) surf_release(c);
    return rc;
}

void surf_release(Ctx *c) {
    Surface *S = c->surf;
    if (!S) return;
    void *p[] = {S->d_gptr, S->d_gcol, S->d_gval, S->d_tptr, S->d_tcol, S->d_tval};
    for (void *q : p)
        if (q) cudaFree(q);
    delete S;
    c->surf = nullptr;
}

// N = G_s^T M G_s of a matrix set, factorised; cached per set and assembly
static int surf_factor(Ctx *c, const MatrixSet &MS, const BandLU **out) {
    Surface *S = c->surf;
    for (auto &en : S->cache)
        if (en.M64 == MS.M64 && en.gen == c->asm_gen) {
            *out = en.lu.get();
            return 0;
        }
    // entries of another assembly are stale
    S->cache.erase(std::remove_if(S->cache.begin(), S->cache.end(),
                                  [&](const Surface::Entry &en) { return en.gen != c->asm_gen; }),
                   S->cache.end());
    std::vector<double> M(c->nnz);
    MVF_CUDA(c, cudaMemcpy(M.data(), MS.M64, M.size() * sizeof(double), cudaMemcpyDeviceToHost));
    const int64_t ns = S->ns;
    std::vector<std::vector<std::pair<int32_t, double>>> nrow(ns);
    int64_t bw = 0;
#pragma omp parallel reduction(max : bw)
    {
        std::vector<double> acc(ns, 0.0);
        std::vector<char> mark(ns, 0);
        std::vector<int32_t> touched;
#pragma omp for schedule(dynamic, 64)
        for (int64_t a = 0; a < ns; ++a) {
            touched.clear();
            for (int64_t k1 = S->tptr[a]; k1 < S->tptr[a + 1]; ++k1) {
                const int32_t i = S->tcol[k1];
                const double g1 = S->tval[k1];
                for (int64_t k = S->rowptr[i]; k < S->rowptr[i + 1]; ++k) {
                    const int32_t j = S->col[k];
                    const int64_t k20 = S->gptr[j], k21 = S->gptr[j + 1];
                    if (k20 == k21) continue;
                    const double m = g1 * M[k];
                    for (int64_t k2 = k20; k2 < k21; ++k2) {
                        const int32_t b = S->gcol[k2];
                        if (!mark[b]) {
                            mark[b] = 1;
                            touched.push_back(b);
                        }
                        acc[b] += m * S->gval[k2];
                    }
                }
            }
            std::sort(touched.begin(), touched.end());
            nrow[a].reserve(touched.size());
            for (int32_t b : touched) {
                nrow[a].push_back({b, acc[b]});
                bw = std::max<int64_t>(bw, std::abs((int64_t)b - a));
                acc[b] = 0.0;
                mark[b] = 0;
            }
        }
    }
    std::unique_ptr<BandLU> lu(new BandLU());
    lu->init(ns, (int)bw, (int)bw);
    for (int64_t a = 0; a < ns; ++a)
        for (auto &pr : nrow[a]) lu->at(a, pr.first) = pr.second;
    if (!lu->factor()) return fail(c, MVF_E_SINGULAR, "surface correction: singular nodal system");
    *out = lu.get();
    S->cache.emplace_back();
    S->cache.back().M64 = MS.M64;
    S->cache.back().gen = c->asm_gen;
    S->cache.back().lu = std::move(lu);
    return 0;
}

int surf_numeric(Ctx *c, const MatrixSet &MS, const double *wq, int R, SurfJob **out) {
    *out = nullptr;
    if (!c->surf) return fail(c, MVF_E_STATE, "surface correction not set up");
    const BandLU *lu = nullptr;
    if (int rc = surf_factor(c, MS, &lu)) return rc;
    SurfJob *J = new SurfJob();
    J->lu = lu;
    J->ns = c->surf->ns;
    J->R = R;
    J->w.assign(wq, wq + R);
    const size_t bytes = (size_t)J->ns * R * sizeof(double2);
    cudaError_t e = cudaMallocHost((void **)&J->h_in, bytes);
    if (e == cudaSuccess) e = cudaMallocHost((void **)&J->h_out, bytes);
    if (e == cudaSuccess) e = cudaMalloc((void **)&J->d_ys, bytes);
    if (e == cudaSuccess) e = cudaMalloc((void **)&J->d_y, bytes);
    if (e != cudaSuccess) {
        surf_free(J);
        return cuda_fail(c, e, "surface correction buffers");
    }
    *out = J;
    return 0;
}

void surf_free(SurfJob *J) {
    if (!J) return;
    if (J->h_in) cudaFreeHost(J->h_in);
    if (J->h_out) cudaFreeHost(J->h_out);
    if (J->d_ys) cudaFree(J->d_ys);
    if (J->d_y) cudaFree(J->d_y);
    delete J;
}

void surf_apply(Ctx *c, SurfJob *J, const MatrixSet &MS, const double *d_wq, const double2 *r, double2 *z,
                double2 *t) {
    const Surface *S = c->surf;
    const int R = J->R;
    const size_t bytes = (size_t)J->ns * R * sizeof(double2);
    count_launch();
    surf_resid<<<grid_of((int64_t)c->nne * R), 256, 0, c->stream>>>(c->nne, c->d.rowptr, c->d.col, MS.K64, MS.M64,
                                                                    d_wq, R, r, z, t);
    count_launch();
    surf_gather<<<grid_of(J->ns * R), 256, 0, c->stream>>>(J->ns, R, S->d_tptr, S->d_tcol, S->d_tval, t, J->d_ys);
    cudaMemcpyAsync(J->h_in, J->d_ys, bytes, cudaMemcpyDeviceToHost, c->stream);
    cudaLaunchHostFunc(c->stream, surf_host, J);
    cudaMemcpyAsync(J->d_y, J->h_out, bytes, cudaMemcpyHostToDevice, c->stream);
    count_launch();
    surf_scatter<<<grid_of((int64_t)c->nne * R), 256, 0, c->stream>>>(c->nne, R, S->d_gptr, S->d_gcol, S->d_gval,
                                                                      J->d_y, z);
}

}  // namespace mvf

using namespace mvf;

// Test hook (host only, no device): the band LU of the surface correction on a dense
// column-major n x n matrix whose entries outside the band [-kl, ku] are ignored;
// solves for nrhs right-hand sides b [nrhs][n] in place.
extern "C" int mvf_band_solve(int64_t n, int32_t kl, int32_t ku, const double *a, double *b, int32_t nrhs) {
    if (n < 1 || kl < 0 || ku < 0 || !a || !b || nrhs < 1) return MVF_E_ARG;
    BandLU lu;
    lu.init(n, kl, ku);
    for (int64_t j = 0; j < n; ++j)
        for (int64_t i = std::max<int64_t>(0, j - ku); i <= std::min<int64_t>(n - 1, j + kl); ++i)
            lu.at(i, j) = a[(size_t)j * n + i];
    if (!lu.factor()) return MVF_E_SINGULAR;
    for (int32_t q = 0; q < nrhs; ++q) lu.solve(b + (size_t)q * n);
    return 0;
}

extern "C" int mvf_set_surface_correction(mvf_ctx *xc, int32_t on) {
    if (!xc) return MVF_E_ARG;
    Ctx *c = &xc->c;
    if (!on) {
        c->surf_on = 0;
        return 0;
    }
    if (!c->use_patches || c->precond != 0 || c->mg.empty())
        return fail(c, MVF_E_UNSUPPORTED, "surface correction needs the multilevel preconditioner (36/54-DOF elements)");
    if (int rc = surf_setup(c)) return rc;
    c->surf_on = 1;
    return 0;
}
