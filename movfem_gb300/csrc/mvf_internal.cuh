// mvf_internal.cuh -- context and shared declarations of the MoVFEM GB300 library.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/movfem_gpu.h"
#include "mvf_basis.cuh"

#define MVF_MAX_NODES 27
#define MVF_MAX_ME 54
#define MVF_MAX_GP 27
#define MVF_MAX_FREQ 16
#define MVF_MG_MAXP 96  // largest direct-solved coarsest level of the multilevel preconditioner

namespace mvf {

#ifdef __CUDACC__
// s += a*b with a, b float-float, as a compensated dot product (Ogita, Rump and Oishi,
// "Accurate sum and dot product", SIAM J. Sci. Comput. 26, 2005, Dot2): the high part
// by TwoSum, every rounding error (the product's by FMA, the cross terms, the sum's)
// collected in a plain FP32 low part without renormalising at each step.  The high
// part's dependency chain is one addition per product.
__device__ __forceinline__ void dot2_mac(float &sh, float &sl, float ah, float al, float bh, float bl) {
    const float p = ah * bh;
    float e = fmaf(ah, bh, -p);
    e = fmaf(ah, bl, fmaf(al, bh, e));
    const float t = sh + p;
    const float bb = t - sh;
    const float err = (sh - (t - bb)) + (p - bb);
    sh = t;
    sl += e + err;
}
#endif

// Element-order constants and tables evaluated at the Gauss points.
struct OrderTables {
    int mn = 0, me = 0, nord = 0, ngp = 0;
    int edge_node[MVF_MAX_ME];  // 0-based node of each edge DOF (mx_edge_dir(:,1))
    int edge_dir[MVF_MAX_ME];   // 0-based direction (mx_edge_dir(:,2))
    int face_cnt = 0;           // DOFs per face
    int face_src[3][12];        // DOFs on the +z, +y, +x face (0-based)
    int face_dst[3][12];        // the same DOFs in the neighbour across that face
    double gp[MVF_MAX_GP][4];   // xi, eta, zeta, weight (integration.f90:267-279)
    // nodal N and dN/dxi at the Gauss points [g][node] / [g][node][3]
    std::vector<double> N, dN;
    // edge factor L and dL/dxi at the Gauss points [g][edge] / [g][edge][3]
    std::vector<double> L, dL;
    // discrete gradient of the element: grad N_n = sum_j G[j][n] * (edge basis j)
    double G[MVF_MAX_ME][MVF_MAX_NODES];
};

// One set of real matrices K, M sharing the CSR pattern: either one per model
// (frequency-independent Dirichlet assembly) or one per frequency (GPML).
struct MatrixSet {
    double *K64 = nullptr, *M64 = nullptr;  // [nnz]
    float *K32 = nullptr, *M32 = nullptr;   // [nnz]
    float2 *Kff = nullptr, *Mff = nullptr;  // [nnz] FP64 values as hi + lo FP32 halves (made on demand)
    // multilevel preconditioner: its mass matrix Mp (conductivity |sigma| + floor at
    // every Gauss point) [nnz], and the Galerkin element matrices on the lowest-order
    // edge space of the same cells, P^T K_e P and P^T Mp_e P, [ne][12][12]
    double *Mp64 = nullptr;
    double *K1e = nullptr, *M1e = nullptr;
    double *kphi = nullptr, *mphi = nullptr, *mabs = nullptr;  // gradient-node diagonals [ngn]
    int first_freq = 0, nfreq = 0;          // frequencies that use this set
};

// Vertex patches of one grid level (host lists; see vertex_patches).
struct PatchHost {
    std::vector<int64_t> ptr, ioff, color_off;  // [np+1], [np+1], [9]
    std::vector<int32_t> dof;
    int pmax = 0;
};

// One level of the multilevel preconditioner below the 36/54-DOF system: the
// lowest-order (12-edge) space on a cell grid.  Level 1 has the context's cells,
// level l+1 merges the cells of level l in pairs along each axis.
struct MgLevel {
    int nx = 0, ny = 0, nz = 0;    // cells
    int32_t n = 0;                 // free DOFs
    int64_t ne = 0, nnz = 0;
    std::vector<int32_t> gne;      // [ne][12], 1-based, <= 0 eliminated
    std::vector<int> ix, iy, iz;   // this level's vertices as vertex indices of the finer level
    int64_t *rowptr = nullptr;     // CSR pattern (both triangles)
    int32_t *col = nullptr;
    int32_t *gne_d = nullptr;
    // prolongation to the next finer level (P: [n_fine][n]) and its transpose
    int64_t *prow = nullptr, *ptrow = nullptr;
    int32_t *pcol = nullptr, *ptcol = nullptr;
    double *pval = nullptr, *ptval = nullptr;
    // levels >= 2: the finer-level children of each element and the local maps
    // Q [ne][8][12 fine][12 this] (child -1: none)
    int32_t *child = nullptr;
    double *Q = nullptr;
    std::vector<int64_t> ecolor_off;  // [9] offsets of the parity colours in elist
    int32_t *elist = nullptr;
    // vertex patches (the coarsest level: one patch holding every DOF)
    int64_t np = 0, pent = 0;
    int pmax = 0;
    std::vector<int64_t> pcolor_off;  // [9]
    int64_t *pptr = nullptr, *pioff = nullptr;
    int32_t *pdof = nullptr;
};

struct Device {
    // model
    double *xp = nullptr, *yp = nullptr, *zp = nullptr;
    double *sigma = nullptr;   // [npt][6][2] current
    double *sigma_f = nullptr; // [nfreq][npt][6][2] per frequency (optional)
    double *mu = nullptr;      // [npt][6]
    int32_t *gne = nullptr;    // [ne][me] element-major
    int32_t *elem_color = nullptr;  // elements sorted by colour
    // tables
    double *N = nullptr, *dN = nullptr, *L = nullptr, *dL = nullptr, *gp = nullptr;
    double *Gloc = nullptr;    // [me][mn]
    int32_t *edge_node = nullptr, *edge_dir = nullptr;
    // CSR (full, both triangles) and discrete gradient
    int64_t *rowptr = nullptr;
    int32_t *col = nullptr;
    int64_t *grow = nullptr;   // G: [nne+1]
    int32_t *gcol = nullptr;
    float *gval = nullptr;
    int64_t *gtrow = nullptr;  // G^T: [ngn+1]
    int32_t *gtcol = nullptr;
    float *gtval = nullptr;
    int32_t *node_gidx = nullptr;  // grid node -> gradient node index or -1
    // right-hand sides and solutions: [nfreq][2][nne] complex
    double *rhs = nullptr;
    double *x = nullptr;
    double *guess = nullptr;  // optional initial guess, same layout (mvf_set_guess)
    // element matrices of the last assembly, kept for the parity hook
    double *Ke = nullptr, *Me = nullptr, *be = nullptr;
    // vertex patches (Schwarz preconditioner of the 36/54-DOF elements)
    int64_t *patch_ptr = nullptr, *patch_ioff = nullptr;
    int32_t *patch_dof = nullptr;
    // Dirichlet primary models 2/3: node -> boundary-node index (-1 elsewhere) and the
    // primary field there, [nfreq][nb][2] complex (E_x of the first polarisation, E_y
    // of the second)
    int32_t *bidx = nullptr;
    double2 *bep = nullptr;
    // the solver's per-batch frequencies (SolveParams, mvf_solve.cu)
    double *wsp = nullptr;
};

struct Ctx {
    mvf_mesh mesh{};
    std::string err;
    int device = 0;
    cudaStream_t stream = nullptr;
    OrderTables T;
    int64_t nnx = 0, nny = 0, nnz_nodes = 0, npt = 0, ne = 0;
    int32_t nne = 0;
    int64_t nnz = 0, nnz_lower = 0;
    int32_t ngn = 0;  // gradient nodes
    std::vector<int32_t> gne_h;  // [ne][me]
    std::vector<double> xp_h, yp_h, zp_h;  // host copies of the coordinates
    std::vector<double> l_sigma_h, l_dz_h;  // layered primary model (inimod 3)
    std::vector<int64_t> bnode_h;           // nodes on the x/y boundary planes (inimod 2/3)
    std::vector<int64_t> color_off;  // 9 offsets into elem_color
    Device d;
    // assembly state
    int nfreq = 0;
    int guess_nfreq = 0;  // frequencies the stored initial guess covers
    double omega[MVF_MAX_FREQ] = {0};
    int ifreq0 = 0;
    std::vector<MatrixSet> sets;
    bool assembled = false, solved = false;
    bool keep_elements = false;
    int64_t ke_count = 0;
    // vertex patches
    bool use_patches = false;
    int64_t npatch = 0, patch_entries = 0, patch_dofs = 0;  // patches, sum P^2, sum P
    int patch_max = 0;
    std::vector<int64_t> pcolor_off;
    // SpMM variant chosen by timing, per [FP64?][log2 R]; -1 = not tuned yet
    int spmm_pick[2][6] = {{-1, -1, -1, -1, -1, -1}, {-1, -1, -1, -1, -1, -1}};
    float spmm_us[2][6] = {};
    std::string spmm_note;
    // FGMRES restart length and Gram-Schmidt passes of the mixed-precision mode
    int restart = 30, mixed_passes = 1;
    // vertex-patch application arithmetic: 1 FP64, 2 float-float on the FP32 pipe; and
    // whether the inverses of the last inversion were split into FP32 halves
    int patch_precision = 2, patch_inv_split = 0;
    int solve_mode = 0;  // mode of the solve in progress (1: plain FP64 throughout)
    // preconditioner of the 36/54-DOF systems: 0 multilevel (default), 1 one-level
    // vertex patches; multilevel hierarchy (levels 1..) and the conductivity floor
    // (S/m) of its operator
    int precond = 0;
    double mg_floor = 1e-8;
    double mg_tau = 0.0;  // optional shift tau diag(K) of the preconditioner's mass
    int mg_abs = 1;       // shift the preconditioner's conductivity positive semidefinite
    int freq_batch = 0;  // mixed mode: 0 every frequency of a matrix set in one batch, 1 one per batch
    std::vector<MgLevel> mg;
    // surface gradient correction of the multilevel method (mvf_surface.cu) and the
    // count of assemblies (its factors are cached per matrix set and assembly)
    int surf_on = 0;
    struct Surface *surf = nullptr;
    uint64_t asm_gen = 0;
};

// process-wide count of the library's kernel launches.  While a thread captures a
// CUDA graph its launches go to that thread's capture tally instead; the graph's
// launches are added to the process count each time it is replayed.
inline std::atomic<int64_t> &launch_counter() {
    static std::atomic<int64_t> n{0};
    return n;
}
inline int64_t *&capture_tally() {
    static thread_local int64_t *t = nullptr;
    return t;
}
inline void count_launch() {
    if (int64_t *t = capture_tally()) ++*t;
    else launch_counter().fetch_add(1, std::memory_order_relaxed);
}

int fail(Ctx *c, int code, const std::string &msg);
int cuda_fail(Ctx *c, cudaError_t e, const char *what);
int64_t element_node(const Ctx &c, int ie, int je, int ke, int l);
int element_matrices(Ctx *c, int64_t e0, int64_t count, int f, double *K, double *M, double *b);

#define MVF_CUDA(c, call)                                         \
    do {                                                          \
        cudaError_t _e = (call);                                  \
        if (_e != cudaSuccess) return ::mvf::cuda_fail((c), _e, #call); \
    } while (0)

void build_tables(int mn, int quirks, OrderTables &T);

// Dirichlet primary models 2/3 (mvf_assemble.cu): true when the boundary DOFs carry
// a non-zero prescribed value that lifts into the right-hand side
inline bool dirichlet_lift(const Ctx &c) { return c.mesh.dirichlet && c.mesh.inimod != 1; }

// assembly (mvf_assemble.cu)
int assemble_set(Ctx *c, MatrixSet &S, bool gpml, int fset);
int assemble_rhs(Ctx *c);
void free_sets(Ctx *c);

// message of this thread's last context-free call (mvf_map_model, mvf_model.cu)
const char *map_last_error();

// numbering and pattern of an element grid (mvf_setup.cu)
int32_t number_grid(const OrderTables &T, int nx, int ny, int nz, bool dirichlet, std::vector<int32_t> &gne);
void pattern_from_gne(const std::vector<int32_t> &gne, int me, int64_t ne, int32_t n, std::vector<int64_t> &rowptr,
                      std::vector<int32_t> &col);

// vertex-patch Schwarz preconditioner (mvf_patch.cu)
void vertex_patches(int nx, int ny, int nz, int me, const std::vector<int32_t> &gne, int32_t n, PatchHost &out);
void launch_patch_invert(cudaStream_t st, int grid, int64_t np, const int64_t *pptr, const int32_t *pdof,
                         const int64_t *ioff, const int64_t *rowptr, const int32_t *col, const double *K,
                         const double *M, double w, double tau, int pmax, double2 *ws, double2 *inv, int *err);
int patch_setup(Ctx *c);
int patch_invert(Ctx *c, const MatrixSet &S, const double *w, int nf, double2 **inv_out);
void patch_apply(Ctx *c, const double2 *inv, int R, int npol, int nfi, const float2 *r, float2 *z);
void patch_apply(Ctx *c, const double2 *inv, int R, int npol, int nfi, const double2 *r, double2 *z);

// multilevel preconditioner (mvf_mg.cu)
int mg_setup(Ctx *c);          // hierarchy, once per context
void mg_release(Ctx *c);
// surface gradient correction (mvf_surface.cu)
struct SurfJob;
int surf_setup(Ctx *c);
void surf_release(Ctx *c);
int surf_numeric(Ctx *c, const MatrixSet &S, const double *wq, int R, SurfJob **out);
void surf_apply(Ctx *c, SurfJob *J, const MatrixSet &S, const double *d_wq, const double2 *r, double2 *z, double2 *t);
void surf_free(SurfJob *J);
struct MgWork;                  // numeric state of one solve batch
int mg_numeric(Ctx *c, const MatrixSet &S, const double *w, int nf, int R, int npol, MgWork **out);
void mg_apply(Ctx *c, MgWork *W, const double2 *r, double2 *z);
void mg_free(Ctx *c, MgWork *W);
// local prolongation of the 12-edge element into the 36/54-DOF element: lists per
// 12-edge DOF a of (36/54-DOF index, coefficient); count per a
struct PLoc {
    int cnt[12];
    int idx[12][8];
    double val[12][8];
};
void p_local(int mn, PLoc &P);

}  // namespace mvf

struct mvf_ctx {
    mvf::Ctx c;
};
