/*
 * movfem_gpu.h -- C-ABI of the GB300 edge-element assembly and complex sparse solve
 * for MoVFEM_3DMT.
 *
 * The reference is a Fortran program whose hot path is three call sites in its
 * frequency loop (MoVFEM_3DMT/src/MoVFEM_3DMT.f90):
 *   :82   call global_vfem(mumps_par%irn, mumps_par%jcn, mumps_par%a, mumps_par%rhs)
 *   :115  call zmumps(mumps_par)              ! job=6: analyse + factor + solve, nrhs=2
 *   :123  call node_solution(mumps_par%rhs)   ! then receiver Z / rho / phi
 * with the numbering built once by ga_init (global_assembly.f90:26-41).  The entry
 * points below replace them; a Fortran host binds them with ISO_C_BINDING.  Plain pointers and sizes only; every function returns 0 on
 * success or a negative MVF_E_* code, and mvf_last_error() gives the message.
 * The library never calls back into the host, and one context is used by one host
 * thread at a time (the reference is single-threaded with module-level state).
 *
 * Conventions (as the reference): node id = (i*nny + j)*nnz + k; element id =
 * (ie*ny + je)*nz + ke; symmetric tensors packed (xx, xy, xz, yy, yz, zz);
 * complex numbers are interleaved (re, im) doubles; DOF numbers are 1-based, negative
 * values are Dirichlet face flags (-1..-6 for x-, y-, z-, x+, y+, z+).
 */
#ifndef MOVFEM_GPU_H
#define MOVFEM_GPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    MVF_OK = 0,
    MVF_E_ARG = -1,        /* invalid argument / size */
    MVF_E_CUDA = -2,       /* a CUDA call failed */
    MVF_E_SINGULAR = -3,   /* zero Jacobian or singular material tensor (n_fem.f90:374-377, problem.f90:260-271) */
    MVF_E_NOCONV = -4,     /* solver stopped at its iteration cap above tolerance */
    MVF_E_STATE = -5,      /* call out of order (e.g. solve before assemble) */
    MVF_E_RECEIVER = -6,   /* receiver outside the inner grid (receiver_data.f90:187-209) */
    MVF_E_NOMEM = -7,      /* device allocation failed */
    MVF_E_UNSUPPORTED = -8 /* option not built */
};

/* Quirk switches; MVF_Q_ALL reproduces the reference. */
#define MVF_Q_LIN_DZETA  1  /* n_fem.f90:193 linear dN/dzeta written with (1+nr1) */
#define MVF_Q_FP32_CONST 2  /* default-real literals and kind-less cmplx() rounded to FP32 */
#define MVF_Q_GPML_LAG   4  /* MoVFEM_3DMT.f90:203-206 GPML stretch uses the previous element's zone flags */
#define MVF_Q_ALL        7

/* Mesh and model: the arrays geometry.f90:17-24 holds after grid_3d, plus the
 * boundary settings of PARAM.INP (MoVFEM_3DMT.f90:303-336).  Host pointers; copied. */
typedef struct mvf_mesh {
    int32_t nodes_per_elem;   /* 8, 20 or 27 (in_mn) */
    int32_t nx, ny, nz;       /* elements per axis (g_nx-1, g_ny-1, g_nz-1) */
    const double *xp;         /* [nnx] g_xp */
    const double *yp;         /* [nny] g_yp */
    const double *zp;         /* [npt] g_zp */
    const double *sigma;      /* [npt][6] complex: g_sigma(6,g_npt) */
    const double *mu;         /* [npt][6]: g_mu(6,g_npt) */
    int32_t dirichlet;        /* PARAM.INP boundary: 1 Dirichlet, 0 GPML */
    int32_t inimod;           /* Dirichlet primary model: 1 zero secondary field, 2 half-space,
                                 3 layered (bd_inimod, boundary_conds.f90:188-250,396-598) */
    int32_t gpml_sch;         /* 0 Fang, 1 Zhou */
    double a0, b0, nn;        /* GPML parameters */
    int32_t nextd;            /* extension cells per side */
    int32_t nzl_top;          /* g_nzl(g_nsf) */
    int32_t nzl_air;          /* g_nzl(g_nsf-1) */
    double ztop;              /* g_ztop */
    int32_t quirks;           /* MVF_Q_* */
    /* Dirichlet primary models 2/3 (PARAM.INP; unused otherwise): */
    double h_sigma;           /* inimod 2: half-space conductivity */
    int32_t nlayers;          /* inimod 3: number of layers (1..16) */
    const double *l_sigma;    /* inimod 3: [nlayers] layer conductivities, top first */
    const double *l_dz;       /* inimod 3: [nlayers-1] layer thicknesses (m) */
} mvf_mesh;

typedef struct mvf_stats {
    int32_t outer_iters;      /* FP64 refinement steps */
    int32_t inner_iters;      /* Krylov iterations (max over right-hand sides) */
    double rel_residual;      /* max over RHS of ||b - A x|| / ||b|| in FP64 */
    double seconds;           /* device time of the solve */
    int64_t bytes_moved;      /* algorithmic HBM bytes of the executed kernels */
    int32_t stagnated;        /* 1: stopped at a residual floor (<= 1e-5) set by the
                                 right-hand side's component in the air-gradient kernel */
} mvf_stats;

typedef struct mvf_ctx mvf_ctx;

/* Set-up (ga_init + init_* of MoVFEM_3DMT.f90:267-406): copies the model to the
 * device, numbers the DOFs (global_assembly.f90:183-475), builds the CSR pattern
 * (both triangles) and the discrete gradient used by the preconditioner.
 * device < 0 keeps the current device. */
int mvf_create(mvf_ctx **ctx, const mvf_mesh *mesh, int32_t device);
void mvf_destroy(mvf_ctx *ctx);
const char *mvf_last_error(const mvf_ctx *ctx); /* NULL: this thread's last context-free call */

/* Sizes: free DOFs nne (global_assembly.f90:194), nnz of the full pattern, nnz of its
 * lower triangle (the reference's nnze minus its never-written upper slots). */
int mvf_sizes(const mvf_ctx *ctx, int32_t *nne, int64_t *nnz_full, int64_t *nnz_lower, int32_t *edges_per_elem,
              int64_t *num_elems);

/* Global DOF numbering gne(ne, me) in the reference's column-major layout
 * (gne[im*ne + e]), bit-exact with c_gne12/36/54. */
int mvf_numbering(const mvf_ctx *ctx, int32_t *gne);

/* Replace the nodal conductivity (update_sigma, geometry.f90:144-153, runs on the host
 * side of the boundary); [npt][6] complex. */
int mvf_set_sigma(mvf_ctx *ctx, const double *sigma);

/* Assembly for nfreq angular frequencies (global_vfem / local_vfem,
 * MoVFEM_3DMT.f90:167-263): element curl-curl K_e, mass M_e and source b_e on the GPU,
 * scattered into the CSR.  sigma_f: optional [nfreq][npt][6] complex per-frequency
 * conductivity (NULL: the current one for all).  ifreq0: position of omega[0] in the
 * reference's frequency loop (for the GPML zone-flag lag). */
int mvf_assemble(mvf_ctx *ctx, int32_t nfreq, const double *omega, const double *sigma_f, int32_t ifreq0);

/* Parity hook: the lower-triangle COO of frequency f that global_vfem would hand to
 * MUMPS (before ga_sort_sparse, exact zeros kept), 1-based, in row-major order.
 * ia/ja/a may be NULL to query *nnz.  a is complex. */
int mvf_export_coo(const mvf_ctx *ctx, int32_t f, int32_t *ia, int32_t *ja, double *a, int64_t *nnz);
/* The same COO with the exact-zero entries left out, as find_zeros / rem_zeros leave
 * them out before the MUMPS call (global_assembly.f90:123-150, MoVFEM_3DMT.f90:85-97):
 * *nnz = entries kept, *nzero = entries dropped (value exactly 0 + 0i).  ia/ja/a may be
 * NULL to query both counts; the kept entries stay in the same order. */
int mvf_export_coo_nz(const mvf_ctx *ctx, int32_t f, int32_t *ia, int32_t *ja, double *a, int64_t *nnz,
                      int64_t *nzero);
/* Right-hand sides of frequency f: [2][nne] complex (mumps_par%rhs layout). */
int mvf_export_rhs(const mvf_ctx *ctx, int32_t f, double *rhs);

/* Parity hook: element matrices of elements [e0, e0+count) at frequency f of the last
 * assembly: K, M [count][me][me] (real), b [count][me][2] complex. */
int mvf_element_matrices(const mvf_ctx *ctx, int64_t e0, int64_t count, int32_t f, double *K, double *M,
                         double *b);

/* Solve (replaces zmumps job=6, MoVFEM_3DMT.f90:113-115): for every assembled
 * frequency and both polarisations.  rhs_inout: [nfreq][2][nne] complex; on entry
 * the right-hand sides (NULL: use the assembled ones), on exit the solutions (the
 * mumps_par%rhs convention).  mode: 0 = mixed (complex FP32 FGMRES inside FP64
 * iterative refinement, all frequencies batched), 1 = plain FP64 FGMRES one
 * right-hand side at a time.  tol: FP64 relative residual target. */
int mvf_solve(mvf_ctx *ctx, double *rhs_inout, double tol, int32_t mode, int32_t max_iters, mvf_stats *st);

/* Solver settings of a context (no counterpart in the reference): FGMRES restart
 * length (2..256, default 30), Gram-Schmidt passes of the mixed mode (1 or 2,
 * default 1), and the arithmetic of the one-level vertex-patch preconditioner of the
 * 36/54-DOF elements (mvf_set_preconditioner kind 1) in the mixed mode: 1 FP64, 2
 * float-float on the FP32 pipe (default; falls back to FP64 when a scaled inverse
 * entry does not fit two FP32 halves).  The plain FP64 mode always applies it in FP64.
 * 0 keeps a setting. */
int mvf_set_solver(mvf_ctx *ctx, int32_t restart, int32_t mixed_passes, int32_t patch_precision);
/* Preconditioner of the 36/54-DOF systems (no counterpart in the reference, which
 * factorises with MUMPS).  kind 0: multilevel (default): vertex-patch smoothing on the
 * 36/54-DOF level, Galerkin coarsening to the 12-edge space on the same cells, then to
 * merged cells, down to a directly solved level.  It works on K + i w Mp, where Mp is
 * the mass matrix of the interpolated conductivity shifted positive semidefinite at
 * every Gauss point (the quadratic interpolation undershoots below zero next to
 * jumps), plus a floor conductivity (S/m; default 1e-8, <= 0 keeps the setting) that
 * makes the air's gradients regular, plus tau diag(K) (default 0, < 0 keeps the
 * setting).  kind 2: the same without the semidefinite shift.  kind 1: the one-level
 * vertex-patch method.  Takes effect at the next mvf_assemble. */
int mvf_set_preconditioner(mvf_ctx *ctx, int32_t kind, double floor_s, double tau);
/* Levels of the multilevel preconditioner (0 when not in use) and the free DOFs of the
 * first cap of them (level 0 is the system itself). */
int mvf_mg_levels(const mvf_ctx *ctx, int32_t *nlevels, int32_t *ndofs, int32_t cap);
/* Test hook: one cycle of the multilevel preconditioner for frequency f applied to R
 * host right-hand sides r [n][R] complex; z [n][R] complex. */
int mvf_mg_apply_once(mvf_ctx *ctx, int32_t f, int32_t R, const double *r, double *z);
/* Measurement hook: one level-0 smoothing sweep of the multilevel preconditioner over
 * every assembled frequency and both polarisations (mixed-mode arithmetic), timed on
 * the library's stream; bytes: its algorithmic bytes (patch inverses, patch rows of
 * the CSR, the patch DOFs' vectors). */
int mvf_profile_mg(mvf_ctx *ctx, int32_t reps, double *sec_per_sweep, int64_t *bytes);
/* Batching of the mixed mode (no counterpart in the reference): per_frequency 0 solves
 * every frequency of a matrix set and both polarisations as one batch of right-hand
 * sides (default), 1 solves one frequency (2 right-hand sides) per batch, so that each
 * frequency stops at its own iteration count. */
int mvf_set_batching(mvf_ctx *ctx, int32_t per_frequency);
/* Surface gradient correction of the multilevel preconditioner (36/54-DOF elements;
 * no counterpart in the reference, which factorises): after each cycle the gradient
 * modes of the grid nodes from one node layer below the earth's surface to the top of
 * the first air cells are solved exactly with the true operator, where the quadratic
 * interpolation of the nodal conductivity makes it indefinite.  The nodal system of
 * those layers is factorised once per assembled matrix set (band LU on the host CPU)
 * and solved on the host between two device stages of each application.  on = 1
 * enables (MVF_E_UNSUPPORTED without the multilevel preconditioner, MVF_E_ARG when the
 * grid has no surface between its earth and air layers), 0 disables. */
int mvf_set_surface_correction(mvf_ctx *ctx, int32_t on);
/* Test hook (host only): the band LU with partial pivoting that the surface correction
 * uses, on a dense column-major n x n matrix a (entries outside the band [-kl, ku]
 * ignored), solving nrhs right-hand sides b [nrhs][n] in place.  MVF_E_SINGULAR on a
 * zero pivot column. */
int mvf_band_solve(int64_t n, int32_t kl, int32_t ku, const double *a, double *b, int32_t nrhs);
/* Arithmetic the last vertex-patch inversion set up: 0 no patches (12-DOF elements),
 * 1 FP64, 2 float-float (scaled inverses split into FP32 halves). */
int32_t mvf_patch_arithmetic(const mvf_ctx *ctx);

/* Solve n independent contexts (models of any size) concurrently: nthreads host
 * threads take contexts from a queue, largest first, and run mvf_solve (with the
 * assembled right-hand sides, solutions kept on the device) on each context's stream.
 * No counterpart in the reference, which solves one model per run.  st: [n] or NULL.
 * Returns the first error other than MVF_E_NOCONV, else MVF_E_NOCONV if any context
 * stopped above tolerance, else 0.  Each context's error text stays in that context. */
int mvf_solve_many(mvf_ctx **ctx, int32_t n, double tol, int32_t mode, int32_t max_iters, mvf_stats *st,
                   int32_t nthreads);

/* FP64 receiver evaluation (get_er / get_hr / interpolate_rx / get_impedance /
 * get_res_phase: solution.f90:207-505, receiver_data.f90:111-253) on the last
 * solution: Z [nfreq][nrx][4] complex, rho/phi [nfreq][nrx][4]; E, H optional
 * [nfreq][nrx][2][3] complex. */
int mvf_impedance(mvf_ctx *ctx, int32_t nrx, const double *xr, const double *yr, double *Z, double *rho,
                  double *phi, double *E, double *H);

/* Full-volume fields (node_solution + z_rho_phi, solution.f90:18-69) on the last
 * solution: E, H [nfreq][npt][2][3] complex at every node (first visiting element),
 * Z [nfreq][npt][4] complex, rho / phi [nfreq][npt][4] from each node's horizontal
 * fields.  Any output may be NULL.  write_solution's SOLUTION.OUT layout is produced
 * from these by movfem_gb300.output. */
int mvf_node_fields(mvf_ctx *ctx, double *E, double *H, double *Z, double *rho, double *phi);

/* Parity hook: y = A_f x for frequency f in FP64 (x, y: [2][nne] complex, host). */
int mvf_spmv(mvf_ctx *ctx, int32_t f, const double *x, double *y);

/* Measurement hooks (no reference counterpart): average device time of the FP32
 * K/M SpMM over all right-hand sides sharing frequency f's matrix, timed with CUDA
 * events on the library's stream, and its algorithmic bytes per launch; and the
 * number of kernels this library has launched in the process so far. */
int mvf_profile_spmm(mvf_ctx *ctx, int32_t f, int32_t reps, double *sec_per_launch, int64_t *bytes);
int64_t mvf_kernel_launches(void);

/* Measurement hook (no reference counterpart): average device time of one vertex-patch
 * preconditioner application (36/54-DOF elements; 8 colour launches, 2 right-hand
 * sides, complex FP64) with frequency f's inverses, and its algorithmic bytes
 * (inverse entries x 16 B + patch gathers/scatters + zeroing).  MVF_E_UNSUPPORTED for
 * 12-DOF elements. */
int mvf_profile_patch(mvf_ctx *ctx, int32_t f, int32_t reps, double *sec_per_apply, int64_t *bytes);

/* Autotuner record (no reference counterpart): the first K/M SpMM of each precision
 * and batch width on a context times every kernel variant on the real operands and
 * keeps the fastest; this returns "fp32 R=2: chunked 227.1 us, direct 173.9 us, ...
 * pick vec/G=8; ..." -- every candidate's time per launch and the choice, for the
 * tunings made so far (the string is owned by the context). */
const char *mvf_spmm_tuning(mvf_ctx *ctx);

/* Parity hook for the autotuner's candidates (no reference counterpart): y = A_f x
 * for R right-hand sides (R a power of two <= 32) with SpMM variant `variant`
 * (0 chunked, 1 direct [R <= 4], 2..5 G = 4/8/16/32 lanes per row [R <= 16],
 * 6 float-float operator of the FP64 Krylov path [fp64 = 1]) in FP64
 * (fp64 = 1: K, M and vectors FP64) or FP32 (K, M, vectors complex64); w is the
 * frequency's omega, rounded to FP32 when the mesh's quirks carry MVF_Q_FP32_CONST,
 * as in assembly.  x, y: host [nne][R] complex. */
int mvf_spmm_variant(mvf_ctx *ctx, int32_t f, int32_t variant, int32_t fp64, int32_t R, const double *x,
                     double *y);

/* y = A_f x like mvf_spmv, for callers that cannot let the library allocate device
 * memory (a host whose device memory is owned by its own pool allocator, where a
 * cudaMalloc inside the library would fail or fragment that pool).  No counterpart in
 * the reference.  x, y: DEVICE pointers, [2][nne] complex.  Nothing is allocated: the
 * staging lives in a fixed 16 MiB device array shared by all calls (part of the
 * library's device image: with CUDA's lazy module loading it becomes resident when the
 * first call loads that code on a device), so nne must be <= 262144 (MVF_E_ARG
 * otherwise) and calls that overlap on the GPU race on it.  The
 * kernels run on the library's stream: x must be complete before the call (synchronise
 * the stream that wrote it); the call synchronises that stream and returns with y
 * complete.  The first call on a device looks up the array's device address and keeps
 * it; no cudaDeviceReset may follow that first call in the process. */
int mvf_spmv_noalloc(mvf_ctx *ctx, int32_t f, const double *x_dev, double *y_dev);

/* Initial guess for the following mvf_solve calls (no counterpart in the reference:
 * MUMPS needs none).  x0: host [nfreq][2][nne] complex for the assembled frequencies,
 * copied to the device; the refinement loop then starts from b - A x0 instead of b.
 * x0 = NULL drops the guess.  A guess stored for another frequency count is ignored. */
int mvf_set_guess(mvf_ctx *ctx, const double *x0);

/* ---- Model mapping (the step before the hot path) ----------------------------------
 * The inner geomodel as read_innermodel / read_geomodel (read_input.f90:104-200) hold
 * it: mx*my*mz model points, point id p = (im*my + jm)*mz + km (0-based form of the
 * reference's (im-1)*my*mz+(jm-1)*mz+km), x from xm[im], y from ym[jm], z from zm[p].
 * Component arrays keep the Fortran layout: ijsigma(isigma,2) is
 * {i_1..i_isigma, j_1..j_isigma} (1-based tensor indices, i <= j), and sigma(isigma,n)
 * is [n][isigma] in memory; the same for mu.  isigma = 1: isotropic; imu = 0: mu = mu0
 * everywhere, 1: isotropic relative mu; more: relative tensor components. */
typedef struct mvf_model {
    int32_t mx, my, mz;       /* in_mx, in_my, in_mz */
    const double *xm;         /* [mx] */
    const double *ym;         /* [my] */
    const double *zm;         /* [mx*my*mz] */
    int32_t isigma;           /* in_isigma (>= 1) */
    const int32_t *ijsigma;   /* [2*isigma] */
    const double *sigma;      /* [mx*my*mz][isigma], S/m */
    int32_t imu;              /* in_imu (>= 0) */
    const int32_t *ijmu;      /* [2*imu] (unused when imu <= 1) */
    const double *mu;         /* [mx*my*mz][imu] relative permeability (unused when imu = 0) */
} mvf_model;

/* Nodal conductivity and permeability of the grid from the inner geomodel
 * (innermodel_gqg, min_dd_inner, assign_model: geometry.f90:804-1085), which grid_3d
 * (geometry.f90:106) calls once before the frequency loop.  Reads the grid fields of
 * `grid` (nodes_per_elem, nx, ny, nz, xp, yp, zp, nextd >= 1, nzl_top + nzl_air >= 1,
 * quirks; its sigma and mu are ignored).  Each node of the inner elements takes the
 * first model point (in point order) within 1e-5 m, else the first nearest one; the
 * extension planes, the bottom layers and the air follow the reference's copy order,
 * and negative entries then take the value of the node below.  omega: the angular
 * frequency of the grid time (2*pi*f_1); eps*omega is rounded to FP32 when quirks
 * carry MVF_Q_FP32_CONST.  sigma_out [npt][6] complex, mu_out [npt][6] (g_sigma,
 * g_mu).  seconds (optional): device time of the kernels.  Context-free: on error,
 * mvf_last_error(NULL) gives this thread's message.  device < 0 uses the current
 * device; otherwise that device, and the caller's current device is restored. */
int mvf_map_model(const mvf_mesh *grid, const mvf_model *model, double omega, double *sigma_out, double *mu_out,
                  double *seconds, int32_t device);

/* ---- Gridding (the step before the model mapping) ---------------------------------
 * grid_3d (geometry.f90:48-118) on the host: padding from the skin depth (extension),
 * sub-layers between interfaces (zblocks), node coordinates (gauss_grid, local_gqg,
 * complete_grid), the interfaces interpolated by the modified quadratic Shepard method
 * of ACM TOMS 660 (toms660.f90).  Arguments as read_input leaves them
 * (read_input.f90:47-162), in the input's coordinates. */
typedef struct mvf_grid_in {
    double dx, dy, dz;        /* core cell sizes (in_dx, in_dy, in_dz) */
    double high, depth;       /* air above the highest / earth below the deepest interface point */
    int32_t nodes_per_elem;   /* 8, 20 or 27 (in_mn) */
    double sigma_bg;          /* conductivity of the skin-depth estimate (in_bcksigma) */
    int32_t nsr;              /* receivers */
    const double *rx;         /* [nsr][3] x, y, z */
    int32_t nsf0;             /* input interfaces, top (earth surface) last */
    const int32_t *nsp;       /* [nsf0] points per interface (>= 20 each) */
    const double *pts;        /* [sum nsp][3] interface points, interface after interface */
    int32_t mx, my, mz;       /* inner model grid */
    const double *xm, *ym;    /* [mx], [my] */
    const double *zm;         /* [mx*my*mz] */
    int32_t nf;               /* frequencies (the lowest sets the padding) */
    const double *freqs;      /* [nf] Hz */
} mvf_grid_in;

typedef struct mvf_grid_info {
    int32_t nodes_per_elem;
    int32_t nextd;            /* padding cells per side */
    int32_t nsf;              /* interfaces incl. the three added ones (in_nsf) */
    int32_t nx, ny, nz;       /* cells per axis (g_nx-1, g_ny-1, g_nz-1) */
    int64_t nnx, nny, nnz, npt;
    int32_t nzl_top, nzl_air; /* g_nzl(nsf), g_nzl(nsf-1) */
    double x0, y0, z0;        /* shift of coord_transform: grid = input - (x0, y0, z0) */
    double ztop;              /* g_ztop: lowest point of the top input interface, shifted */
    double skin_depth, nd;    /* the padding's target: sum of padding widths > nd * skin_depth */
} mvf_grid_info;

typedef struct mvf_grid mvf_grid;
/* Build the grid.  MVF_E_ARG for invalid input, including an interface with fewer than
 * 20 points or one QSHEP2 cannot fit (the reference reads unset memory there); the
 * message is mvf_last_error(NULL). */
int mvf_grid_3d(const mvf_grid_in *in, mvf_grid **grid);
int mvf_grid_get_info(const mvf_grid *grid, mvf_grid_info *info);
/* g_xp [nnx], g_yp [nny], g_zp [npt] (node (i*nny + j)*nnz + k), g_nzl [nsf]; any may be NULL. */
int mvf_grid_export(const mvf_grid *grid, double *xp, double *yp, double *zp, int32_t *nzl);
void mvf_grid_destroy(mvf_grid *grid);

/* ---- Learned warm start (no counterpart in the reference) -------------------------
 * A dilated 3-D convolutional operator on a cell grid: nconv 3x3x3 convolutions of
 * `width` channels with ReLU (dilations[l] each), then a 1x1x1 convolution to `cout`
 * channels.  BF16 weights and activations, FP32 accumulation; training keeps FP32
 * master weights and runs Adam.  Grids are channels-last [X][Y][Z][c], FP32 on the
 * host.  Parameters are laid out layer by layer: weights [3^3 or 1][cin][cout], then
 * the bias [cout]. */
typedef struct mvf_net mvf_net;
int mvf_net_create(mvf_net **net, int32_t cin, int32_t width, int32_t cout, int32_t nconv, const int32_t *dilations,
                   uint64_t seed, int32_t device);
void mvf_net_destroy(mvf_net *net);
const char *mvf_net_last_error(mvf_net *net);
int64_t mvf_net_num_params(mvf_net *net);
int mvf_net_get_params(mvf_net *net, float *params);
int mvf_net_set_params(mvf_net *net, const float *params); /* also resets Adam */
int mvf_net_forward(mvf_net *net, int32_t X, int32_t Y, int32_t Z, const float *in, float *out);
/* loss = mean over all outputs of (out - target)^2, and d loss / d params (FP32) */
int mvf_net_gradients(mvf_net *net, int32_t X, int32_t Y, int32_t Z, const float *in, const float *target,
                      float *loss, float *grad);
/* forward + backward + one Adam step (beta 0.9 / 0.999, eps 1e-8) at learning rate lr */
int mvf_net_train_step(mvf_net *net, int32_t X, int32_t Y, int32_t Z, const float *in, const float *target, float lr,
                       float *loss);

#ifdef __cplusplus
}
#endif
#endif
