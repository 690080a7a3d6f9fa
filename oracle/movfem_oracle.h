/*
 * movfem_oracle.h -- CPU oracle for the MoVFEM_3DMT assembly / post-processing hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * Fortran (MoVFEM_3DMT/src/{n_fem,v_fem,integration,problem,boundary_conds,
 * global_assembly,solution,receiver_data}.f90 and the global_vfem/local_vfem
 * routines of MoVFEM_3DMT.f90).  It exists so that tests, the smoke check and the
 * CPU baseline leg of bench.py can check or time the CUDA path.  The product
 * library never links, loads or calls it.
 *
 * Parity pin: the reference is Fortran and no Fortran compiler exists on either
 * machine, so the reference itself cannot be run to produce golden outputs, and it
 * ships no golden vectors or tests.  "parity unpinned" against reference outputs;
 * the oracle is pinned instead by known-answer tests (tangential continuity of the
 * edge basis -- the reference's own vf_check_sharing check --, the uniform
 * half-space MT response, the 1-D Wait recursion) and by committed fixtures.
 *
 * Conventions follow the reference: node id = (i*nny + j)*nnz + k (0-based form of
 * geometry.f90's (i-1)*g_nyz+(j-1)*g_nnz+k), element id = (ie*ny + je)*nz + ke,
 * complex values are interleaved (re, im) doubles, symmetric 3x3 tensors are
 * packed (xx, xy, xz, yy, yz, zz) as in problem.f90.
 */
#ifndef MOVFEM_ORACLE_H
#define MOVFEM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Quirk switches (bitmask).  All on = the reference's behaviour. */
#define ORC_Q_LIN_DZETA   1  /* n_fem.f90:193 linear dN/dzeta uses (1+nr1) not (1+nr1*xi) */
#define ORC_Q_FP32_CONST  2  /* default-real literals / cmplx() without kind= rounded to FP32 */
#define ORC_Q_GPML_LAG    4  /* MoVFEM_3DMT.f90:203-206 stretch uses previous element's zone flags */
#define ORC_Q_ALL         7

typedef struct orc_mesh {
    int32_t nodes_per_elem;   /* 8, 20 or 27 */
    int32_t nx, ny, nz;       /* element counts (g_nx-1, g_ny-1, g_nz-1) */
    const double *xp;         /* [nnx] */
    const double *yp;         /* [nny] */
    const double *zp;         /* [npt] */
    const double *sigma;      /* [npt][6] complex interleaved: g_sigma(6,g_npt) */
    const double *mu;         /* [npt][6]: g_mu(6,g_npt) */
    int32_t dirichlet;        /* 1 = Dirichlet boundary, 0 = GPML */
    int32_t inimod;           /* Dirichlet primary model (1 zero, 2 half-space, 3 layered) */
    int32_t gpml_sch;         /* 0 = Fang, 1 = Zhou */
    double a0, b0, nn;        /* GPML parameters from PARAM.INP */
    int32_t nextd;            /* extension (PML) cells per side */
    int32_t nzl_top;          /* g_nzl(g_nsf): element layers of the top zone */
    int32_t nzl_air;          /* g_nzl(g_nsf-1): element layers of the air zone below it */
    double ztop;              /* g_ztop (surface level) for inimod 2/3 */
    double h_sigma;           /* half-space conductivity (inimod 2) */
    int32_t nlayers;          /* inimod 3 */
    const double *l_sigma;    /* [nlayers] */
    const double *l_dz;       /* [nlayers-1] */
    int32_t quirks;           /* ORC_Q_* */
} orc_mesh;

int orc_edges_per_elem(int nodes_per_elem);
int orc_num_nodes(const orc_mesh *m, int32_t *nnx, int32_t *nny, int32_t *nnz, int64_t *npt);

/* Global edge numbering gne (global_assembly.f90:183-475 + boundary_conds.f90:252-390).
 * gne is written column-major like the reference: gne[im*ne + e].  Returns nne. */
int32_t orc_numbering(const orc_mesh *m, int32_t *gne);

/* Slot map nzindx (global_assembly.f90:197-229,477-1906): nzindx[e*me*me + im*me + jm],
 * 1-based slot or -1.  Returns nnze, or -1 on inconsistency. */
int64_t orc_slot_map(const orc_mesh *m, const int32_t *gne, int32_t *nzindx);

/* COO coordinates of every slot (ga_assemble_nze, global_assembly.f90:81-121).
 * ia/ja are 1-based; returns 0 or -1 if a slot gets two coordinates. */
int orc_coo_coords(const orc_mesh *m, const int32_t *gne, const int32_t *nzindx,
                   int64_t nnze, int32_t *ia, int32_t *ja);

/* Element matrices of element e at angular frequency omega: K, M (me x me real,
 * row-major), b (me x 2 complex interleaved, b[(im*2+d)*2+{0,1}]).  The GPML zone flags
 * used are those the reference's loop order would use (lag quirk; ifreq is the 0-based
 * position of this frequency in the reference's frequency loop); *pml_out gets the 3
 * flags actually applied.  A_e = K + i*w32*M (integration.f90:76-86). */
int orc_element(const orc_mesh *m, int64_t e, double omega, int32_t ifreq, double *K,
                double *M, double *b, int32_t *pml_out);

/* Full assembly: a[nnze] complex (pre-sort COO values), rhs[2*nne] complex
 * (MoVFEM_3DMT.f90:167-263). */
int orc_assemble(const orc_mesh *m, const int32_t *gne, const int32_t *nzindx,
                 int64_t nnze, int32_t nne, double omega, int32_t ifreq, double *a,
                 double *rhs);

/* Receiver evaluation (solution.f90:207-505, receiver_data.f90:111-253): x is the
 * solution [2*nne] complex (column-major, pol 1 then pol 2).  For each receiver
 * (xr, yr): E, H [nrx][2 pol][3] complex, Z[nrx][4] complex, rho/phi [nrx][4]. */
int orc_receivers(const orc_mesh *m, const int32_t *gne, int32_t nne, double omega,
                  const double *x, int32_t nrx, const double *xr, const double *yr,
                  double *E, double *H, double *Z, double *rho, double *phi);

/* node_solution + z_rho_phi (solution.f90:18-69): E, H [npt][2][3] complex, Z [npt][4]
 * complex, rho, phi [npt][4] at every node; outputs may be NULL. */
int orc_node_fields(const orc_mesh *m, const int32_t *gne, int32_t nne, double omega, const double *x,
                    double *E, double *H, double *Z, double *rho, double *phi);

/* Inner geomodel (read_input.f90:104-200): point id p = (im*my + jm)*mz + km;
 * ijsigma/ijmu in the Fortran layout {i_1..i_n, j_1..j_n}; sigma [npts][isigma],
 * mu [npts][imu] (relative). */
typedef struct orc_model {
    int32_t mx, my, mz;
    const double *xm, *ym, *zm;
    int32_t isigma;
    const int32_t *ijsigma;
    const double *sigma;
    int32_t imu;
    const int32_t *ijmu;
    const double *mu;
} orc_model;

/* Nodal sigma [npt][6] complex and mu [npt][6] of the grid from the inner geomodel,
 * in the reference's sequence (innermodel_gqg, min_dd_inner, assign_model:
 * geometry.f90:804-1085): brute-force search of every model point for each node of
 * each inner element (element order ie, je, ke; first point within 1e-5 m, else first
 * nearest), copies to the extension planes, bottom layers, air, then negative entries
 * from the node below.  The grid fields of m are read (sigma/mu ignored).  Returns 0,
 * -1 on a size error, -2 when a node finds no model point (the reference would index
 * sigma(:,-1)). */
int orc_map_model(const orc_mesh *m, const orc_model *md, double omega, double *sigma, double *mu);

/* Basis self-check of the reference's vf_check_sharing kind: maximum mismatch of the
 * tangential component of shared edge basis functions between face neighbours. */
double orc_check_sharing(const orc_mesh *m);

/* Test switch, not the reference: assemble the multilevel preconditioner's mass
 * instead of the reference's: on = 1 the interpolated conductivity shifted positive
 * semidefinite plus floor_s S/m, on = 2 plus floor_s only, on = 0 the reference's. */
void orc_set_pmass(int on, double floor_s);

#ifdef __cplusplus
}
#endif
#endif
