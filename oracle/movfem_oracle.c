/*
 * movfem_oracle.c -- CPU oracle (test infrastructure only; see movfem_oracle.h).
 *
 * Each routine names the reference file:line it restates.  The element loop runs in
 * the reference's order (ie, je, ke with ke fastest) because the GPML stretch of an
 * element depends on the zone flags left by the previous element
 * (MoVFEM_3DMT.f90:200-206: int_elem_params evaluates gpml_h before get_pml).
 */
#include "movfem_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef double complex cplx;

/* Not the reference: the mass rule of the GPU library's multilevel preconditioner
 * (mvf_mg.cu), switched on by orc_set_pmass for tests of that preconditioner.  The real
 * part of the interpolated conductivity tensor at a Gauss point is shifted by twice the
 * negative part of its Gershgorin lower bound (|sigma| for an isotropic tensor; on = 1
 * only) plus a floor conductivity (on = 1 or 2). */
static int g_pmass_on = 0;
static double g_pmass_floor = 0.0;

void orc_set_pmass(int on, double floor_s) {
    g_pmass_on = on;
    g_pmass_floor = floor_s;
}

static const int PK6[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};

static void pmass_sigma(cplx *mf2) {
    double gmin = 1e300, shift;
    int a, b;
    for (a = 0; a < 3; a++) {
        double off = 0.0, v;
        for (b = 0; b < 3; b++)
            if (b != a) off += fabs(creal(mf2[PK6[a][b]]));
        v = creal(mf2[PK6[a][a]]) - off;
        if (v < gmin) gmin = v;
    }
    shift = (g_pmass_on == 1 ? 2.0 * (gmin < 0.0 ? -gmin : 0.0) : 0.0) + g_pmass_floor;
    for (a = 0; a < 3; a++) mf2[PK6[a][a]] += shift;
}

static const double PI = 3.1415926535897932384626433;      /* geometry.f90:25 */
static const double EPS0 = 8.854187817e-12;                 /* geometry.f90:25 */
static const double B0_PRIMARY = 1.0e-9;                     /* problem.f90:27 */

/* ------------------------------------------------------------------ tables */
/* Reference coordinates of the 27 element nodes (n_fem.f90:112-134). */
static const int NR[3][27] = {
    {1, 1, -1, -1, 1, 1, -1, -1, 1, 0, -1, 0, 1, 0, -1, 0, 1, 1, -1, -1, 1, 0, -1, 0, 0, 0, 0},
    {-1, 1, 1, -1, -1, 1, 1, -1, 0, 1, 0, -1, 0, 1, 0, -1, -1, 1, 1, -1, 0, 1, 0, -1, 0, 0, 0},
    {-1, -1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, -1, 1, 0}};

/* Edge DOF -> (node, direction), 1-based (v_fem.f90:488-506). */
static const int EDGE12_NODE[12] = {4, 4, 8, 3, 4, 8, 3, 7, 1, 1, 5, 2};
static const int EDGE12_DIR[12] = {3, 2, 2, 3, 1, 1, 1, 1, 3, 2, 2, 3};
static const int EDGE36_NODE[36] = {4, 8, 4, 3, 8, 7, 3, 7, 4, 1, 8, 5, 3, 2, 7, 6, 1, 5,
                                    1, 2, 5, 6, 2, 6, 12, 20, 12, 16, 10, 17, 11, 20, 11, 15, 19, 9};
static const int EDGE36_DIR[36] = {3, 3, 2, 2, 2, 2, 3, 3, 1, 1, 1, 1, 1, 1, 1, 1, 3, 3,
                                   2, 2, 2, 2, 3, 3, 3, 2, 2, 2, 3, 2, 3, 1, 1, 1, 1, 3};
static const int EDGE54_NODE[54] = {4, 8, 4, 20, 8, 11, 15, 3, 19, 7, 3, 7, 4, 20, 8, 11, 15, 3,
                                    19, 7, 12, 16, 12, 10, 16, 14, 10, 14, 1, 17, 5, 9, 13, 2, 18, 6,
                                    1, 5, 1, 17, 5, 9, 13, 2, 18, 6, 2, 6, 25, 26, 24, 22, 23, 21};
static const int EDGE54_DIR[54] = {3, 3, 2, 2, 2, 3, 3, 2, 2, 2, 3, 3, 1, 1, 1, 1, 1, 1,
                                   1, 1, 3, 3, 2, 2, 2, 2, 3, 3, 1, 1, 1, 1, 1, 1, 1, 1,
                                   3, 3, 2, 2, 2, 3, 3, 2, 2, 2, 3, 3, 3, 3, 2, 2, 1, 1};

/* Face maps: DOF on the + face of an element -> the same DOF in the neighbour across
 * that face (its - face).  Order z, y, x.  These are the tables of c_gne12/36/54
 * (global_assembly.f90:242-265,310-351,396-443), shr_nzindx12/36/54 and the
 * boundary-edge lists of edge_bdary (boundary_conds.f90:262-390). */
static const int FACE12[3][2][4] = {{{3, 6, 8, 11}, {2, 5, 7, 10}},
                                    {{4, 7, 8, 12}, {1, 5, 6, 9}},
                                    {{9, 10, 11, 12}, {1, 2, 3, 4}}};
static const int FACE36[3][2][10] = {
    {{5, 6, 11, 12, 15, 16, 21, 22, 28, 34}, {3, 4, 9, 10, 13, 14, 19, 20, 27, 33}},
    {{7, 8, 13, 14, 15, 16, 23, 24, 29, 35}, {1, 2, 9, 10, 11, 12, 17, 18, 25, 32}},
    {{17, 18, 19, 20, 21, 22, 23, 24, 30, 36}, {1, 2, 3, 4, 5, 6, 7, 8, 26, 31}}};
static const int FACE54[3][2][12] = {
    {{5, 10, 15, 17, 20, 25, 26, 31, 33, 36, 41, 46}, {3, 8, 13, 16, 18, 23, 24, 29, 32, 34, 39, 44}},
    {{11, 12, 18, 19, 20, 27, 28, 34, 35, 36, 47, 48}, {1, 2, 13, 14, 15, 21, 22, 29, 30, 31, 37, 38}},
    {{37, 38, 39, 40, 41, 42, 43, 44, 45, 46, 47, 48}, {1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12}}};

typedef struct {
    int mn, me, nord, nface;
    const int *enode, *edir;
    int src[3][12], dst[3][12];
} elem_tab;

static int get_tab(int mn, elem_tab *t) {
    int f, k;
    memset(t, 0, sizeof(*t));
    t->mn = mn;
    switch (mn) {
        case 8:
            t->me = 12; t->nord = 2; t->nface = 4; t->enode = EDGE12_NODE; t->edir = EDGE12_DIR;
            for (f = 0; f < 3; f++) for (k = 0; k < 4; k++) { t->src[f][k] = FACE12[f][0][k]; t->dst[f][k] = FACE12[f][1][k]; }
            return 0;
        case 20:
            t->me = 36; t->nord = 3; t->nface = 10; t->enode = EDGE36_NODE; t->edir = EDGE36_DIR;
            for (f = 0; f < 3; f++) for (k = 0; k < 10; k++) { t->src[f][k] = FACE36[f][0][k]; t->dst[f][k] = FACE36[f][1][k]; }
            return 0;
        case 27:
            t->me = 54; t->nord = 3; t->nface = 12; t->enode = EDGE54_NODE; t->edir = EDGE54_DIR;
            for (f = 0; f < 3; f++) for (k = 0; k < 12; k++) { t->src[f][k] = FACE54[f][0][k]; t->dst[f][k] = FACE54[f][1][k]; }
            return 0;
    }
    return -1;
}

int orc_edges_per_elem(int mn) { return mn == 8 ? 12 : mn == 20 ? 36 : mn == 27 ? 54 : -1; }

int orc_num_nodes(const orc_mesh *m, int32_t *nnx, int32_t *nny, int32_t *nnz, int64_t *npt) {
    int nord = m->nodes_per_elem == 8 ? 2 : 3;
    *nnx = m->nx * (nord - 1) + 1;
    *nny = m->ny * (nord - 1) + 1;
    *nnz = m->nz * (nord - 1) + 1;
    *npt = (int64_t)(*nnx) * (*nny) * (*nnz);
    return 0;
}

/* Rounding applied where the reference uses default-real literals or cmplx() without
 * a kind (integration.f90:84,297-402; problem.f90:112,250,352-356; boundary_conds.f90). */
static double r32(const orc_mesh *m, double v) {
    return (m->quirks & ORC_Q_FP32_CONST) ? (double)(float)v : v;
}

/* ------------------------------------------------- nodal basis (n_fem.f90:138-317) */
static double nf_ln(int mn, int i, double xi, double eta, double zeta) {
    double a = NR[0][i], b = NR[1][i], c = NR[2][i];
    if (mn == 8) return (1 + a * xi) * (1 + b * eta) * (1 + c * zeta) / 8.0;
    if (mn == 20) {
        if (i < 8) return (1 + a * xi) * (1 + b * eta) * (1 + c * zeta) * (a * xi + b * eta + c * zeta - 2) / 8.0;
        if (a == 0) return (1 - xi * xi) * (1 + b * eta) * (1 + c * zeta) / 4.0;
        if (b == 0) return (1 + a * xi) * (1 - eta * eta) * (1 + c * zeta) / 4.0;
        return (1 + a * xi) * (1 + b * eta) * (1 - zeta * zeta) / 4.0;
    }
    /* 27-node: tensor product of 1-D quadratic Lagrange factors */
    {
        double p[3], t[3] = {xi, eta, zeta};
        int d;
        for (d = 0; d < 3; d++) {
            int n = NR[d][i];
            p[d] = n == 0 ? (1 - t[d] * t[d]) : 0.5 * n * t[d] * (1 + n * t[d]);
        }
        return p[0] * p[1] * p[2];
    }
}

static double nf_dln(const orc_mesh *m, int mn, int d, int i, double xi, double eta, double zeta) {
    double a = NR[0][i], b = NR[1][i], c = NR[2][i];
    if (mn == 8) {
        if (d == 0) return a * (1 + b * eta) * (1 + c * zeta) / 8.0;
        if (d == 1) return (1 + a * xi) * b * (1 + c * zeta) / 8.0;
        /* n_fem.f90:193 writes (1+nr1) where (1+nr1*xi) is meant */
        if (m->quirks & ORC_Q_LIN_DZETA) return (1 + a) * (1 + b * eta) * c / 8.0;
        return (1 + a * xi) * (1 + b * eta) * c / 8.0;
    }
    if (mn == 20) {
        if (i < 8) {
            double s = a * xi + b * eta + c * zeta;
            if (d == 0) return (1 + b * eta) * (1 + c * zeta) * a * (2 * a * xi + b * eta + c * zeta - 1) / 8.0;
            if (d == 1) return (1 + a * xi) * (1 + c * zeta) * b * (2 * b * eta + a * xi + c * zeta - 1) / 8.0;
            (void)s;
            return (1 + a * xi) * (1 + b * eta) * c * (2 * c * zeta + a * xi + b * eta - 1) / 8.0;
        }
        if (a == 0) {
            if (d == 0) return -xi * (1 + b * eta) * (1 + c * zeta) / 2.0;
            if (d == 1) return b * (1 - xi * xi) * (1 + c * zeta) / 4.0;
            return c * (1 - xi * xi) * (1 + b * eta) / 4.0;
        }
        if (b == 0) {
            if (d == 0) return a * (1 - eta * eta) * (1 + c * zeta) / 4.0;
            if (d == 1) return -eta * (1 + a * xi) * (1 + c * zeta) / 2.0;
            return c * (1 - eta * eta) * (1 + a * xi) / 4.0;
        }
        if (d == 0) return a * (1 - zeta * zeta) * (1 + b * eta) / 4.0;
        if (d == 1) return b * (1 - zeta * zeta) * (1 + a * xi) / 4.0;
        return -zeta * (1 + a * xi) * (1 + b * eta) / 2.0;
    }
    {
        double p[3], dp[3], t[3] = {xi, eta, zeta};
        int k;
        for (k = 0; k < 3; k++) {
            int n = NR[k][i];
            if (n == 0) { p[k] = 1 - t[k] * t[k]; dp[k] = -2 * t[k]; }
            else { p[k] = 0.5 * n * t[k] * (1 + n * t[k]); dp[k] = 0.5 * n * (1 + 2 * n * t[k]); }
        }
        if (d == 0) return dp[0] * p[1] * p[2];
        if (d == 1) return p[0] * dp[1] * p[2];
        return p[0] * p[1] * dp[2];
    }
}

/* ------------------------------------------- edge (mixed-order) factors (v_fem.f90:78-466) */
/* L(node i, dir) and dL/dxi_d.  dir in 0..2. */
static void mix_ln_grad(int mn, int i, int dir, const double t[3], double *L, double g[3]) {
    int a[3] = {NR[0][i], NR[1][i], NR[2][i]};
    int k;
    if (mn == 8) {
        /* product of (1+n t)/2 over the two axes other than dir */
        double f[3], df[3];
        for (k = 0; k < 3; k++) {
            if (k == dir) { f[k] = 1; df[k] = 0; }
            else { f[k] = 0.5 * (1 + a[k] * t[k]); df[k] = 0.5 * a[k]; }
        }
        *L = f[0] * f[1] * f[2];
        g[0] = df[0] * f[1] * f[2]; g[1] = f[0] * df[1] * f[2]; g[2] = f[0] * f[1] * df[2];
        return;
    }
    if (mn == 20) {
        if (i < 8) {
            /* prod_{k!=dir}(1+a_k t_k) * (sum_k a_k t_k - 1) / 8 */
            double s = a[0] * t[0] + a[1] * t[1] + a[2] * t[2] - 1;
            double f[3];
            for (k = 0; k < 3; k++) f[k] = (k == dir) ? 1 : (1 + a[k] * t[k]);
            *L = f[0] * f[1] * f[2] * s / 8.0;
            for (k = 0; k < 3; k++) {
                double pf = 1, dpf = 0;
                int q;
                for (q = 0; q < 3; q++) {
                    if (q == dir) continue;
                    if (q == k) dpf = a[q]; else pf *= f[q];
                }
                if (k == dir) g[k] = f[0] * f[1] * f[2] * a[k] / 8.0;
                else g[k] = (dpf * pf * s + f[0] * f[1] * f[2] * a[k]) / 8.0;
            }
            return;
        }
        {
            /* mid-edge node: axis z0 with a=0 carries (1-t^2); the remaining axis other
             * than dir carries (1+a t); overall /2 */
            double f[3], df[3];
            for (k = 0; k < 3; k++) {
                if (a[k] == 0) { f[k] = 1 - t[k] * t[k]; df[k] = -2 * t[k]; }
                else if (k == dir) { f[k] = 1; df[k] = 0; }
                else { f[k] = 1 + a[k] * t[k]; df[k] = a[k]; }
            }
            *L = f[0] * f[1] * f[2] / 2.0;
            g[0] = df[0] * f[1] * f[2] / 2.0; g[1] = f[0] * df[1] * f[2] / 2.0; g[2] = f[0] * f[1] * df[2] / 2.0;
            return;
        }
    }
    {
        /* 27-node: along dir (1+a t)/2, other axes 1-D quadratic Lagrange factor */
        double f[3], df[3];
        for (k = 0; k < 3; k++) {
            if (k == dir) { f[k] = 0.5 * (1 + a[k] * t[k]); df[k] = 0.5 * a[k]; }
            else if (a[k] == 0) { f[k] = 1 - t[k] * t[k]; df[k] = -2 * t[k]; }
            else { f[k] = 0.5 * a[k] * t[k] * (1 + a[k] * t[k]); df[k] = 0.5 * a[k] * (1 + 2 * a[k] * t[k]); }
        }
        *L = f[0] * f[1] * f[2];
        g[0] = df[0] * f[1] * f[2]; g[1] = f[0] * df[1] * f[2]; g[2] = f[0] * f[1] * df[2];
    }
}

/* ------------------------------------------------------ element geometry */
typedef struct {
    int mn, nord, me;
    int64_t node[27];
    double re[27][3];
} elem_geo;

static void node_dims(const orc_mesh *m, int nord, int64_t *nnx, int64_t *nny, int64_t *nnz) {
    *nnx = (int64_t)m->nx * (nord - 1) + 1;
    *nny = (int64_t)m->ny * (nord - 1) + 1;
    *nnz = (int64_t)m->nz * (nord - 1) + 1;
}

/* nf_get_r (n_fem.f90:66-102): node coordinates of element (ie,je,ke), 0-based. */
static void get_elem(const orc_mesh *m, const elem_tab *t, int ie, int je, int ke, elem_geo *g) {
    int64_t nnx, nny, nnz;
    int ni;
    node_dims(m, t->nord, &nnx, &nny, &nnz);
    g->mn = t->mn; g->nord = t->nord; g->me = t->me;
    for (ni = 0; ni < t->mn; ni++) {
        int i1 = (NR[0][ni] + 1) * (t->nord - 1) / 2;
        int j1 = (NR[1][ni] + 1) * (t->nord - 1) / 2;
        int k1 = (NR[2][ni] + 1) * (t->nord - 1) / 2;
        int64_t ii = (int64_t)ie * (t->nord - 1) + i1;
        int64_t jj = (int64_t)je * (t->nord - 1) + j1;
        int64_t kk = (int64_t)ke * (t->nord - 1) + k1;
        int64_t id = (ii * nny + jj) * nnz + kk;
        g->node[ni] = id;
        g->re[ni][0] = m->xp[ii];
        g->re[ni][1] = m->yp[jj];
        g->re[ni][2] = m->zp[id];
    }
}

/* nf_jacobian / nf_inv_jac / nf_det (n_fem.f90:355-395) */
static double jacobian(const orc_mesh *m, const elem_geo *g, const double t[3], double J[3][3], double Ji[3][3]) {
    int a, b, l;
    double det, ad;
    for (a = 0; a < 3; a++)
        for (b = 0; b < 3; b++) {
            double s = 0;
            for (l = 0; l < g->mn; l++) s += nf_dln(m, g->mn, a, l, t[0], t[1], t[2]) * g->re[l][b];
            J[a][b] = s;
        }
    det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) + J[0][1] * (J[1][2] * J[2][0] - J[1][0] * J[2][2]) +
          J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    ad = fabs(det);
    Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / ad;
    Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / ad;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / ad;
    Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / ad;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / ad;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / ad;
    Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / ad;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / ad;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / ad;
    return det;
}

/* vf_elem_ve / vf_elem_curl (v_fem.f90:38-60): value and the six curl partials of
 * edge basis function im at reference point t, given the inverse Jacobian there. */
static void edge_basis(const elem_tab *tb, int im, const double t[3], double Ji[3][3], double ve[3], double cv[3][2]) {
    int node = tb->enode[im] - 1, dir = tb->edir[im] - 1;
    double L, gL[3], dni[3], vij[3];
    int a;
    mix_ln_grad(tb->mn, node, dir, t, &L, gL);
    for (a = 0; a < 3; a++) {
        vij[a] = Ji[a][dir];
        dni[a] = Ji[a][0] * gL[0] + Ji[a][1] * gL[1] + Ji[a][2] * gL[2];
    }
    for (a = 0; a < 3; a++) ve[a] = L * vij[a];
    cv[0][0] = dni[1] * vij[2]; cv[0][1] = dni[2] * vij[1];
    cv[1][0] = dni[2] * vij[0]; cv[1][1] = dni[0] * vij[2];
    cv[2][0] = dni[0] * vij[1]; cv[2][1] = dni[1] * vij[0];
}

/* ----------------------------------------------------------- Gauss rule */
/* get_intpoints / get_intweights / int_pts_wgt (integration.f90:267-496): tensor
 * rule, k fastest; abscissae and the 3-point weights are default-real literals. */
static int gauss_rule(const orc_mesh *m, int me, double rw[27][4]) {
    double gp[3], gw[3];
    int n, i, j, k, id = 0;
    if (me == 12) {
        n = 2;
        gp[0] = -r32(m, 0.577350269189625764509148780502); gp[1] = -gp[0];
        gw[0] = gw[1] = 1.0;
    } else {
        n = 3;
        gp[0] = -r32(m, 0.774596669241483377035853079956); gp[1] = 0.0; gp[2] = -gp[0];
        gw[0] = gw[2] = r32(m, 0.555555555555555555555555555556);
        gw[1] = r32(m, 0.888888888888888888888888888889);
    }
    for (i = 0; i < n; i++)
        for (j = 0; j < n; j++)
            for (k = 0; k < n; k++) {
                rw[id][0] = gp[i]; rw[id][1] = gp[j]; rw[id][2] = gp[k];
                rw[id][3] = gw[i] * gw[j] * gw[k];
                id++;
            }
    return id;
}

/* --------------------------------------------------------------- numbering */
static inline int64_t eidx(const orc_mesh *m, int ie, int je, int ke) {
    return ((int64_t)ie * m->ny + je) * m->nz + ke;
}

/* edge_bdary (boundary_conds.f90:262-390): first matching face in the order
 * x-, y-, z-, x+, y+, z+ -> 1..6. */
static int edge_face(const orc_mesh *m, const elem_tab *t, int ie, int je, int ke, int im1) {
    int f, k;
    int cond[6] = {ie == 0, je == 0, ke == 0, ie == m->nx - 1, je == m->ny - 1, ke == m->nz - 1};
    /* face order x-,y-,z- use the dst lists of x,y,z; x+,y+,z+ the src lists */
    const int axis[6] = {2, 1, 0, 2, 1, 0};
    for (f = 0; f < 6; f++) {
        if (!cond[f]) continue;
        for (k = 0; k < t->nface; k++) {
            int v = f < 3 ? t->dst[axis[f]][k] : t->src[axis[f]][k];
            if (v == im1) return f + 1;
        }
    }
    return 0;
}

int32_t orc_numbering(const orc_mesh *m, int32_t *gne) {
    elem_tab t;
    int ie, je, ke, im, k, f;
    int64_t ne = (int64_t)m->nx * m->ny * m->nz;
    int32_t indx = 0, nne = 0;
    if (get_tab(m->nodes_per_elem, &t)) return -1;
    for (ie = 0; ie < m->nx; ie++)
        for (je = 0; je < m->ny; je++)
            for (ke = 0; ke < m->nz; ke++) {
                int64_t e = eidx(m, ie, je, ke);
                int inh[54] = {0};
                int bd;
                /* inherit from the -z, -y, -x neighbours, in that order */
                for (f = 0; f < 3; f++) {
                    int64_t e1;
                    if (f == 0) { if (ke == 0) continue; e1 = eidx(m, ie, je, ke - 1); }
                    else if (f == 1) { if (je == 0) continue; e1 = eidx(m, ie, je - 1, ke); }
                    else { if (ie == 0) continue; e1 = eidx(m, ie - 1, je, ke); }
                    for (k = 0; k < t.nface; k++) {
                        int d = t.dst[f][k] - 1, s = t.src[f][k] - 1;
                        gne[(int64_t)d * ne + e] = gne[(int64_t)s * ne + e1];
                        inh[d] = 1;
                    }
                }
                bd = m->dirichlet && (ie == 0 || ie == m->nx - 1 || je == 0 || je == m->ny - 1 || ke == 0 ||
                                      ke == m->nz - 1);
                for (im = 0; im < t.me; im++) {
                    int face = bd ? edge_face(m, &t, ie, je, ke, im + 1) : 0;
                    if (face) gne[(int64_t)im * ne + e] = -face;
                    else if (!inh[im]) gne[(int64_t)im * ne + e] = ++indx;
                }
            }
    for (k = 0; k < (int)(ne * t.me); k++) if (gne[k] > nne) nne = gne[k];
    return nne;
}

/* Slot map (global_assembly.f90:197-229 and shr_nzindx12/36/54 :477-1906).  The
 * reference's 1,400 lines of per-DOF cases follow one rule, restated here: a row DOF
 * first takes slots for its own free columns; if the DOF lies on a + face, the
 * neighbour across that face inherits the slots of the shared columns for the same
 * DOF's row and takes new slots for its other free columns; a DOF on two + faces
 * does this for both faces (z before y before x) and then for the diagonal
 * neighbour, which inherits first from the first face's neighbour through the second
 * face map, then from the second face's neighbour through the first face map. */
static int face_of(const elem_tab *t, int f, int im1) {
    int k;
    for (k = 0; k < t->nface; k++) if (t->src[f][k] == im1) return k;
    return -1;
}

static void own_fill(int32_t *nz, const int32_t *gne, int64_t ne, int me, int64_t e, int im, int32_t *indx) {
    int jm;
    for (jm = 0; jm < me; jm++) {
        int64_t s;
        if (gne[(int64_t)jm * ne + e] < 0) continue;
        s = e * me * me + (int64_t)im * me + jm;
        if (nz[s] == -1) nz[s] = ++(*indx);
    }
}

static void inherit(int32_t *nz, const elem_tab *t, int me, int f, int64_t esrc, int imsrc, int64_t edst, int imdst) {
    int k;
    for (k = 0; k < t->nface; k++) {
        int64_t s = esrc * me * me + (int64_t)imsrc * me + (t->src[f][k] - 1);
        int64_t d = edst * me * me + (int64_t)imdst * me + (t->dst[f][k] - 1);
        if (nz[d] != -1) continue;
        nz[d] = nz[s];
    }
}

int64_t orc_slot_map(const orc_mesh *m, const int32_t *gne, int32_t *nz) {
    elem_tab t;
    int ie, je, ke, im, f;
    int64_t ne = (int64_t)m->nx * m->ny * m->nz, i, nnze = 0;
    int32_t indx = 0;
    if (get_tab(m->nodes_per_elem, &t)) return -1;
    for (i = 0; i < ne * t.me * t.me; i++) nz[i] = -1;
    for (ie = 0; ie < m->nx; ie++)
        for (je = 0; je < m->ny; je++)
            for (ke = 0; ke < m->nz; ke++) {
                int64_t e = eidx(m, ie, je, ke);
                int has[3] = {ke < m->nz - 1, je < m->ny - 1, ie < m->nx - 1};
                int64_t en[3];
                en[0] = has[0] ? eidx(m, ie, je, ke + 1) : -1;
                en[1] = has[1] ? eidx(m, ie, je + 1, ke) : -1;
                en[2] = has[2] ? eidx(m, ie + 1, je, ke) : -1;
                for (im = 0; im < t.me; im++) {
                    int pos[3], nf = 0, fl[2];
                    if (gne[(int64_t)im * ne + e] < 0) continue;
                    own_fill(nz, gne, ne, t.me, e, im, &indx);
                    for (f = 0; f < 3; f++) {
                        pos[f] = face_of(&t, f, im + 1);
                        if (pos[f] >= 0) fl[nf++] = f;
                    }
                    for (f = 0; f < nf; f++) {
                        int a = fl[f];
                        int im1 = t.dst[a][pos[a]] - 1;
                        if (!has[a]) continue;
                        inherit(nz, &t, t.me, a, e, im, en[a], im1);
                        own_fill(nz, gne, ne, t.me, en[a], im1, &indx);
                    }
                    if (nf == 2 && has[fl[0]] && has[fl[1]]) {
                        int A = fl[0], B = fl[1];
                        int imA = t.dst[A][pos[A]] - 1, imB = t.dst[B][pos[B]] - 1;
                        int pB = face_of(&t, B, imA + 1);
                        int imD = t.dst[B][pB] - 1;
                        int64_t eD;
                        int dI = (A == 2 || B == 2), dJ = (A == 1 || B == 1), dK = (A == 0 || B == 0);
                        eD = eidx(m, ie + dI, je + dJ, ke + dK);
                        inherit(nz, &t, t.me, B, en[A], imA, eD, imD);
                        inherit(nz, &t, t.me, A, en[B], imB, eD, imD);
                        own_fill(nz, gne, ne, t.me, eD, imD, &indx);
                    }
                }
            }
    for (i = 0; i < ne * t.me * t.me; i++) if (nz[i] > nnze) nnze = nz[i];
    return nnze;
}

int orc_coo_coords(const orc_mesh *m, const int32_t *gne, const int32_t *nz, int64_t nnze, int32_t *ia, int32_t *ja) {
    int me = orc_edges_per_elem(m->nodes_per_elem);
    int64_t ne = (int64_t)m->nx * m->ny * m->nz, e, i;
    int im, jm;
    for (i = 0; i < nnze; i++) ia[i] = ja[i] = -1;
    for (e = 0; e < ne; e++)
        for (im = 0; im < me; im++) {
            int32_t gi = gne[(int64_t)im * ne + e];
            if (gi < 0) continue;
            for (jm = 0; jm < me; jm++) {
                int32_t gj = gne[(int64_t)jm * ne + e], s;
                if (gj < 0) continue;
                s = nz[e * me * me + (int64_t)im * me + jm];
                if (s == -1) continue;
                s -= 1;
                if (ia[s] == -1 && ja[s] == -1) { ia[s] = gi; ja[s] = gj; }
                else if (ia[s] != gi || ja[s] != gj) return -1;
            }
        }
    return 0;
}

/* ----------------------------------------------------------- GPML stretch */
/* init_gpml / get_pml / gpml_h (boundary_conds.f90:51-186). */
typedef struct {
    int el_a[3][2], el_b[3][2];
    double za[3][2], zb[3][2];  /* xa/xb, ya/yb, za/zb */
    double omegar[2];
} gpml_ctx;

static void gpml_init(const orc_mesh *m, int nord, gpml_ctx *c) {
    int64_t nnx, nny, nnz;
    int n[3] = {m->nx + 1, m->ny + 1, m->nz + 1}; /* g_nx, g_ny, g_nz */
    int d;
    int64_t id1, id2;
    node_dims(m, nord, &nnx, &nny, &nnz);
    for (d = 0; d < 3; d++) {
        c->el_a[d][0] = m->nextd; c->el_a[d][1] = n[d] - m->nextd;
        c->el_b[d][0] = 1; c->el_b[d][1] = n[d] - 1;
    }
    c->za[0][0] = m->xp[m->nextd * (nord - 1)]; c->za[0][1] = m->xp[nnx - 1 - m->nextd * (nord - 1)];
    c->zb[0][0] = m->xp[0]; c->zb[0][1] = m->xp[nnx - 1];
    c->za[1][0] = m->yp[m->nextd * (nord - 1)]; c->za[1][1] = m->yp[nny - 1 - m->nextd * (nord - 1)];
    c->zb[1][0] = m->yp[0]; c->zb[1][1] = m->yp[nny - 1];
    id1 = (int64_t)m->nextd * (nord - 1);
    id2 = (nnx - 1) * nny * nnz + (nny - 1) * nnz + nnz - 1 - (int64_t)m->nzl_top * (nord - 1);
    c->za[2][0] = m->zp[id1]; c->za[2][1] = m->zp[id2];
    c->zb[2][0] = m->zp[0]; c->zb[2][1] = m->zp[(nnx - 1) * nny * nnz + (nny - 1) * nnz + nnz - 1];
    c->omegar[0] = 2.0 * PI * r32(m, 1.e-5);
    c->omegar[1] = 2.0 * PI * 1.e3;
}

/* get_pml with 1-based element indices */
static void gpml_flags(const gpml_ctx *c, int i1, int j1, int k1, int fl[3]) {
    int idx[3] = {i1, j1, k1}, d;
    for (d = 0; d < 3; d++) {
        fl[d] = 0;
        if (idx[d] >= c->el_a[d][0] && idx[d] <= c->el_b[d][0]) fl[d] = -1;
        if (idx[d] >= c->el_a[d][1] && idx[d] <= c->el_b[d][1]) fl[d] = 1;
    }
}

static void gpml_h(const orc_mesh *m, const gpml_ctx *c, const int fl[3], const double r[3], double omega, cplx h[3]) {
    double ww_pml = fabs(c->omegar[1] - c->omegar[0]);
    double ww = fabs(omega - c->omegar[0]);
    double a0 = m->a0, b0 = m->b0;
    int d;
    if (m->gpml_sch == 1) {
        a0 = 100.0 * (ww / ww_pml);
        b0 = (1.e6 - 1.e-2) * (ww / ww_pml) + 1.e-2;
    }
    for (d = 0; d < 3; d++) {
        int s;
        double rr_pml, rr;
        if (fl[d] == 0) { h[d] = 1.0; continue; }
        s = fl[d] < 0 ? 0 : 1;
        rr_pml = fabs(c->zb[d][s] - c->za[d][s]);
        rr = fabs(r[d] - c->za[d][s]);
        if (m->gpml_sch == 0) {
            double hx0 = 1.0 + a0 * pow(rr / rr_pml, m->nn);
            double sn = sin((PI / 2.0) * (rr / rr_pml));
            double bx = b0 * sn * sn;
            /* hx0*cmplx(1.d0,-bx/(omega*eps)): single-precision cmplx */
            h[d] = hx0 * (r32(m, 1.0) + I * r32(m, -bx / (omega * EPS0)));
        } else {
            /* bx (real) = Re(b0*(rr/rr_pml)**nn / cmplx(a0,omega)), cmplx single precision */
            cplx den = r32(m, a0) + I * r32(m, omega);
            double bx = creal(b0 * pow(rr / rr_pml, m->nn) / den);
            h[d] = 1.0 + I * r32(m, bx);
        }
    }
}

/* --------------------------------------------------- primary fields, Dirichlet */
typedef struct {
    int nl;
    cplx psig[16];
    double zl[16], dl[16];
    cplx cz[16], ez[16];
    double pmu;
} layered_ctx;

/* bd_setmodel + bd_updatemodel (boundary_conds.f90:47-49,396-430) */
static void primary_model(const orc_mesh *m, double omega, layered_ctx *L) {
    int i;
    memset(L, 0, sizeof(*L));
    L->pmu = 4.0 * PI * 1.e-7;
    if (m->inimod == 2) {
        L->nl = 2;
        L->psig[0] = I * r32(m, EPS0 * omega);
        L->psig[1] = r32(m, m->h_sigma) + I * r32(m, EPS0 * omega);
    } else if (m->inimod == 3) {
        L->nl = m->nlayers;
        L->zl[0] = 0;
        for (i = 0; i < L->nl - 1; i++) L->dl[i] = m->l_dz[i];
        for (i = 1; i < L->nl; i++) L->zl[i] = L->zl[i - 1] - L->dl[i - 1];
        for (i = 0; i < L->nl; i++) L->psig[i] = r32(m, m->l_sigma[i]) + I * r32(m, EPS0 * omega);
        /* wait_recursion (boundary_conds.f90:521-553) */
        {
            int nl = L->nl, l;
            cplx g = csqrt(I * (omega * L->pmu * L->psig[nl - 1]));
            L->cz[nl - 1] = 1.0 / g;
            for (l = nl - 2; l >= 0; l--) {
                cplx gl = csqrt(I * (omega * L->pmu * L->psig[l]));
                cplx r = (1.0 - gl * L->cz[l + 1]) / (1.0 + gl * L->cz[l + 1]);
                cplx ex = cexp(-2.0 * gl * L->dl[l]);
                L->cz[l] = (1.0 - r * ex) / (gl * (1.0 + r * ex));
            }
            L->ez[0] = 1.0;
            for (l = 0; l < nl - 1; l++) {
                cplx gl = csqrt(I * (omega * L->pmu * L->psig[l]));
                L->ez[l + 1] = cexp(-gl * L->dl[l]) * (L->ez[l] * L->cz[l + 1] * (1.0 + L->cz[l] * gl)) /
                               (L->cz[l] * (1.0 + L->cz[l + 1] * gl));
            }
        }
    }
}

/* ezl (boundary_conds.f90:558-598) */
static cplx ezl(const layered_ctx *L, double omega, int d, double z) {
    cplx r = 0;
    int l, nl = L->nl;
    for (l = 0; l < nl - 1; l++) {
        if (z <= L->zl[l] && z > L->zl[l + 1]) {
            cplx g = csqrt(I * (omega * L->pmu * L->psig[l]));
            cplx rr = (1.0 - g * L->cz[l + 1]) / (1.0 + g * L->cz[l + 1]);
            if (d == 0)
                r = (L->ez[l] / 2.0) * (1.0 + 1.0 / (L->cz[l] * g)) * (1.0 - rr * cexp(-2.0 * g * (z - L->zl[l + 1]))) *
                    cexp(-g * (L->zl[l] - z));
            else
                r = -(L->ez[l] / 2.0) * (g + 1.0 / L->cz[l]) * (1.0 + rr * cexp(-2.0 * g * (z - L->zl[l + 1]))) *
                    cexp(-g * (L->zl[l] - z));
        }
    }
    if (z <= L->zl[nl - 1]) {
        cplx g = csqrt(I * (omega * L->pmu * L->psig[nl - 1]));
        r = L->ez[nl - 1] * cexp(-g * (L->zl[nl - 1] - z));
        if (d == 1) r = r / (-g);
    }
    return r;
}

/* boundary_conds.f90 p_pfields (:436-516): Ep at node z for both polarisations */
static void boundary_ep(const orc_mesh *m, const layered_ctx *L, double omega, double znode, cplx ep[2][3]) {
    double bb0 = 1.e-9, z = (m->ztop - znode) / 1000.0;
    memset(ep, 0, sizeof(cplx) * 6);
    if (m->inimod == 2) {
        cplx fp;
        if (znode > m->ztop) {
            cplx sa = csqrt(I * (omega * L->pmu * L->psig[0]));
            fp = (1.0 / sa) * (1.0 - z * sa);
        } else {
            cplx sa = csqrt(I * (omega * L->pmu * L->psig[1]));
            fp = (1.0 / sa) * cexp(-z * sa);
        }
        ep[0][0] = (I * r32(m, -2.0 * omega * bb0)) * fp;
        ep[1][1] = (I * r32(m, 2.0 * omega * bb0)) * fp;
    } else if (m->inimod == 3) {
        if (znode > m->ztop) {
            ep[0][0] = (I * r32(m, 2.0 * omega * bb0)) * (L->cz[0] - z);
            ep[1][1] = (I * r32(m, -2.0 * omega * bb0)) * (L->cz[0] - z);
        } else {
            ep[0][0] = (I * r32(m, 2.0 * omega * bb0)) * L->cz[0] * ezl(L, omega, 0, z);
            ep[1][1] = (I * r32(m, -2.0 * omega * bb0)) * L->cz[0] * ezl(L, omega, 0, z);
        }
    }
}

/* f_boundary (boundary_conds.f90:188-250): prescribed DOF value of Dirichlet edge jm
 * on face bd of the current element, both polarisations. */
static void f_boundary(const orc_mesh *m, const elem_tab *t, const elem_geo *g, const layered_ctx *L, double omega,
                       int bd, int jm, cplx out[2]) {
    out[0] = out[1] = 0;
    if (!m->dirichlet || m->inimod == 1) return;
    if (bd == 3 || bd == 6) return;
    {
        int node = t->enode[jm] - 1, dir = t->edir[jm] - 1;
        double tr[3] = {NR[0][node], NR[1][node], NR[2][node]};
        double J[3][3], Ji[3][3];
        cplx ep[2][3];
        jacobian(m, g, tr, J, Ji);
        boundary_ep(m, L, omega, m->zp[g->node[node]], ep);
        out[0] = ep[0][0] * J[dir][0] + ep[0][1] * J[dir][1] + ep[0][2] * J[dir][2];
        out[1] = ep[1][0] * J[dir][0] + ep[1][1] * J[dir][1] + ep[1][2] * J[dir][2];
    }
}

/* ---------------------------------------------------------- tensors */
static double rdet6(const double *a) {
    return a[0] * (a[3] * a[5] - a[4] * a[4]) + a[1] * (a[2] * a[4] - a[1] * a[5]) + a[2] * (a[1] * a[4] - a[3] * a[2]);
}
/* inv_tensor (problem.f90:279-288) */
static int rinv6(const double *a, double *b) {
    double d = rdet6(a);
    if (d == 0.0) return -1;
    b[0] = (a[3] * a[5] - a[4] * a[4]) / d;
    b[1] = (a[2] * a[4] - a[1] * a[5]) / d;
    b[2] = (a[1] * a[4] - a[2] * a[3]) / d;
    b[3] = (a[0] * a[5] - a[2] * a[2]) / d;
    b[4] = (a[2] * a[1] - a[0] * a[4]) / d;
    b[5] = (a[3] * a[0] - a[1] * a[1]) / d;
    return 0;
}
static const int PK[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};

/* ------------------------------------------------------ element integrals */
typedef struct {
    int ngp, me;
    double rw[27][4];
    double wgt[27];
    double mf1[27][6];  /* mu^-1 at g (real) */
    cplx mf2[27][6];    /* sigma at g */
    cplx h[27][3];
    cplx src[27][2][3];
    double ve[27][54][3];
    double cv[27][54][3][2];
} elem_work;

typedef struct {
    int64_t it; /* elements processed so far, for the lag state */
    int last[3];
} lag_state;

/* int_elem_params / int_param / int_edges / p_elem_fields / p_source / p_intmodels
 * (integration.f90:60-152, problem.f90:70-149,257-457). */
static int element_work(const orc_mesh *m, const elem_tab *t, const elem_geo *g, double omega, const int fl[3],
                        const gpml_ctx *gc, elem_work *w) {
    int i, gq, j, d, c;
    double mu0 = 4.0 * PI * 1.e-7;
    double inmu[27][6], dmu[27][6];
    cplx dsig[27][6], ep[27][2][3], hp[27][2][3];
    double w_eps = r32(m, omega * EPS0);
    double w32 = r32(m, omega);
    w->ngp = gauss_rule(m, t->me, w->rw);
    w->me = t->me;
    for (i = 0; i < t->mn; i++) {
        const double *mu = m->mu + g->node[i] * 6;
        const double *sg = m->sigma + g->node[i] * 12;
        double z = m->zp[g->node[i]];
        if (rinv6(mu, inmu[i])) return -2;
        for (c = 0; c < 6; c++) {
            dsig[i][c] = sg[2 * c] + I * sg[2 * c + 1];
            dmu[i][c] = mu[c];
        }
        dsig[i][0] -= I * w_eps; dsig[i][3] -= I * w_eps; dsig[i][5] -= I * w_eps;
        dmu[i][0] -= mu0; dmu[i][3] -= mu0; dmu[i][5] -= mu0;
        memset(ep[i], 0, sizeof(ep[i]));
        memset(hp[i], 0, sizeof(hp[i]));
        ep[i][0][0] = 0.0 - I * r32(m, omega * B0_PRIMARY * z);
        hp[i][0][1] = r32(m, B0_PRIMARY) / (4 * PI * 1.e-7);
        ep[i][1][1] = 0.0 + I * r32(m, omega * B0_PRIMARY * z);
        hp[i][1][0] = r32(m, B0_PRIMARY) / (4 * PI * 1.e-7);
    }
    for (gq = 0; gq < w->ngp; gq++) {
        double *t3 = w->rw[gq];
        double J[3][3], Ji[3][3], Nn[27];
        double det = jacobian(m, g, t3, J, Ji);
        if (det == 0.0) return -1;
        w->wgt[gq] = det * t3[3];
        for (i = 0; i < t->mn; i++) Nn[i] = nf_ln(t->mn, i, t3[0], t3[1], t3[2]);
        for (c = 0; c < 6; c++) { w->mf1[gq][c] = 0; w->mf2[gq][c] = 0; }
        for (i = 0; i < t->mn; i++) {
            const double *sg = m->sigma + g->node[i] * 12;
            for (c = 0; c < 6; c++) {
                w->mf1[gq][c] += Nn[i] * inmu[i][c];
                w->mf2[gq][c] += Nn[i] * (sg[2 * c] + I * sg[2 * c + 1]);
            }
        }
        if (g_pmass_on) pmass_sigma(w->mf2[gq]);
        if (!m->dirichlet) {
            double r[3] = {0, 0, 0};
            for (j = 0; j < t->mn; j++)
                for (c = 0; c < 3; c++) r[c] += Nn[j] * g->re[j][c];
            gpml_h(m, gc, fl, r, omega, w->h[gq]);
        } else {
            w->h[gq][0] = w->h[gq][1] = w->h[gq][2] = 1.0;
        }
        for (d = 0; d < 2; d++) {
            cplx dm[3] = {0, 0, 0}, pc[3] = {0, 0, 0};
            for (i = 0; i < t->mn; i++) {
                cplx v[3];
                double dn[3], gr[3];
                int a, b;
                /* p_dmpf: N_i * (dsigma_i . Ep_i) */
                for (a = 0; a < 3; a++) {
                    v[a] = 0;
                    for (b = 0; b < 3; b++) v[a] += dsig[i][PK[a][b]] * ep[i][d][b];
                    dm[a] += Nn[i] * v[a];
                }
                /* p_pcurl: grad N_i x (mu^-1_i dmu_i Hp_i) */
                for (a = 0; a < 3; a++) gr[a] = nf_dln(m, t->mn, a, i, t3[0], t3[1], t3[2]);
                for (a = 0; a < 3; a++) dn[a] = Ji[a][0] * gr[0] + Ji[a][1] * gr[1] + Ji[a][2] * gr[2];
                for (a = 0; a < 3; a++) {
                    int q;
                    v[a] = 0;
                    for (b = 0; b < 3; b++) {
                        double mm = 0;
                        for (q = 0; q < 3; q++) mm += inmu[i][PK[a][q]] * dmu[i][PK[q][b]];
                        v[a] += mm * hp[i][d][b];
                    }
                }
                pc[0] += v[2] * dn[1] - v[1] * dn[2];
                pc[1] += v[0] * dn[2] - v[2] * dn[0];
                pc[2] += v[1] * dn[0] - v[0] * dn[1];
            }
            for (c = 0; c < 3; c++) w->src[gq][d][c] = (dm[c] + pc[c]) * (0.0 - I * w32);
        }
        for (j = 0; j < t->me; j++) edge_basis(t, j, t3, Ji, w->ve[gq][j], w->cv[gq][j]);
    }
    return 0;
}

/* derivative axis of curl partial (component c, partial p) */
static const int DAX[3][2] = {{1, 2}, {2, 0}, {0, 1}};

/* f1 / f2 / f3 (integration.f90:154-265) -> element K, M, b */
static void element_integrals(const orc_mesh *m, const elem_work *w, double *K, double *M, cplx *bvec) {
    int me = w->me, im, jm, gq, c, p, d, q, pol;
    for (im = 0; im < me; im++)
        for (jm = 0; jm < me; jm++) {
            double ks = 0, ms = 0;
            for (gq = 0; gq < w->ngp; gq++) {
                double f1, f2;
                if (m->dirichlet) {
                    double s1 = 0, s2 = 0;
                    for (c = 0; c < 3; c++)
                        for (d = 0; d < 3; d++) {
                            double mc = w->mf1[gq][PK[c][d]];
                            double ci = w->cv[gq][im][c][0] - w->cv[gq][im][c][1];
                            double cj = w->cv[gq][jm][d][0] - w->cv[gq][jm][d][1];
                            s1 += mc * ci * cj;
                            s2 += w->ve[gq][jm][d] * creal(w->mf2[gq][PK[c][d]]) * w->ve[gq][im][c];
                        }
                    f1 = s1; f2 = s2;
                } else {
                    const cplx *h = w->h[gq];
                    cplx s1 = 0, s2 = 0, H = h[0] * h[1] * h[2];
                    for (c = 0; c < 3; c++)
                        for (p = 0; p < 2; p++)
                            for (d = 0; d < 3; d++)
                                for (q = 0; q < 2; q++) {
                                    int a1 = DAX[c][p], a2 = DAX[d][q];
                                    cplx coef;
                                    if (a1 == a2) {
                                        int o1 = (a1 + 1) % 3, o2 = (a1 + 2) % 3;
                                        if (o1 > o2) { int tt = o1; o1 = o2; o2 = tt; }
                                        coef = h[o1] * h[o2] / h[a1];
                                    } else {
                                        coef = h[3 - a1 - a2];
                                    }
                                    if ((p + q) & 1) coef = -coef;
                                    s1 += coef * w->mf1[gq][PK[c][d]] * w->cv[gq][im][c][p] * w->cv[gq][jm][d][q];
                                }
                    for (c = 0; c < 3; c++)
                        for (d = 0; d < 3; d++) s2 += H * w->ve[gq][jm][d] * w->mf2[gq][PK[c][d]] * w->ve[gq][im][c];
                    f1 = creal(s1); f2 = creal(s2);
                }
                ks += w->wgt[gq] * f1;
                ms += w->wgt[gq] * f2;
            }
            K[im * me + jm] = ks;
            M[im * me + jm] = ms;
        }
    for (im = 0; im < me; im++)
        for (pol = 0; pol < 2; pol++) {
            cplx s = 0;
            for (gq = 0; gq < w->ngp; gq++) {
                cplx H = m->dirichlet ? 1.0 : w->h[gq][0] * w->h[gq][1] * w->h[gq][2];
                cplx f3 = 0;
                for (c = 0; c < 3; c++) f3 += (m->dirichlet ? 1.0 : H) * w->ve[gq][im][c] * w->src[gq][pol][c];
                s += w->wgt[gq] * f3;
            }
            bvec[im * 2 + pol] = s;
        }
}

/* zone flags an element is assembled with: those of the previous element in loop
 * order (lag quirk) or its own. */
static void applied_flags(const orc_mesh *m, const gpml_ctx *gc, int ie, int je, int ke, int ifreq, int fl[3]) {
    fl[0] = fl[1] = fl[2] = 0;
    if (m->dirichlet) return;
    if (m->quirks & ORC_Q_GPML_LAG) {
        int pi = ie, pj = je, pk = ke - 1;
        if (pk < 0) { pk = m->nz - 1; pj--; }
        if (pj < 0) { pj = m->ny - 1; pi--; }
        if (pi < 0) {
            /* first element: the module variable in_pml starts at zero and, from the
             * second frequency on, still holds the last element's flags */
            if (ifreq == 0) return;
            pi = m->nx - 1; pj = m->ny - 1; pk = m->nz - 1;
        }
        gpml_flags(gc, pi + 1, pj + 1, pk + 1, fl);
    } else {
        gpml_flags(gc, ie + 1, je + 1, ke + 1, fl);
    }
}

int orc_element(const orc_mesh *m, int64_t e, double omega, int32_t ifreq, double *K, double *M, double *b,
                int32_t *pml_out) {
    elem_tab t;
    elem_geo g;
    gpml_ctx gc;
    elem_work *w;
    int fl[3], rc, ie, je, ke;
    if (get_tab(m->nodes_per_elem, &t)) return -1;
    ie = (int)(e / ((int64_t)m->ny * m->nz));
    je = (int)((e / m->nz) % m->ny);
    ke = (int)(e % m->nz);
    get_elem(m, &t, ie, je, ke, &g);
    if (!m->dirichlet) gpml_init(m, t.nord, &gc);
    applied_flags(m, &gc, ie, je, ke, ifreq, fl);
    if (pml_out) { pml_out[0] = fl[0]; pml_out[1] = fl[1]; pml_out[2] = fl[2]; }
    w = (elem_work *)malloc(sizeof(elem_work));
    rc = element_work(m, &t, &g, omega, fl, &gc, w);
    if (!rc) element_integrals(m, w, K, M, (cplx *)b);
    free(w);
    return rc;
}

/* global_vfem / local_vfem (MoVFEM_3DMT.f90:167-263), no sort (Q1 excluded). */
int orc_assemble(const orc_mesh *m, const int32_t *gne, const int32_t *nz, int64_t nnze, int32_t nne, double omega,
                 int32_t ifreq, double *a, double *rhs) {
    elem_tab t;
    elem_geo g;
    gpml_ctx gc;
    layered_ctx L;
    elem_work *w;
    int ie, je, ke, im, jm, me, fl[3];
    int64_t ne = (int64_t)m->nx * m->ny * m->nz, i;
    double *K, *M;
    cplx *b;
    cplx *A = (cplx *)a, *R = (cplx *)rhs;
    double w32 = r32(m, omega);
    if (get_tab(m->nodes_per_elem, &t)) return -1;
    me = t.me;
    if (!m->dirichlet) gpml_init(m, t.nord, &gc);
    primary_model(m, omega, &L);
    w = (elem_work *)malloc(sizeof(elem_work));
    K = (double *)malloc(sizeof(double) * me * me);
    M = (double *)malloc(sizeof(double) * me * me);
    b = (cplx *)malloc(sizeof(cplx) * me * 2);
    for (i = 0; i < nnze; i++) A[i] = 0;
    for (i = 0; i < 2 * (int64_t)nne; i++) R[i] = 0;
    for (ie = 0; ie < m->nx; ie++)
        for (je = 0; je < m->ny; je++)
            for (ke = 0; ke < m->nz; ke++) {
                int64_t e = eidx(m, ie, je, ke);
                int rc;
                get_elem(m, &t, ie, je, ke, &g);
                applied_flags(m, &gc, ie, je, ke, ifreq, fl);
                rc = element_work(m, &t, &g, omega, fl, &gc, w);
                if (rc) { free(w); free(K); free(M); free(b); return rc; }
                element_integrals(m, w, K, M, b);
                for (im = 0; im < me; im++) {
                    int32_t gi = gne[(int64_t)im * ne + e];
                    cplx lift[2] = {0, 0};
                    if (gi < 0) continue;
                    for (jm = 0; jm < me; jm++) {
                        int32_t gj = gne[(int64_t)jm * ne + e];
                        cplx aij = K[im * me + jm] + (I * w32) * M[im * me + jm];
                        if (gj < 0) {
                            cplx fb[2];
                            f_boundary(m, &t, &g, &L, omega, -gj, jm, fb);
                            lift[0] += fb[0] * aij;
                            lift[1] += fb[1] * aij;
                            continue;
                        }
                        if (gi < gj) continue;
                        {
                            int32_t s = nz[e * me * me + (int64_t)im * me + jm];
                            if (s < 1) { free(w); free(K); free(M); free(b); return -3; }
                            A[s - 1] += aij;
                        }
                    }
                    R[gi - 1] += b[im * 2 + 0] - lift[0];
                    R[(int64_t)nne + gi - 1] += b[im * 2 + 1] - lift[1];
                }
            }
    free(w); free(K); free(M); free(b);
    return 0;
}

/* ------------------------------------------------------- post-processing */
/* First element (reference loop order) that visits global node-grid position. */
static int first_elem_axis(int IX, int nord, int nel) {
    int e = (IX == 0) ? 0 : (IX - 1) / (nord - 1);
    if (e >= nel) e = nel - 1;
    return e;
}

/* E (secondary + primary) at a node, from its first visiting element
 * (solution.f90:207-241,304-343; problem.f90:151-168). */
static void node_E(const orc_mesh *m, const elem_tab *t, const int32_t *gne, int32_t nne, double omega,
                   const layered_ctx *L, const cplx *x, int64_t IX, int64_t JY, int64_t Kk, cplx E[2][3]) {
    int nord = t->nord;
    int ie = first_elem_axis((int)IX, nord, m->nx), je = first_elem_axis((int)JY, nord, m->ny),
        ke = first_elem_axis((int)Kk, nord, m->nz);
    int64_t ne = (int64_t)m->nx * m->ny * m->nz, e = eidx(m, ie, je, ke);
    elem_geo g;
    double r[3], Jm[3][3], Ji[3][3];
    int im, pol, c, i;
    get_elem(m, t, ie, je, ke, &g);
    r[0] = -1.0 + 2.0 * (double)(IX - (int64_t)ie * (nord - 1)) / (nord - 1);
    r[1] = -1.0 + 2.0 * (double)(JY - (int64_t)je * (nord - 1)) / (nord - 1);
    r[2] = -1.0 + 2.0 * (double)(Kk - (int64_t)ke * (nord - 1)) / (nord - 1);
    jacobian(m, &g, r, Jm, Ji);
    for (pol = 0; pol < 2; pol++) for (c = 0; c < 3; c++) E[pol][c] = 0;
    for (im = 0; im < t->me; im++) {
        double ve[3], cv[3][2];
        int32_t gi = gne[(int64_t)im * ne + e];
        cplx f[2];
        edge_basis(t, im, r, Ji, ve, cv);
        if (gi < 0) f_boundary(m, t, &g, L, omega, -gi, im, f);
        else { f[0] = x[gi - 1]; f[1] = x[(int64_t)nne + gi - 1]; }
        for (pol = 0; pol < 2; pol++)
            for (c = 0; c < 3; c++) E[pol][c] += f[pol] * ve[c];
    }
    /* get_ep: primary field interpolated with the nodal functions */
    for (i = 0; i < t->mn; i++) {
        double Nn = nf_ln(t->mn, i, r[0], r[1], r[2]);
        double z = m->zp[g.node[i]];
        cplx e1 = 0.0 - I * r32(m, omega * B0_PRIMARY * z);
        cplx e2 = 0.0 + I * r32(m, omega * B0_PRIMARY * z);
        E[0][0] += e1 * Nn;
        E[1][1] += e2 * Nn;
    }
}

/* H at a node from its first visiting element (solution.f90:242-260,370-416). */
static int node_H(const orc_mesh *m, const elem_tab *t, const int32_t *gne, int32_t nne, double omega,
                  const layered_ctx *L, const cplx *x, int64_t IX, int64_t JY, int64_t Kk, cplx H[2][3]) {
    int nord = t->nord;
    int ie = first_elem_axis((int)IX, nord, m->nx), je = first_elem_axis((int)JY, nord, m->ny),
        ke = first_elem_axis((int)Kk, nord, m->nz);
    int64_t nnx, nny, nnz;
    elem_geo g;
    double r[3], Jm[3][3], Ji[3][3], mf1[6] = {0, 0, 0, 0, 0, 0};
    cplx ef[2][3] = {{0, 0, 0}, {0, 0, 0}};
    int i, pol, c;
    node_dims(m, nord, &nnx, &nny, &nnz);
    get_elem(m, t, ie, je, ke, &g);
    r[0] = -1.0 + 2.0 * (double)(IX - (int64_t)ie * (nord - 1)) / (nord - 1);
    r[1] = -1.0 + 2.0 * (double)(JY - (int64_t)je * (nord - 1)) / (nord - 1);
    r[2] = -1.0 + 2.0 * (double)(Kk - (int64_t)ke * (nord - 1)) / (nord - 1);
    jacobian(m, &g, r, Jm, Ji);
    for (i = 0; i < t->mn; i++) {
        int64_t id = g.node[i];
        int64_t Ii = id / (nny * nnz), Jj = (id / nnz) % nny, Kz = id % nnz;
        cplx En[2][3];
        double gr[3], dn[3], inmu[6], Nn;
        node_E(m, t, gne, nne, omega, L, x, Ii, Jj, Kz, En);
        for (c = 0; c < 3; c++) gr[c] = nf_dln(m, t->mn, c, i, r[0], r[1], r[2]);
        for (c = 0; c < 3; c++) dn[c] = Ji[c][0] * gr[0] + Ji[c][1] * gr[1] + Ji[c][2] * gr[2];
        for (pol = 0; pol < 2; pol++) {
            ef[pol][0] += En[pol][2] * dn[1] - En[pol][1] * dn[2];
            ef[pol][1] += En[pol][0] * dn[2] - En[pol][2] * dn[0];
            ef[pol][2] += En[pol][1] * dn[0] - En[pol][0] * dn[1];
        }
        if (rinv6(m->mu + id * 6, inmu)) return -2;
        Nn = nf_ln(t->mn, i, r[0], r[1], r[2]);
        for (c = 0; c < 6; c++) mf1[c] += Nn * inmu[c];
    }
    for (pol = 0; pol < 2; pol++) {
        cplx md[6];
        cplx fac = 0.0 + I * r32(m, -1.0 / omega);
        for (c = 0; c < 6; c++) md[c] = fac * mf1[c];
        H[pol][0] = md[0] * ef[pol][0] + md[1] * ef[pol][1] + md[2] * ef[pol][2];
        H[pol][1] = md[1] * ef[pol][0] + md[3] * ef[pol][1] + md[4] * ef[pol][2];
        H[pol][2] = md[2] * ef[pol][0] + md[4] * ef[pol][1] + md[5] * ef[pol][2];
    }
    return 0;
}

/* get_impedance / inv_matrix / get_res_phase (solution.f90:456-505) */
static void impedance(double omega, const cplx e[4], const cplx h[4], cplx z[4], double rho[4], double phi[4]) {
    cplx det = h[0] * h[3] - h[1] * h[2];
    cplx ih[4] = {h[3] / det, -h[1] / det, -h[2] / det, h[0] / det};
    double mu0 = 4 * PI * 1.e-7;
    int i;
    z[0] = ih[0] * e[0] + ih[2] * e[1];
    z[1] = ih[1] * e[0] + ih[3] * e[1];
    z[2] = ih[0] * e[2] + ih[2] * e[3];
    z[3] = ih[1] * e[2] + ih[3] * e[3];
    for (i = 0; i < 4; i++) {
        rho[i] = (1.0 / (omega * mu0)) * (creal(z[i]) * creal(z[i]) + cimag(z[i]) * cimag(z[i]));
        if (rho[i] < 1.e-2) { rho[i] = 0; phi[i] = 0; }
        else phi[i] = atan(cimag(z[i]) / creal(z[i])) * (180.0 / PI);
    }
}

int orc_receivers(const orc_mesh *m, const int32_t *gne, int32_t nne, double omega, const double *xs, int32_t nrx,
                  const double *xr, const double *yr, double *Eo, double *Ho, double *Zo, double *rho, double *phi) {
    elem_tab t;
    layered_ctx L;
    int64_t nnx, nny, nnz;
    const cplx *x = (const cplx *)xs;
    int r;
    if (get_tab(m->nodes_per_elem, &t)) return -1;
    node_dims(m, t.nord, &nnx, &nny, &nnz);
    primary_model(m, omega, &L);
    for (r = 0; r < nrx; r++) {
        /* get_rx_element (receiver_data.f90:187-209): element column of the receiver in
         * the inner grid, top earth layer */
        int ie = -1, je = -1, ke, a, b, pol, c;
        double x1, x2, y1, y2, X = xr[r], Y = yr[r];
        cplx Ec[2][2][2][3], Hc[2][2][2][3], E[2][3], Hh[2][3];
        int i;
        for (i = m->nextd; i <= m->nx - 1 - m->nextd; i++) {
            int ii1 = i * (t.nord - 1), ii2 = ii1 + t.nord - 1;
            if (X >= m->xp[ii1] && X < m->xp[ii2]) ie = i;
        }
        for (i = m->nextd; i <= m->ny - 1 - m->nextd; i++) {
            int jj1 = i * (t.nord - 1), jj2 = jj1 + t.nord - 1;
            if (Y >= m->yp[jj1] && Y < m->yp[jj2]) je = i;
        }
        if (ie < 0 || je < 0) return -4;
        ke = m->nz - m->nzl_top - m->nzl_air - 1;
        x1 = m->xp[ie * (t.nord - 1)]; x2 = m->xp[ie * (t.nord - 1) + t.nord - 1];
        y1 = m->yp[je * (t.nord - 1)]; y2 = m->yp[je * (t.nord - 1) + t.nord - 1];
        for (a = 0; a < 2; a++)
            for (b = 0; b < 2; b++) {
                int64_t IX = (int64_t)ie * (t.nord - 1) + a * (t.nord - 1);
                int64_t JY = (int64_t)je * (t.nord - 1) + b * (t.nord - 1);
                int64_t Kk = (int64_t)ke * (t.nord - 1) + (t.nord - 1);
                node_E(m, &t, gne, nne, omega, &L, x, IX, JY, Kk, Ec[a][b]);
                if (node_H(m, &t, gne, nne, omega, &L, x, IX, JY, Kk, Hc[a][b])) return -2;
            }
        for (pol = 0; pol < 2; pol++)
            for (c = 0; c < 3; c++) {
                cplx fx1 = ((x2 - X) / (x2 - x1)) * Ec[0][0][pol][c] + ((X - x1) / (x2 - x1)) * Ec[1][0][pol][c];
                cplx fx2 = ((x2 - X) / (x2 - x1)) * Ec[0][1][pol][c] + ((X - x1) / (x2 - x1)) * Ec[1][1][pol][c];
                cplx hx1 = ((x2 - X) / (x2 - x1)) * Hc[0][0][pol][c] + ((X - x1) / (x2 - x1)) * Hc[1][0][pol][c];
                cplx hx2 = ((x2 - X) / (x2 - x1)) * Hc[0][1][pol][c] + ((X - x1) / (x2 - x1)) * Hc[1][1][pol][c];
                E[pol][c] = ((y2 - Y) / (y2 - y1)) * fx1 + ((Y - y1) / (y2 - y1)) * fx2;
                Hh[pol][c] = ((y2 - Y) / (y2 - y1)) * hx1 + ((Y - y1) / (y2 - y1)) * hx2;
            }
        {
            cplx ev[4] = {E[0][0], E[1][0], E[0][1], E[1][1]};
            cplx hv[4] = {Hh[0][0], Hh[1][0], Hh[0][1], Hh[1][1]};
            cplx z[4];
            impedance(omega, ev, hv, z, rho + 4 * r, phi + 4 * r);
            for (i = 0; i < 4; i++) { Zo[8 * r + 2 * i] = creal(z[i]); Zo[8 * r + 2 * i + 1] = cimag(z[i]); }
        }
        if (Eo)
            for (pol = 0; pol < 2; pol++)
                for (c = 0; c < 3; c++) {
                    Eo[((r * 2 + pol) * 3 + c) * 2] = creal(E[pol][c]);
                    Eo[((r * 2 + pol) * 3 + c) * 2 + 1] = cimag(E[pol][c]);
                }
        if (Ho)
            for (pol = 0; pol < 2; pol++)
                for (c = 0; c < 3; c++) {
                    Ho[((r * 2 + pol) * 3 + c) * 2] = creal(Hh[pol][c]);
                    Ho[((r * 2 + pol) * 3 + c) * 2 + 1] = cimag(Hh[pol][c]);
                }
    }
    return 0;
}

/* node_solution + z_rho_phi (solution.f90:18-69): E and H at every node (first
 * visiting element), then Z, rho, phi from the node's own horizontal fields
 * (hor_fields, solution.f90:440-455).  E, H: [npt][2][3] complex; Z [npt][4] complex;
 * rho, phi [npt][4].  Any output may be NULL. */
int orc_node_fields(const orc_mesh *m, const int32_t *gne, int32_t nne, double omega, const double *xs, double *Eo,
                    double *Ho, double *Zo, double *rho, double *phi) {
    elem_tab t;
    layered_ctx L;
    int64_t nnx, nny, nnz, id;
    const cplx *x = (const cplx *)xs;
    if (get_tab(m->nodes_per_elem, &t)) return -1;
    node_dims(m, t.nord, &nnx, &nny, &nnz);
    primary_model(m, omega, &L);
    for (id = 0; id < nnx * nny * nnz; id++) {
        int64_t IX = id / (nny * nnz), JY = (id / nnz) % nny, Kk = id % nnz;
        cplx E[2][3], H[2][3], z[4];
        double rr[4], pp[4];
        int pol, c, i;
        node_E(m, &t, gne, nne, omega, &L, x, IX, JY, Kk, E);
        if (node_H(m, &t, gne, nne, omega, &L, x, IX, JY, Kk, H)) return -2;
        {
            cplx ev[4] = {E[0][0], E[1][0], E[0][1], E[1][1]};
            cplx hv[4] = {H[0][0], H[1][0], H[0][1], H[1][1]};
            impedance(omega, ev, hv, z, rr, pp);
        }
        for (pol = 0; pol < 2; pol++)
            for (c = 0; c < 3; c++) {
                if (Eo) { Eo[((id * 2 + pol) * 3 + c) * 2] = creal(E[pol][c]); Eo[((id * 2 + pol) * 3 + c) * 2 + 1] = cimag(E[pol][c]); }
                if (Ho) { Ho[((id * 2 + pol) * 3 + c) * 2] = creal(H[pol][c]); Ho[((id * 2 + pol) * 3 + c) * 2 + 1] = cimag(H[pol][c]); }
            }
        for (i = 0; i < 4; i++) {
            if (Zo) { Zo[(id * 4 + i) * 2] = creal(z[i]); Zo[(id * 4 + i) * 2 + 1] = cimag(z[i]); }
            if (rho) rho[id * 4 + i] = rr[i];
            if (phi) phi[id * 4 + i] = pp[i];
        }
    }
    return 0;
}

/* vf_check_sharing (v_fem.f90:556-863): basis vectors of the DOFs shared across each
 * - face, evaluated at the DOF's own node in both elements. */
double orc_check_sharing(const orc_mesh *m) {
    elem_tab t;
    int ie, je, ke, f, k, a;
    double worst = 0;
    if (get_tab(m->nodes_per_elem, &t)) return -1;
    for (ie = 0; ie < m->nx; ie++)
        for (je = 0; je < m->ny; je++)
            for (ke = 0; ke < m->nz; ke++) {
                elem_geo g2, g1;
                get_elem(m, &t, ie, je, ke, &g2);
                for (f = 0; f < 3; f++) {
                    int pi = ie, pj = je, pk = ke;
                    if (f == 0) { if (ke == 0) continue; pk--; }
                    if (f == 1) { if (je == 0) continue; pj--; }
                    if (f == 2) { if (ie == 0) continue; pi--; }
                    get_elem(m, &t, pi, pj, pk, &g1);
                    for (k = 0; k < t.nface; k++) {
                        int d2 = t.dst[f][k] - 1, s1 = t.src[f][k] - 1;
                        int n2 = t.enode[d2] - 1, n1 = t.enode[s1] - 1;
                        double r2[3] = {NR[0][n2], NR[1][n2], NR[2][n2]};
                        double r1[3] = {NR[0][n1], NR[1][n1], NR[2][n1]};
                        double J[3][3], Ji[3][3], v2[3], v1[3], cv[3][2];
                        jacobian(m, &g2, r2, J, Ji);
                        edge_basis(&t, d2, r2, Ji, v2, cv);
                        jacobian(m, &g1, r1, J, Ji);
                        edge_basis(&t, s1, r1, Ji, v1, cv);
                        for (a = 0; a < 3; a++) if (fabs(v2[a] - v1[a]) > worst) worst = fabs(v2[a] - v1[a]);
                    }
                }
            }
    return worst;
}

/* ------------------------------------------------------------------ model mapping */
/* Tensor slot of a model component (assign_model's select case, geometry.f90:1053-1080):
 * (1, j) -> j, (2 or 3, j) -> i + j, 1-based packed (xx, xy, xz, yy, yz, zz). */
static int map_slot(int i, int j) { return i == 1 ? j : i + j; }

static int map_components_ok(int32_t n, const int32_t *ij) {
    int32_t c;
    for (c = 0; c < n; c++)
        if (ij[c] < 1 || ij[c] > 3 || ij[n + c] < 1 || ij[n + c] > 3) return 0;
    return 1;
}

/* assign_model (geometry.f90:1037-1085): node id takes point p unless already valued.
 * cmplx(0.d0, eps*omega) has the default kind, so ieps arrives FP32-rounded (Q4). */
static void map_assign(const orc_model *md, int64_t p, double ieps, unsigned char *valued, int64_t id,
                       double *sigma, double *mu) {
    const double mu0 = 4.0 * PI * 1.e-7;
    double *s = sigma + id * 12, *u = mu + id * 6;
    int c;
    if (valued[id]) return;
    for (c = 0; c < 12; c++) s[c] = 0.0;
    if (md->isigma == 1) {
        const double v = md->sigma[p];
        s[0] = v; s[1] = ieps;   /* sigma(1) + cmplx(0, eps*omega) */
        s[6] = v; s[7] = ieps;
        s[10] = v; s[11] = ieps;
    } else {
        for (c = 0; c < md->isigma; c++) {
            const int slot = map_slot(md->ijsigma[c], md->ijsigma[md->isigma + c]) - 1;
            s[2 * slot] = md->sigma[p * md->isigma + c];
            s[2 * slot + 1] = 0.0;
        }
        s[0] = s[0] + 0.0; s[1] = s[1] + ieps;
        s[6] = s[6] + 0.0; s[7] = s[7] + ieps;
        s[10] = s[10] + 0.0; s[11] = s[11] + ieps;
    }
    for (c = 0; c < 6; c++) u[c] = 0.0;
    if (md->imu <= 1) {
        /* imu = 0: read_geomodel fills in_mu(1,:) with 1 (read_input.f90:188-190) */
        const double v = mu0 * (md->imu == 0 ? 1.0 : md->mu[p]);
        u[0] = v; u[3] = v; u[5] = v;
    } else {
        for (c = 0; c < md->imu; c++)
            u[map_slot(md->ijmu[c], md->ijmu[md->imu + c]) - 1] = mu0 * md->mu[p * md->imu + c];
    }
    valued[id] = 1;
}

/* min_dd_inner's scan for one node (geometry.f90:971-1031): model points in order,
 * the first within 1e-5 wins (assign_model marks the node valued at once), else the
 * first with the smallest distance.  Returns the point, or -1 if none is below 1e20. */
static int64_t map_search(const orc_model *md, double x, double y, double z) {
    double ddmin = 1.e20;
    int64_t best = -1;
    int32_t im, jm, km;
    for (im = 0; im < md->mx; im++)
        for (jm = 0; jm < md->my; jm++)
            for (km = 0; km < md->mz; km++) {
                const int64_t p = ((int64_t)im * md->my + jm) * md->mz + km;
                const double dx = x - md->xm[im], dy = y - md->ym[jm], dz = z - md->zm[p];
                const double dd = sqrt(dx * dx + dy * dy + dz * dz);
                if (dd <= 1.e-5) return p;
                if (dd < ddmin) { ddmin = dd; best = p; }
            }
    return best;
}

static void map_copy(double *sigma, double *mu, unsigned char *valued, int64_t id, int64_t ip) {
    if (valued[id]) return;
    memcpy(sigma + id * 12, sigma + ip * 12, 12 * sizeof(double));
    memcpy(mu + id * 6, mu + ip * 6, 6 * sizeof(double));
    valued[id] = 1;
}

int orc_map_model(const orc_mesh *m, const orc_model *md, double omega, double *sigma, double *mu) {
    int32_t nnx, nny, nnz;
    int64_t npt, id, nyz;
    const int o = m->nodes_per_elem == 8 ? 1 : 2, nord = o + 1;
    const int nair = m->nzl_top + m->nzl_air, E = m->nextd * o;
    const double ieps = r32(m, EPS0 * omega), mu0 = 4.0 * PI * 1.e-7;
    int ie, je, ke, ii, jj, kk, c;
    int64_t im, jm, km;
    unsigned char *valued;
    if (m->nextd < 1 || nair < 1 || m->nx - 2 * m->nextd < 1 || m->ny - 2 * m->nextd < 1 ||
        m->nz - nair < m->nextd)
        return -1;
    if (md->mx < 1 || md->my < 1 || md->mz < 1 || md->isigma < 1 || md->imu < 0) return -1;
    if (md->isigma > 1 && !map_components_ok(md->isigma, md->ijsigma)) return -1;
    if (md->imu > 1 && !map_components_ok(md->imu, md->ijmu)) return -1;
    orc_num_nodes(m, &nnx, &nny, &nnz, &npt);
    nyz = (int64_t)nny * nnz;
    valued = (unsigned char *)calloc((size_t)npt, 1);
    if (!valued) return -1;
    for (id = 0; id < npt; id++) {  /* g_sigma = cmplx(-1,0); g_mu = -1 */
        for (c = 0; c < 6; c++) {
            sigma[id * 12 + 2 * c] = -1.0;
            sigma[id * 12 + 2 * c + 1] = 0.0;
            mu[id * 6 + c] = -1.0;
        }
    }
    /* element loop (geometry.f90:832-852); 1-based element indices as the reference */
    for (ie = m->nextd + 1; ie <= m->nx - m->nextd; ie++)
        for (je = m->nextd + 1; je <= m->ny - m->nextd; je++)
            for (ke = m->nextd; ke <= m->nz - nair; ke++) {
                const int64_t no = (int64_t)(ie - 1) * o * nyz + (int64_t)(je - 1) * o * nnz + (int64_t)(ke - 1) * o;
                for (ii = 0; ii < nord; ii++)
                    for (jj = 0; jj < nord; jj++)
                        for (kk = 0; kk < nord; kk++) {
                            const int64_t nid = no + ii * nyz + (int64_t)jj * nnz + kk;
                            const int64_t p = map_search(md, m->xp[(ie - 1) * o + ii], m->yp[(je - 1) * o + jj],
                                                         m->zp[nid]);
                            if (p < 0) { free(valued); return -2; }
                            map_assign(md, p, ieps, valued, nid, sigma, mu);
                        }
            }
    /* 1. (y,z) planes (geometry.f90:854-883); k range 1-based [E, nnz - nair*o] */
    for (im = 0; im < E; im++)
        for (jm = E; jm < nny - E; jm++)
            for (km = E - 1; km < nnz - (int64_t)nair * o; km++)
                map_copy(sigma, mu, valued, im * nyz + jm * nnz + km, (int64_t)E * nyz + jm * nnz + km);
    for (im = nnx - E; im < nnx; im++)
        for (jm = E; jm < nny - E; jm++)
            for (km = E - 1; km < nnz - (int64_t)nair * o; km++)
                map_copy(sigma, mu, valued, im * nyz + jm * nnz + km, (int64_t)(nnx - E - 1) * nyz + jm * nnz + km);
    /* 2. (x,z) planes (geometry.f90:885-913) */
    for (im = 0; im < nnx; im++)
        for (jm = 0; jm < E; jm++)
            for (km = E - 1; km < nnz - (int64_t)nair * o; km++)
                map_copy(sigma, mu, valued, im * nyz + jm * nnz + km, im * nyz + (int64_t)E * nnz + km);
    for (im = 0; im < nnx; im++)
        for (jm = nny - E; jm < nny; jm++)
            for (km = E - 1; km < nnz - (int64_t)nair * o; km++)
                map_copy(sigma, mu, valued, im * nyz + jm * nnz + km, im * nyz + (int64_t)(nny - E - 1) * nnz + km);
    /* 3. (x,y) planes below the inner elements (geometry.f90:915-926) */
    for (im = 0; im < nnx; im++)
        for (jm = 0; jm < nny; jm++)
            for (km = 0; km < E - 1; km++)
                map_copy(sigma, mu, valued, im * nyz + jm * nnz + km, im * nyz + jm * nnz + (E - 1));
    /* 4. air (geometry.f90:928-940) */
    for (im = 0; im < nnx; im++)
        for (jm = 0; jm < nny; jm++)
            for (km = nnz - (int64_t)nair * o; km < nnz; km++) {
                id = im * nyz + jm * nnz + km;
                for (c = 0; c < 12; c++) sigma[id * 12 + c] = 0.0;
                for (c = 0; c < 6; c++) mu[id * 6 + c] = 0.0;
                sigma[id * 12 + 1] = ieps; sigma[id * 12 + 7] = ieps; sigma[id * 12 + 11] = ieps;
                mu[id * 6 + 0] = mu0; mu[id * 6 + 3] = mu0; mu[id * 6 + 5] = mu0;
            }
    /* 5. negative entries take the node below (geometry.f90:942-955).  The reference's
     * first node would read before the start of its arrays; it is left as it is. */
    for (id = 1; id < npt; id++)
        for (c = 0; c < 6; c++) {
            if (sigma[id * 12 + 2 * c] < 0) {
                sigma[id * 12 + 2 * c] = sigma[(id - 1) * 12 + 2 * c];
                sigma[id * 12 + 2 * c + 1] = sigma[(id - 1) * 12 + 2 * c + 1];
            }
            if (mu[id * 6 + c] < 0) mu[id * 6 + c] = mu[(id - 1) * 6 + c];
        }
    free(valued);
    return 0;
}
