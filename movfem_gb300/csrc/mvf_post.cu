// mvf_post.cu -- FP64 receiver evaluation on the GPU: nodal E and H
// (node_solution / get_elem_sol / get_er / get_hr, solution.f90:18-49,207-438),
// bilinear interpolation on the top-earth element (rx_data / interpolate_rx,
// receiver_data.f90:111-253) and Z, rho, phi (get_impedance / inv_matrix /
// get_res_phase, solution.f90:456-505).
//
// The reference values a node from the first element, in its (ie, je, ke) loop order,
// that contains it; E uses that element's edge DOFs and H the nodal gradients of that
// element applied to the (first-visitor) E of its nodes.  One CTA per (frequency,
// receiver): threads over (corner, element node) pairs evaluate nodal E, then one
// thread per corner forms H.
#include <cmath>

#include "mvf_internal.cuh"

namespace mvf {

struct PostParams {
    int mn, me, nord, nx, ny, nz;
    int64_t nny, nnz_nodes;
    int32_t nne;
    int r32;
    int q9;
    double omega[MVF_MAX_FREQ];
    // Dirichlet primary models 2/3: boundary-node index and primary field (f_boundary)
    int lift;
    int64_t nb;
    const int32_t *bidx;
    const double2 *bep;
};
__constant__ PostParams c_pp;

__device__ __forceinline__ double p32(double v) { return c_pp.r32 ? (double)__double2float_rn(v) : v; }

__device__ int first_elem(int64_t I, int nel) {
    const int nord = c_pp.nord;
    int e = (I == 0) ? 0 : (int)((I - 1) / (nord - 1));
    return e >= nel ? nel - 1 : e;
}

__device__ void elem_coords(const double *xp, const double *yp, const double *zp, int ie, int je, int ke,
                            double X[MVF_MAX_NODES][3], int64_t ids[MVF_MAX_NODES]) {
    const int nord = c_pp.nord;
    for (int l = 0; l < c_pp.mn; ++l) {
        const int64_t ii = (int64_t)ie * (nord - 1) + (node_ref(l, 0) + 1) * (nord - 1) / 2;
        const int64_t jj = (int64_t)je * (nord - 1) + (node_ref(l, 1) + 1) * (nord - 1) / 2;
        const int64_t kk = (int64_t)ke * (nord - 1) + (node_ref(l, 2) + 1) * (nord - 1) / 2;
        const int64_t id = (ii * c_pp.nny + jj) * c_pp.nnz_nodes + kk;
        ids[l] = id;
        X[l][0] = xp[ii];
        X[l][1] = yp[jj];
        X[l][2] = zp[id];
    }
}

__device__ void jac_inv(const double X[MVF_MAX_NODES][3], const double r[3], double Ji[3][3]) {
    double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int l = 0; l < c_pp.mn; ++l) {
        double N, g[3];
        nodal(c_pp.mn, l, r, N, g, c_pp.q9 != 0);
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) J[a][b] += g[a] * X[l][b];
    }
    const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) + J[0][1] * (J[1][2] * J[2][0] - J[1][0] * J[2][2]) +
                       J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    const double ad = fabs(det);
    Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / ad;
    Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / ad;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / ad;
    Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / ad;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / ad;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / ad;
    Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / ad;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / ad;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / ad;
}

// E (secondary + primary, both polarisations) at global node-grid position (I,J,K)
__device__ void node_E(const double *xp, const double *yp, const double *zp, const int32_t *gne,
                       const int32_t *edge_node, const int32_t *edge_dir, const double2 *x, int f, int64_t I,
                       int64_t J, int64_t K, double2 E[2][3]) {
    const int nord = c_pp.nord;
    const int ie = first_elem(I, c_pp.nx), je = first_elem(J, c_pp.ny), ke = first_elem(K, c_pp.nz);
    double X[MVF_MAX_NODES][3];
    int64_t ids[MVF_MAX_NODES];
    elem_coords(xp, yp, zp, ie, je, ke, X, ids);
    const double r[3] = {-1.0 + 2.0 * (double)(I - (int64_t)ie * (nord - 1)) / (nord - 1),
                         -1.0 + 2.0 * (double)(J - (int64_t)je * (nord - 1)) / (nord - 1),
                         -1.0 + 2.0 * (double)(K - (int64_t)ke * (nord - 1)) / (nord - 1)};
    double Ji[3][3];
    jac_inv(X, r, Ji);
    for (int p = 0; p < 2; ++p)
        for (int a = 0; a < 3; ++a) E[p][a] = make_double2(0.0, 0.0);
    const int64_t e = ((int64_t)ie * c_pp.ny + je) * c_pp.nz + ke;
    const int64_t nne = c_pp.nne;
    for (int j = 0; j < c_pp.me; ++j) {
        const int32_t g = gne[e * c_pp.me + j];
        double2 fb[2] = {make_double2(0.0, 0.0), make_double2(0.0, 0.0)};
        if (g <= 0) {
            // Dirichlet DOF: f_boundary (boundary_conds.f90:188-250), zero for the
            // zero-secondary-field model and on the z faces
            const int bd = -g;
            if (!c_pp.lift || bd == 3 || bd == 6) continue;
            const int nd = edge_node[j], dir = edge_dir[j];
            const int32_t bi = c_pp.bidx[ids[nd]];
            if (bi < 0) continue;
            const double rn[3] = {(double)node_ref(nd, 0), (double)node_ref(nd, 1), (double)node_ref(nd, 2)};
            double jr[2] = {0.0, 0.0};
            for (int l = 0; l < c_pp.mn; ++l) {
                double N, gg[3];
                nodal(c_pp.mn, l, rn, N, gg, c_pp.q9 != 0);
                jr[0] += gg[dir] * X[l][0];
                jr[1] += gg[dir] * X[l][1];
            }
            for (int p = 0; p < 2; ++p) {
                const double2 ep = c_pp.bep[((int64_t)f * c_pp.nb + bi) * 2 + p];
                fb[p] = make_double2(ep.x * jr[p], ep.y * jr[p]);
            }
        }
        double L, gL[3];
        const int dir = edge_dir[j];
        edge_factor(c_pp.mn, edge_node[j], dir, r, L, gL);
        for (int p = 0; p < 2; ++p) {
            const double2 v = g > 0 ? x[((int64_t)f * 2 + p) * nne + (g - 1)] : fb[p];
            for (int a = 0; a < 3; ++a) {
                const double ve = L * Ji[a][dir];
                E[p][a].x += v.x * ve;
                E[p][a].y += v.y * ve;
            }
        }
    }
    // get_ep: primary field interpolated with the nodal functions (problem.f90:151-168)
    const double om = c_pp.omega[f];
    for (int l = 0; l < c_pp.mn; ++l) {
        double N, g[3];
        nodal(c_pp.mn, l, r, N, g, c_pp.q9 != 0);
        const double ez = p32(om * 1.0e-9 * X[l][2]);
        E[0][0].y += -ez * N;
        E[1][1].y += ez * N;
    }
}

__global__ void receivers_kernel(const double *__restrict__ xp, const double *__restrict__ yp,
                                 const double *__restrict__ zp, const double *__restrict__ mu,
                                 const int32_t *__restrict__ gne, const int32_t *__restrict__ edge_node,
                                 const int32_t *__restrict__ edge_dir, const double2 *__restrict__ x, int nrx,
                                 const int *__restrict__ rx_e, const double *__restrict__ rx_xy, double2 *__restrict__ Zo,
                                 double *__restrict__ rho, double *__restrict__ phi, double2 *__restrict__ Eo,
                                 double2 *__restrict__ Ho) {
    const int rx = blockIdx.x % nrx, f = blockIdx.x / nrx;
    const int ie = rx_e[rx * 3 + 0], je = rx_e[rx * 3 + 1], ke = rx_e[rx * 3 + 2];
    const int nord = c_pp.nord, mn = c_pp.mn;
    __shared__ double2 En[4][MVF_MAX_NODES][2][3];  // E at the nodes of each corner's visiting element
    __shared__ double2 Hc[4][2][3], Ec[4][2][3];
    __shared__ double XcS[4][MVF_MAX_NODES][3];  // element of each corner (kept off the thread stack)
    __shared__ int64_t idS[4][MVF_MAX_NODES];
    // corner c = a + 2b: top face of element (ie, je, ke)
    for (int t = threadIdx.x; t < 4 * mn; t += blockDim.x) {
        const int c = t / mn, l = t % mn;
        const int a = c & 1, b = c >> 1;
        const int64_t I = (int64_t)ie * (nord - 1) + a * (nord - 1);
        const int64_t J = (int64_t)je * (nord - 1) + b * (nord - 1);
        const int64_t K = (int64_t)ke * (nord - 1) + (nord - 1);
        // node l of the corner's first-visiting element
        const int fe[3] = {first_elem(I, c_pp.nx), first_elem(J, c_pp.ny), first_elem(K, c_pp.nz)};
        const int64_t Il = (int64_t)fe[0] * (nord - 1) + (node_ref(l, 0) + 1) * (nord - 1) / 2;
        const int64_t Jl = (int64_t)fe[1] * (nord - 1) + (node_ref(l, 1) + 1) * (nord - 1) / 2;
        const int64_t Kl = (int64_t)fe[2] * (nord - 1) + (node_ref(l, 2) + 1) * (nord - 1) / 2;
        double2 E[2][3];
        node_E(xp, yp, zp, gne, edge_node, edge_dir, x, f, Il, Jl, Kl, E);
        for (int p = 0; p < 2; ++p)
            for (int q = 0; q < 3; ++q) En[c][l][p][q] = E[p][q];
        if (Il == I && Jl == J && Kl == K)
            for (int p = 0; p < 2; ++p)
                for (int q = 0; q < 3; ++q) Ec[c][p][q] = E[p][q];
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        const int c = threadIdx.x, a = c & 1, b = c >> 1;
        const int64_t I = (int64_t)ie * (nord - 1) + a * (nord - 1);
        const int64_t J = (int64_t)je * (nord - 1) + b * (nord - 1);
        const int64_t K = (int64_t)ke * (nord - 1) + (nord - 1);
        const int fi = first_elem(I, c_pp.nx), fj = first_elem(J, c_pp.ny), fk = first_elem(K, c_pp.nz);
        double(&X)[MVF_MAX_NODES][3] = XcS[c];
        int64_t(&ids)[MVF_MAX_NODES] = idS[c];
        elem_coords(xp, yp, zp, fi, fj, fk, X, ids);
        const double r[3] = {-1.0 + 2.0 * (double)(I - (int64_t)fi * (nord - 1)) / (nord - 1),
                             -1.0 + 2.0 * (double)(J - (int64_t)fj * (nord - 1)) / (nord - 1),
                             -1.0 + 2.0 * (double)(K - (int64_t)fk * (nord - 1)) / (nord - 1)};
        double Ji[3][3];
        jac_inv(X, r, Ji);
        double2 ef[2][3];
        for (int p = 0; p < 2; ++p)
            for (int q = 0; q < 3; ++q) ef[p][q] = make_double2(0.0, 0.0);
        double mf1[6] = {0, 0, 0, 0, 0, 0};
        for (int l = 0; l < mn; ++l) {
            double N, g[3], dn[3];
            nodal(mn, l, r, N, g, c_pp.q9 != 0);
            for (int q = 0; q < 3; ++q) dn[q] = Ji[q][0] * g[0] + Ji[q][1] * g[1] + Ji[q][2] * g[2];
            for (int p = 0; p < 2; ++p) {
                const double2 *e3 = En[c][l][p];
                ef[p][0].x += e3[2].x * dn[1] - e3[1].x * dn[2];
                ef[p][0].y += e3[2].y * dn[1] - e3[1].y * dn[2];
                ef[p][1].x += e3[0].x * dn[2] - e3[2].x * dn[0];
                ef[p][1].y += e3[0].y * dn[2] - e3[2].y * dn[0];
                ef[p][2].x += e3[1].x * dn[0] - e3[0].x * dn[1];
                ef[p][2].y += e3[1].y * dn[0] - e3[0].y * dn[1];
            }
            const double *m = mu + ids[l] * 6;
            const double det = m[0] * (m[3] * m[5] - m[4] * m[4]) + m[1] * (m[2] * m[4] - m[1] * m[5]) +
                               m[2] * (m[1] * m[4] - m[3] * m[2]);
            const double inv[6] = {(m[3] * m[5] - m[4] * m[4]) / det, (m[2] * m[4] - m[1] * m[5]) / det,
                                   (m[1] * m[4] - m[2] * m[3]) / det, (m[0] * m[5] - m[2] * m[2]) / det,
                                   (m[2] * m[1] - m[0] * m[4]) / det, (m[3] * m[0] - m[1] * m[1]) / det};
            for (int q = 0; q < 6; ++q) mf1[q] += N * inv[q];
        }
        // md = cmplx(0, -1/omega) * mu^-1 (single-precision cmplx)
        const double fac = p32(-1.0 / c_pp.omega[f]);
        const int P[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
        for (int p = 0; p < 2; ++p)
            for (int q = 0; q < 3; ++q) {
                double sr = 0, si = 0;
                for (int s = 0; s < 3; ++s) {
                    // (i fac m) * ef = fac m (-ef.y + i ef.x)
                    sr += -fac * mf1[P[q][s]] * ef[p][s].y;
                    si += fac * mf1[P[q][s]] * ef[p][s].x;
                }
                Hc[c][p][q] = make_double2(sr, si);
            }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const double X = rx_xy[rx * 6 + 0], Y = rx_xy[rx * 6 + 1];
        const double x1 = rx_xy[rx * 6 + 2], x2 = rx_xy[rx * 6 + 3], y1 = rx_xy[rx * 6 + 4], y2 = rx_xy[rx * 6 + 5];
        const double wx1 = (x2 - X) / (x2 - x1), wx2 = (X - x1) / (x2 - x1);
        const double wy1 = (y2 - Y) / (y2 - y1), wy2 = (Y - y1) / (y2 - y1);
        double2 E[2][3], H[2][3];
        for (int p = 0; p < 2; ++p)
            for (int q = 0; q < 3; ++q) {
                // corners: c = a + 2b; f11=(0,0) f21=(1,0) f12=(0,1) f22=(1,1)
                double2 fx1, fx2, hx1, hx2;
                fx1.x = wx1 * Ec[0][p][q].x + wx2 * Ec[1][p][q].x; fx1.y = wx1 * Ec[0][p][q].y + wx2 * Ec[1][p][q].y;
                fx2.x = wx1 * Ec[2][p][q].x + wx2 * Ec[3][p][q].x; fx2.y = wx1 * Ec[2][p][q].y + wx2 * Ec[3][p][q].y;
                hx1.x = wx1 * Hc[0][p][q].x + wx2 * Hc[1][p][q].x; hx1.y = wx1 * Hc[0][p][q].y + wx2 * Hc[1][p][q].y;
                hx2.x = wx1 * Hc[2][p][q].x + wx2 * Hc[3][p][q].x; hx2.y = wx1 * Hc[2][p][q].y + wx2 * Hc[3][p][q].y;
                E[p][q] = make_double2(wy1 * fx1.x + wy2 * fx2.x, wy1 * fx1.y + wy2 * fx2.y);
                H[p][q] = make_double2(wy1 * hx1.x + wy2 * hx2.x, wy1 * hx1.y + wy2 * hx2.y);
            }
        const double2 e[4] = {E[0][0], E[1][0], E[0][1], E[1][1]};
        const double2 h[4] = {H[0][0], H[1][0], H[0][1], H[1][1]};
        auto mul = [](double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); };
        auto dv = [](double2 a, double2 b) {
            const double s = b.x * b.x + b.y * b.y;
            return make_double2((a.x * b.x + a.y * b.y) / s, (a.y * b.x - a.x * b.y) / s);
        };
        const double2 det = make_double2(mul(h[0], h[3]).x - mul(h[1], h[2]).x, mul(h[0], h[3]).y - mul(h[1], h[2]).y);
        const double2 ih[4] = {dv(h[3], det), dv(make_double2(-h[1].x, -h[1].y), det),
                               dv(make_double2(-h[2].x, -h[2].y), det), dv(h[0], det)};
        double2 z[4];
        auto add = [](double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); };
        z[0] = add(mul(ih[0], e[0]), mul(ih[2], e[1]));
        z[1] = add(mul(ih[1], e[0]), mul(ih[3], e[1]));
        z[2] = add(mul(ih[0], e[2]), mul(ih[2], e[3]));
        z[3] = add(mul(ih[1], e[2]), mul(ih[3], e[3]));
        const double pi = 3.1415926535897932384626433, mu0 = 4 * pi * 1.e-7;
        const int o = f * nrx + rx;
        for (int i = 0; i < 4; ++i) {
            Zo[o * 4 + i] = z[i];
            double rr = (1.0 / (c_pp.omega[f] * mu0)) * (z[i].x * z[i].x + z[i].y * z[i].y);
            double ph = 0.0;
            if (rr < 1.e-2) rr = 0.0;
            else ph = atan(z[i].y / z[i].x) * (180.0 / pi);
            rho[o * 4 + i] = rr;
            phi[o * 4 + i] = ph;
        }
        if (Eo)
            for (int p = 0; p < 2; ++p)
                for (int q = 0; q < 3; ++q) Eo[(o * 2 + p) * 3 + q] = E[p][q];
        if (Ho)
            for (int p = 0; p < 2; ++p)
                for (int q = 0; q < 3; ++q) Ho[(o * 2 + p) * 3 + q] = H[p][q];
    }
}

static int set_post_params(Ctx *c) {
    const mvf_mesh &m = c->mesh;
    PostParams pp{};
    pp.mn = c->T.mn; pp.me = c->T.me; pp.nord = c->T.nord;
    pp.nx = m.nx; pp.ny = m.ny; pp.nz = m.nz;
    pp.nny = c->nny; pp.nnz_nodes = c->nnz_nodes; pp.nne = c->nne;
    pp.r32 = (m.quirks & MVF_Q_FP32_CONST) ? 1 : 0;
    pp.q9 = (m.quirks & MVF_Q_LIN_DZETA) ? 1 : 0;
    pp.lift = dirichlet_lift(*c) && c->d.bep ? 1 : 0;
    pp.nb = (int64_t)c->bnode_h.size();
    pp.bidx = c->d.bidx;
    pp.bep = c->d.bep;
    for (int f = 0; f < c->nfreq; ++f) pp.omega[f] = c->omega[f];
    MVF_CUDA(c, cudaMemcpyToSymbolAsync(c_pp, &pp, sizeof pp, 0, cudaMemcpyHostToDevice, c->stream));
    return 0;
}

// ---------------------------------------------------------------- full volume
// node_solution + z_rho_phi (solution.f90:18-69): E at every node from its first
// visiting element, then H from that element's nodal gradients applied to the nodes'
// E (get_hr), and Z, rho, phi from the node's own horizontal fields (hor_fields,
// solution.f90:440-455).  Two launches: E for all nodes, then H and Z.

// Z (z[4]), rho, phi from e = (Ex1, Ex2, Ey1, Ey2), h likewise (get_impedance,
// inv_matrix, get_res_phase: solution.f90:456-505)
__device__ void impedance4(const double2 e[4], const double2 h[4], double omega, double2 z[4], double rho[4],
                           double phi[4]) {
    auto mul = [](double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); };
    auto dv = [](double2 a, double2 b) {
        const double s = b.x * b.x + b.y * b.y;
        return make_double2((a.x * b.x + a.y * b.y) / s, (a.y * b.x - a.x * b.y) / s);
    };
    auto add = [](double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); };
    const double2 det = make_double2(mul(h[0], h[3]).x - mul(h[1], h[2]).x, mul(h[0], h[3]).y - mul(h[1], h[2]).y);
    const double2 ih[4] = {dv(h[3], det), dv(make_double2(-h[1].x, -h[1].y), det),
                           dv(make_double2(-h[2].x, -h[2].y), det), dv(h[0], det)};
    z[0] = add(mul(ih[0], e[0]), mul(ih[2], e[1]));
    z[1] = add(mul(ih[1], e[0]), mul(ih[3], e[1]));
    z[2] = add(mul(ih[0], e[2]), mul(ih[2], e[3]));
    z[3] = add(mul(ih[1], e[2]), mul(ih[3], e[3]));
    const double pi = 3.1415926535897932384626433, mu0 = 4 * pi * 1.e-7;
    for (int i = 0; i < 4; ++i) {
        double rr = (1.0 / (omega * mu0)) * (z[i].x * z[i].x + z[i].y * z[i].y);
        double ph = 0.0;
        if (rr < 1.e-2) rr = 0.0;
        else ph = atan(z[i].y / z[i].x) * (180.0 / pi);
        rho[i] = rr;
        phi[i] = ph;
    }
}

__global__ void node_e_all(const double *__restrict__ xp, const double *__restrict__ yp,
                           const double *__restrict__ zp, const int32_t *__restrict__ gne,
                           const int32_t *__restrict__ edge_node, const int32_t *__restrict__ edge_dir,
                           const double2 *__restrict__ x, int nf, int64_t npt, double2 *__restrict__ Eall) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nf * npt; q += (int64_t)gridDim.x * blockDim.x) {
        const int f = (int)(q / npt);
        const int64_t id = q % npt;
        const int64_t I = id / (c_pp.nny * c_pp.nnz_nodes), J = (id / c_pp.nnz_nodes) % c_pp.nny,
                      K = id % c_pp.nnz_nodes;
        double2 E[2][3];
        node_E(xp, yp, zp, gne, edge_node, edge_dir, x, f, I, J, K, E);
        for (int p = 0; p < 2; ++p)
            for (int a = 0; a < 3; ++a) Eall[(q * 2 + p) * 3 + a] = E[p][a];
    }
}

__global__ void node_h_all(const double *__restrict__ xp, const double *__restrict__ yp,
                           const double *__restrict__ zp, const double *__restrict__ mu, int nf, int64_t npt,
                           const double2 *__restrict__ Eall, double2 *__restrict__ Hall, double2 *__restrict__ Zo,
                           double *__restrict__ rho, double *__restrict__ phi) {
    const int nord = c_pp.nord, mn = c_pp.mn;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nf * npt; q += (int64_t)gridDim.x * blockDim.x) {
        const int f = (int)(q / npt);
        const int64_t id = q % npt;
        const int64_t I = id / (c_pp.nny * c_pp.nnz_nodes), J = (id / c_pp.nnz_nodes) % c_pp.nny,
                      K = id % c_pp.nnz_nodes;
        const int fi = first_elem(I, c_pp.nx), fj = first_elem(J, c_pp.ny), fk = first_elem(K, c_pp.nz);
        double X[MVF_MAX_NODES][3];
        int64_t ids[MVF_MAX_NODES];
        elem_coords(xp, yp, zp, fi, fj, fk, X, ids);
        const double r[3] = {-1.0 + 2.0 * (double)(I - (int64_t)fi * (nord - 1)) / (nord - 1),
                             -1.0 + 2.0 * (double)(J - (int64_t)fj * (nord - 1)) / (nord - 1),
                             -1.0 + 2.0 * (double)(K - (int64_t)fk * (nord - 1)) / (nord - 1)};
        double Ji[3][3];
        jac_inv(X, r, Ji);
        double2 ef[2][3];
        for (int p = 0; p < 2; ++p)
            for (int a = 0; a < 3; ++a) ef[p][a] = make_double2(0.0, 0.0);
        double mf1[6] = {0, 0, 0, 0, 0, 0};
        for (int l = 0; l < mn; ++l) {
            double N, g[3], dn[3];
            nodal(mn, l, r, N, g, c_pp.q9 != 0);
            for (int a = 0; a < 3; ++a) dn[a] = Ji[a][0] * g[0] + Ji[a][1] * g[1] + Ji[a][2] * g[2];
            const double2 *El = Eall + ((int64_t)f * npt + ids[l]) * 6;
            for (int p = 0; p < 2; ++p) {
                const double2 *e3 = El + p * 3;
                ef[p][0].x += e3[2].x * dn[1] - e3[1].x * dn[2];
                ef[p][0].y += e3[2].y * dn[1] - e3[1].y * dn[2];
                ef[p][1].x += e3[0].x * dn[2] - e3[2].x * dn[0];
                ef[p][1].y += e3[0].y * dn[2] - e3[2].y * dn[0];
                ef[p][2].x += e3[1].x * dn[0] - e3[0].x * dn[1];
                ef[p][2].y += e3[1].y * dn[0] - e3[0].y * dn[1];
            }
            const double *m = mu + ids[l] * 6;
            const double det = m[0] * (m[3] * m[5] - m[4] * m[4]) + m[1] * (m[2] * m[4] - m[1] * m[5]) +
                               m[2] * (m[1] * m[4] - m[3] * m[2]);
            const double inv[6] = {(m[3] * m[5] - m[4] * m[4]) / det, (m[2] * m[4] - m[1] * m[5]) / det,
                                   (m[1] * m[4] - m[2] * m[3]) / det, (m[0] * m[5] - m[2] * m[2]) / det,
                                   (m[2] * m[1] - m[0] * m[4]) / det, (m[3] * m[0] - m[1] * m[1]) / det};
            for (int a = 0; a < 6; ++a) mf1[a] += N * inv[a];
        }
        const double fac = p32(-1.0 / c_pp.omega[f]);
        const int P[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
        double2 H[2][3];
        for (int p = 0; p < 2; ++p)
            for (int a = 0; a < 3; ++a) {
                double sr = 0, si = 0;
                for (int b = 0; b < 3; ++b) {
                    sr += -fac * mf1[P[a][b]] * ef[p][b].y;
                    si += fac * mf1[P[a][b]] * ef[p][b].x;
                }
                H[p][a] = make_double2(sr, si);
            }
        if (Hall)
            for (int p = 0; p < 2; ++p)
                for (int a = 0; a < 3; ++a) Hall[(q * 2 + p) * 3 + a] = H[p][a];
        const double2 *Eo = Eall + q * 6;
        const double2 e[4] = {Eo[0], Eo[3], Eo[1], Eo[4]};
        const double2 h[4] = {H[0][0], H[1][0], H[0][1], H[1][1]};
        double2 z[4];
        double rr[4], pp[4];
        impedance4(e, h, c_pp.omega[f], z, rr, pp);
        for (int i = 0; i < 4; ++i) {
            if (Zo) Zo[q * 4 + i] = z[i];
            if (rho) rho[q * 4 + i] = rr[i];
            if (phi) phi[q * 4 + i] = pp[i];
        }
    }
}

}  // namespace mvf

using namespace mvf;

extern "C" int mvf_node_fields(mvf_ctx *xc, double *E, double *H, double *Z, double *rho, double *phi) {
    if (!xc) return MVF_E_ARG;
    Ctx *c = &xc->c;
    if (!c->solved) return fail(c, MVF_E_STATE, "solve before evaluating node fields");
    if (int rc = set_post_params(c)) return rc;
    const int nf = c->nfreq;
    const int64_t npt = c->npt, n = (int64_t)nf * npt;
    double2 *dE = nullptr, *dH = nullptr, *dZ = nullptr;
    double *drho = nullptr, *dphi = nullptr;
    auto cleanup = [&]() {
        cudaFree(dE); cudaFree(dH); cudaFree(dZ); cudaFree(drho); cudaFree(dphi);
    };
    cudaError_t e = cudaMalloc((void **)&dE, n * 6 * sizeof(double2));
    if (e == cudaSuccess && H) e = cudaMalloc((void **)&dH, n * 6 * sizeof(double2));
    if (e == cudaSuccess && Z) e = cudaMalloc((void **)&dZ, n * 4 * sizeof(double2));
    if (e == cudaSuccess && rho) e = cudaMalloc((void **)&drho, n * 4 * sizeof(double));
    if (e == cudaSuccess && phi) e = cudaMalloc((void **)&dphi, n * 4 * sizeof(double));
    if (e != cudaSuccess) {
        cleanup();
        return cuda_fail(c, e, "node field buffers");
    }
    const unsigned grid = (unsigned)std::min<int64_t>((n + 127) / 128, 152 * 32);
    count_launch();
    node_e_all<<<grid, 128, 0, c->stream>>>(c->d.xp, c->d.yp, c->d.zp, c->d.gne, c->d.edge_node, c->d.edge_dir,
                                            (const double2 *)c->d.x, nf, npt, dE);
    count_launch();
    node_h_all<<<grid, 128, 0, c->stream>>>(c->d.xp, c->d.yp, c->d.zp, c->d.mu, nf, npt, dE, dH, dZ, drho, dphi);
    e = cudaGetLastError();
    if (e == cudaSuccess && E) e = cudaMemcpyAsync(E, dE, n * 6 * sizeof(double2), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && H) e = cudaMemcpyAsync(H, dH, n * 6 * sizeof(double2), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && Z) e = cudaMemcpyAsync(Z, dZ, n * 4 * sizeof(double2), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && rho) e = cudaMemcpyAsync(rho, drho, n * 4 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && phi) e = cudaMemcpyAsync(phi, dphi, n * 4 * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    cleanup();
    if (e != cudaSuccess) return cuda_fail(c, e, "node fields");
    return 0;
}

extern "C" int mvf_impedance(mvf_ctx *xc, int32_t nrx, const double *xr, const double *yr, double *Z, double *rho,
                             double *phi, double *E, double *H) {
    if (!xc || nrx < 1 || !xr || !yr || !Z || !rho || !phi) return MVF_E_ARG;
    Ctx *c = &xc->c;
    if (!c->solved) return fail(c, MVF_E_STATE, "solve before evaluating receivers");
    const mvf_mesh &m = c->mesh;
    const int nord = c->T.nord;
    std::vector<int> re(nrx * 3);
    std::vector<double> rxy(nrx * 6);
    // get_rx_element (receiver_data.f90:187-209): element column in the inner grid,
    // top earth layer k = g_nz - g_nzl(g_nsf) - g_nzl(g_nsf-1) - 1
    for (int r = 0; r < nrx; ++r) {
        int ie = -1, je = -1;
        for (int i = m.nextd; i <= m.nx - 1 - m.nextd; ++i)
            if (xr[r] >= c->xp_h[i * (nord - 1)] && xr[r] < c->xp_h[i * (nord - 1) + nord - 1]) ie = i;
        for (int j = m.nextd; j <= m.ny - 1 - m.nextd; ++j)
            if (yr[r] >= c->yp_h[j * (nord - 1)] && yr[r] < c->yp_h[j * (nord - 1) + nord - 1]) je = j;
        const int ke = m.nz - m.nzl_top - m.nzl_air - 1;
        if (ie < 0 || je < 0 || ke < 0) return fail(c, MVF_E_RECEIVER, "receiver " + std::to_string(r) + " outside the inner grid");
        re[r * 3] = ie; re[r * 3 + 1] = je; re[r * 3 + 2] = ke;
        rxy[r * 6 + 0] = xr[r]; rxy[r * 6 + 1] = yr[r];
        rxy[r * 6 + 2] = c->xp_h[ie * (nord - 1)]; rxy[r * 6 + 3] = c->xp_h[ie * (nord - 1) + nord - 1];
        rxy[r * 6 + 4] = c->yp_h[je * (nord - 1)]; rxy[r * 6 + 5] = c->yp_h[je * (nord - 1) + nord - 1];
    }
    if (int rc = set_post_params(c)) return rc;
    int *d_re;
    double *d_rxy, *d_rho, *d_phi;
    double2 *d_Z, *d_E = nullptr, *d_H = nullptr;
    const int nout = c->nfreq * nrx;
    MVF_CUDA(c, cudaMalloc((void **)&d_re, re.size() * sizeof(int)));
    MVF_CUDA(c, cudaMalloc((void **)&d_rxy, rxy.size() * sizeof(double)));
    MVF_CUDA(c, cudaMalloc((void **)&d_Z, (size_t)nout * 4 * sizeof(double2)));
    MVF_CUDA(c, cudaMalloc((void **)&d_rho, (size_t)nout * 4 * sizeof(double)));
    MVF_CUDA(c, cudaMalloc((void **)&d_phi, (size_t)nout * 4 * sizeof(double)));
    if (E) MVF_CUDA(c, cudaMalloc((void **)&d_E, (size_t)nout * 6 * sizeof(double2)));
    if (H) MVF_CUDA(c, cudaMalloc((void **)&d_H, (size_t)nout * 6 * sizeof(double2)));
    MVF_CUDA(c, cudaMemcpyAsync(d_re, re.data(), re.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream));
    MVF_CUDA(c, cudaMemcpyAsync(d_rxy, rxy.data(), rxy.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    count_launch();
    receivers_kernel<<<nout, 128, 0, c->stream>>>(c->d.xp, c->d.yp, c->d.zp, c->d.mu, c->d.gne, c->d.edge_node,
                                                   c->d.edge_dir, (const double2 *)c->d.x, nrx, d_re, d_rxy, d_Z,
                                                   d_rho, d_phi, d_E, d_H);
    MVF_CUDA(c, cudaGetLastError());
    MVF_CUDA(c, cudaMemcpyAsync(Z, d_Z, (size_t)nout * 4 * sizeof(double2), cudaMemcpyDeviceToHost, c->stream));
    MVF_CUDA(c, cudaMemcpyAsync(rho, d_rho, (size_t)nout * 4 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    MVF_CUDA(c, cudaMemcpyAsync(phi, d_phi, (size_t)nout * 4 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (E) MVF_CUDA(c, cudaMemcpyAsync(E, d_E, (size_t)nout * 6 * sizeof(double2), cudaMemcpyDeviceToHost, c->stream));
    if (H) MVF_CUDA(c, cudaMemcpyAsync(H, d_H, (size_t)nout * 6 * sizeof(double2), cudaMemcpyDeviceToHost, c->stream));
    MVF_CUDA(c, cudaStreamSynchronize(c->stream));
    cudaFree(d_re); cudaFree(d_rxy); cudaFree(d_Z); cudaFree(d_rho); cudaFree(d_phi);
    if (d_E) cudaFree(d_E);
    if (d_H) cudaFree(d_H);
    return 0;
}
