// mvf_assemble.cu -- element assembly on the GPU (global_vfem / local_vfem,
// MoVFEM_3DMT.f90:167-263; integrands integration.f90:60-265; physics problem.f90:70-149,
// 247-457; GPML boundary_conds.f90:51-186).
//
// One CTA per element.  For each Gauss point the CTA forms the Jacobian from the
// nodal-derivative table, the material tensors interpolated with the nodal functions
// (sigma and mu^-1 are nodal fields, problem.f90:132-149), the GPML stretch and the
// source term.  Per chunk of Gauss points it stores, per edge DOF, the basis value
// (3), the curl partials (6, or the 3 curl components without GPML) and the same
// vectors premultiplied by the Gauss weight and the material matrix; each thread then
// accumulates a few (i <= j) entries of K_e and M_e in registers.  The element block
// is scattered into the CSR by binary search in each row; elements are launched by
// 2x2x2 parity colour so no two CTAs of a launch touch the same row entry (no
// atomics, deterministic sums).
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>

#include "mvf_internal.cuh"

namespace mvf {

struct GpmlParams {
    int on;          // GPML boundary
    int sch;         // 0 Fang, 1 Zhou
    int lag;         // zone flags of the previous element (MoVFEM_3DMT.f90:203-206)
    int ifreq;       // position of this frequency in the reference's loop
    int nextd;
    double a0, b0, nn;
    double za[3][2], zb[3][2];  // xa/xb, ya/yb, za/zb (boundary_conds.f90:60-63)
    int el_a[3][2], el_b[3][2]; // element zones (boundary_conds.f90:53-55)
    double omegar0, omegar1;    // 2 pi f1, 2 pi f2 (boundary_conds.f90:40,68)
};

struct AsmParams {
    int nx, ny, nz;
    int64_t nny, nnz_nodes;
    int nf;                        // frequencies for the right-hand side
    double omega[MVF_MAX_FREQ];    // rhs frequencies
    double omega_km;               // frequency of K/M (GPML stretch)
    int r32;                       // FP32 constant rounding
    int have_sigma_f;
    int64_t npt;
    GpmlParams g;
    // Dirichlet primary models 2/3: prescribed boundary values lift into b
    int lift, q9;
    int64_t nb;
    const int32_t *bidx;
    const double2 *bep;
    double mg_tau;  // shift tau diag(K_e) of the multilevel preconditioner's mass
    int mg_abs;     // shift the preconditioner's conductivity positive semidefinite
};

__constant__ AsmParams c_ap;
__constant__ int c_glist_n[MVF_MAX_NODES];
__constant__ unsigned char c_glist_i[MVF_MAX_NODES][24];
__constant__ double c_glist_v[MVF_MAX_NODES][24];

__device__ __forceinline__ double rr32(double v) { return c_ap.r32 ? (double)__double2float_rn(v) : v; }

struct cd {
    double re, im;
};
__device__ __forceinline__ cd cmul(cd a, cd b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ __forceinline__ cd cadd(cd a, cd b) { return {a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cd cdiv(cd a, cd b) {
    const double s = b.re * b.re + b.im * b.im;
    return {(a.re * b.re + a.im * b.im) / s, (a.im * b.re - a.re * b.im) / s};
}
__device__ __forceinline__ cd cscale(cd a, double s) { return {a.re * s, a.im * s}; }

static const double PI_D = 3.1415926535897932384626433;
static const double EPS0_D = 8.854187817e-12;

// packed symmetric index
__device__ __forceinline__ int pk(int a, int b) {
    const int t[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
    return t[a][b];
}

// get_pml (boundary_conds.f90:72-82), 1-based element indices
__device__ void zone_flags(const GpmlParams &g, int i1, int j1, int k1, int fl[3]) {
    const int idx[3] = {i1, j1, k1};
    for (int d = 0; d < 3; ++d) {
        fl[d] = 0;
        if (idx[d] >= g.el_a[d][0] && idx[d] <= g.el_b[d][0]) fl[d] = -1;
        if (idx[d] >= g.el_a[d][1] && idx[d] <= g.el_b[d][1]) fl[d] = 1;
    }
}

// gpml_h (boundary_conds.f90:84-186)
__device__ void stretch(const GpmlParams &g, const int fl[3], const double r[3], double omega, cd h[3]) {
    const double ww_pml = fabs(g.omegar1 - g.omegar0);
    const double ww = fabs(omega - g.omegar0);
    double a0 = g.a0, b0 = g.b0;
    if (g.sch == 1) {
        a0 = 100.0 * (ww / ww_pml);
        b0 = (1.e6 - 1.e-2) * (ww / ww_pml) + 1.e-2;
    }
    for (int d = 0; d < 3; ++d) {
        if (fl[d] == 0) { h[d] = {1.0, 0.0}; continue; }
        const int s = fl[d] < 0 ? 0 : 1;
        const double rp = fabs(g.zb[d][s] - g.za[d][s]);
        const double rr = fabs(r[d] - g.za[d][s]);
        if (g.sch == 0) {
            const double hx0 = 1.0 + a0 * pow(rr / rp, g.nn);
            const double sn = sin((PI_D / 2.0) * (rr / rp));
            const double bx = b0 * sn * sn;
            h[d] = {hx0 * rr32(1.0), hx0 * rr32(-bx / (omega * EPS0_D))};
        } else {
            const cd den = {rr32(a0), rr32(omega)};
            const double num = b0 * pow(rr / rp, g.nn);
            const double bx = cdiv({num, 0.0}, den).re;
            h[d] = {1.0, rr32(bx)};
        }
    }
}

template <int MN, int ME, int NGP, bool GPML>
struct Geom {
    static constexpr int GC = NGP == 8 ? 8 : 9;            // Gauss points per chunk
    static constexpr int NCH = NGP / GC;
    static constexpr int CW = GPML ? 6 : 3;               // curl width
    static constexpr int NPAIR = ME * (ME + 1) / 2;
    static constexpr int PPT = (NPAIR + 255) / 256;        // pairs per thread
};

// Shared memory layout (doubles)
template <int MN, int ME, int NGP, bool GPML>
struct Smem {
    using G = Geom<MN, ME, NGP, GPML>;
    double x[MN][3];
    double inmu[MN][6];
    double sig[MVF_MAX_FREQ][MN][12];   // per rhs frequency (complex packed)
    double v[MN][2][3];                  // mu^-1 dmu Hp per polarisation (real)
    double ez[MN];                       // z of the node
    double sigkm[MN][12];                // sigma used by M (current)
    // per Gauss point of the chunk
    double jinv[G::GC][9];
    double wgt[G::GC];
    double dk[G::GC][G::CW][G::CW];      // curl material matrix (times weight)
    double dm[G::GC][3][3];              // mass material matrix (times weight)
    double dmp[G::GC][3][3];             // the same with |sigma| + floor (multilevel preconditioner)
    double srcw[G::GC][MVF_MAX_FREQ][2][6];  // weight*H*source, complex
    double bc[G::GC][ME][G::CW];
    double tc[G::GC][ME][G::CW];
    double bv[G::GC][ME][3];
    double tv[G::GC][ME][3];
    double tvp[G::GC][ME][3];
    int gne[ME];
    int64_t node[MN];
    int err;
};

// local prolongation of the 12-edge space into this element's space (p_local)
__constant__ PLoc c_ploc;

template <int MN, int ME, int NGP, bool GPML>
__global__ void __launch_bounds__(256) element_kernel(
    const int32_t *__restrict__ elems, int64_t nelem, const double *__restrict__ xp, const double *__restrict__ yp,
    const double *__restrict__ zp, const double *__restrict__ sigma, const double *__restrict__ sigma_f,
    const double *__restrict__ mu, const int32_t *__restrict__ gne, const double *__restrict__ tN,
    const double *__restrict__ tdN, const double *__restrict__ tL, const double *__restrict__ tdL,
    const double *__restrict__ tgp, const int32_t *__restrict__ edge_node, const int32_t *__restrict__ edge_dir,
    const int64_t *__restrict__ rowptr, const int32_t *__restrict__ col, double *__restrict__ K64,
    double *__restrict__ M64, double *__restrict__ rhs, int32_t nne, const int32_t *__restrict__ node_gidx,
    double *__restrict__ kphi, double *__restrict__ mphi, double *__restrict__ mabs, double *__restrict__ Kst,
    double *__restrict__ Mst, double *__restrict__ bst, int64_t store_base, int *__restrict__ errflag,
    double *__restrict__ K1e, double *__restrict__ M1e, double *__restrict__ Mp64, double sfloor) {
    using G = Geom<MN, ME, NGP, GPML>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem<MN, ME, NGP, GPML> &S = *reinterpret_cast<Smem<MN, ME, NGP, GPML> *>(smem_raw);
    const int tid = threadIdx.x;
    const int nf = c_ap.nf;
    for (int64_t ei = blockIdx.x; ei < nelem; ei += gridDim.x) {
        const int64_t e = elems ? elems[ei] : store_base + ei;
        const int ie = (int)(e / ((int64_t)c_ap.ny * c_ap.nz));
        const int je = (int)((e / c_ap.nz) % c_ap.ny);
        const int ke = (int)(e % c_ap.nz);
        constexpr int NORD = MN == 8 ? 2 : 3;
        if (tid == 0) S.err = 0;
        // ---- nodes: coordinates, materials, primary fields (p_elem_fields, problem.f90:70-87)
        for (int l = tid; l < MN; l += blockDim.x) {
            const int64_t ii = (int64_t)ie * (NORD - 1) + (node_ref(l, 0) + 1) * (NORD - 1) / 2;
            const int64_t jj = (int64_t)je * (NORD - 1) + (node_ref(l, 1) + 1) * (NORD - 1) / 2;
            const int64_t kk = (int64_t)ke * (NORD - 1) + (node_ref(l, 2) + 1) * (NORD - 1) / 2;
            const int64_t id = (ii * c_ap.nny + jj) * c_ap.nnz_nodes + kk;
            S.node[l] = id;
            S.x[l][0] = xp[ii];
            S.x[l][1] = yp[jj];
            S.x[l][2] = zp[id];
            S.ez[l] = zp[id];
            const double *a = mu + id * 6;
            // inv_tensor (problem.f90:279-288)
            const double det = a[0] * (a[3] * a[5] - a[4] * a[4]) + a[1] * (a[2] * a[4] - a[1] * a[5]) +
                               a[2] * (a[1] * a[4] - a[3] * a[2]);
            if (det == 0.0) S.err = 1;
            double b[6];
            b[0] = (a[3] * a[5] - a[4] * a[4]) / det;
            b[1] = (a[2] * a[4] - a[1] * a[5]) / det;
            b[2] = (a[1] * a[4] - a[2] * a[3]) / det;
            b[3] = (a[0] * a[5] - a[2] * a[2]) / det;
            b[4] = (a[2] * a[1] - a[0] * a[4]) / det;
            b[5] = (a[3] * a[0] - a[1] * a[1]) / det;
            for (int q = 0; q < 6; ++q) S.inmu[l][q] = b[q];
            // mu^-1 (mu - mu0 I) Hp (pe_modelcurl, problem.f90:376-403)
            const double mu0 = 4.0 * PI_D * 1.e-7;
            double dmu[6] = {a[0] - mu0, a[1], a[2], a[3] - mu0, a[4], a[5] - mu0};
            const double hp = rr32(1.0e-9) / (4 * PI_D * 1.e-7);
            for (int p = 0; p < 2; ++p) {
                const double H[3] = {p == 1 ? hp : 0.0, p == 0 ? hp : 0.0, 0.0};
                for (int r = 0; r < 3; ++r) {
                    double s = 0.0;
                    for (int cc = 0; cc < 3; ++cc) {
                        double m = 0.0;
                        for (int q = 0; q < 3; ++q) m += b[pk(r, q)] * dmu[pk(q, cc)];
                        s += m * H[cc];
                    }
                    S.v[l][p][r] = s;
                }
            }
            for (int q = 0; q < 12; ++q) S.sigkm[l][q] = sigma[id * 12 + q];
            for (int f = 0; f < nf; ++f) {
                const double *sf = c_ap.have_sigma_f ? sigma_f + ((int64_t)f * c_ap.npt + id) * 12 : sigma + id * 12;
                for (int q = 0; q < 12; ++q) S.sig[f][l][q] = sf[q];
            }
        }
        for (int j = tid; j < ME; j += blockDim.x) S.gne[j] = gne[e * ME + j];
        // GPML zone flags the reference applies to this element
        int fl[3] = {0, 0, 0};
        if (GPML) {
            int pi = ie, pj = je, pkk = ke;
            bool use = true;
            if (c_ap.g.lag) {
                pkk = ke - 1;
                if (pkk < 0) { pkk = c_ap.nz - 1; pj--; }
                if (pj < 0) { pj = c_ap.ny - 1; pi--; }
                if (pi < 0) {
                    if (c_ap.g.ifreq == 0) use = false;
                    else { pi = c_ap.nx - 1; pj = c_ap.ny - 1; pkk = c_ap.nz - 1; }
                }
            }
            if (use) zone_flags(c_ap.g, pi + 1, pj + 1, pkk + 1, fl);
        }
        __syncthreads();
        // accumulators
        double kacc[G::PPT], macc[G::PPT], mpacc[G::PPT];
#pragma unroll
        for (int q = 0; q < G::PPT; ++q) kacc[q] = macc[q] = mpacc[q] = 0.0;
        constexpr int NB = ME * 2 * MVF_MAX_FREQ;
        constexpr int BPT = (ME * 2 + 255) / 256;  // (edge, pol) slots per thread per frequency
        double bacc[BPT][MVF_MAX_FREQ][2];
        (void)NB;
#pragma unroll
        for (int q = 0; q < BPT; ++q)
            for (int f = 0; f < MVF_MAX_FREQ; ++f) bacc[q][f][0] = bacc[q][f][1] = 0.0;

        for (int ch = 0; ch < G::NCH; ++ch) {
            // ---- per Gauss point quantities (int_elem_params / int_param / p_source)
            for (int gl = tid; gl < G::GC; gl += blockDim.x) {
                const int g = ch * G::GC + gl;
                double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                for (int l = 0; l < MN; ++l) {
                    const double *d = tdN + (g * MN + l) * 3;
                    for (int a = 0; a < 3; ++a)
                        for (int b = 0; b < 3; ++b) J[a][b] += d[a] * S.x[l][b];
                }
                const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) +
                                   J[0][1] * (J[1][2] * J[2][0] - J[1][0] * J[2][2]) +
                                   J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
                if (det == 0.0) S.err = 2;
                const double ad = fabs(det);
                double *ji = S.jinv[gl];
                ji[0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / ad;
                ji[1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / ad;
                ji[2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / ad;
                ji[3] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / ad;
                ji[4] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / ad;
                ji[5] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / ad;
                ji[6] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / ad;
                ji[7] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / ad;
                ji[8] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / ad;
                const double w = det * tgp[g * 4 + 3];
                S.wgt[gl] = w;
                // materials at the Gauss point (p_intmodels)
                double mf1[6] = {0, 0, 0, 0, 0, 0};
                cd mf2[6];
                for (int q = 0; q < 6; ++q) mf2[q] = {0.0, 0.0};
                double r[3] = {0, 0, 0};
                for (int l = 0; l < MN; ++l) {
                    const double nv = tN[g * MN + l];
                    for (int q = 0; q < 6; ++q) {
                        mf1[q] += nv * S.inmu[l][q];
                        mf2[q].re += nv * S.sigkm[l][2 * q];
                        mf2[q].im += nv * S.sigkm[l][2 * q + 1];
                    }
                    for (int a = 0; a < 3; ++a) r[a] += nv * S.x[l][a];
                }
                cd h[3] = {{1, 0}, {1, 0}, {1, 0}};
                if (GPML) stretch(c_ap.g, fl, r, c_ap.omega_km, h);
                const cd H = cmul(cmul(h[0], h[1]), h[2]);
                // mass material matrix: Re(H sigma) (f2, integration.f90:211-238)
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b) S.dm[gl][a][b] = w * cmul(H, mf2[pk(a, b)]).re;
                if (K1e) {
                    // the multilevel preconditioner's conductivity: the interpolated real
                    // part, shifted to be positive semidefinite where the quadratic
                    // interpolation of a jump undershoots (|sigma| for an isotropic one),
                    // plus a floor that makes the air's gradients regular
                    double gmin = 1e300;
                    for (int a = 0; a < 3; ++a) {
                        double off = 0.0;
                        for (int b = 0; b < 3; ++b)
                            if (b != a) off += fabs(mf2[pk(a, b)].re);
                        gmin = fmin(gmin, mf2[pk(a, a)].re - off);
                    }
                    const double shift = (c_ap.mg_abs ? 2.0 * fmax(0.0, -gmin) : 0.0) + sfloor;
                    for (int a = 0; a < 3; ++a)
                        for (int b = 0; b < 3; ++b)
                            S.dmp[gl][a][b] = w * (cmul(H, mf2[pk(a, b)]).re + (a == b ? H.re * shift : 0.0));
                }
                // curl material matrix (f1, integration.f90:154-209)
                if (GPML) {
                    // partial (c,p) is a derivative along axis ax[c][p]
                    const int ax[3][2] = {{1, 2}, {2, 0}, {0, 1}};
                    double rc[3][3];
                    for (int a = 0; a < 3; ++a)
                        for (int b = 0; b < 3; ++b) {
                            cd coef;
                            if (a == b) {
                                int o1 = (a + 1) % 3, o2 = (a + 2) % 3;
                                if (o1 > o2) { const int t = o1; o1 = o2; o2 = t; }
                                coef = cdiv(cmul(h[o1], h[o2]), h[a]);
                            } else {
                                coef = h[3 - a - b];
                            }
                            rc[a][b] = coef.re;
                        }
                    for (int c1 = 0; c1 < 3; ++c1)
                        for (int p = 0; p < 2; ++p)
                            for (int d1 = 0; d1 < 3; ++d1)
                                for (int q = 0; q < 2; ++q) {
                                    const double sgn = ((p + q) & 1) ? -1.0 : 1.0;
                                    S.dk[gl][c1 * 2 + p][d1 * 2 + q] =
                                        w * sgn * rc[ax[c1][p]][ax[d1][q]] * mf1[pk(c1, d1)];
                                }
                } else {
                    for (int a = 0; a < 3; ++a)
                        for (int b = 0; b < 3; ++b) S.dk[gl][a][b] = w * mf1[pk(a, b)];
                }
                // source for every rhs frequency and both polarisations (p_source)
                for (int f = 0; f < nf; ++f) {
                    const double om = c_ap.omega[f];
                    const double weps = rr32(om * EPS0_D);
                    const double w32 = rr32(om);
                    for (int p = 0; p < 2; ++p) {
                        cd dm3[3] = {{0, 0}, {0, 0}, {0, 0}};
                        double pc[3] = {0, 0, 0};
                        for (int l = 0; l < MN; ++l) {
                            const double nv = tN[g * MN + l];
                            // Ep: pol 1 (-i w b0 z, 0, 0), pol 2 (0, +i w b0 z, 0) (problem.f90:352-355)
                            const double ezv = rr32(om * 1.0e-9 * S.ez[l]);
                            const cd ep = {0.0, p == 0 ? -ezv : ezv};
                            const int cidx = p == 0 ? 0 : 1;
                            for (int a = 0; a < 3; ++a) {
                                cd ds = {S.sig[f][l][2 * pk(a, cidx)], S.sig[f][l][2 * pk(a, cidx) + 1]};
                                if (a == cidx) ds.im -= weps;
                                const cd t = cmul(ds, ep);
                                dm3[a].re += nv * t.re;
                                dm3[a].im += nv * t.im;
                            }
                            const double *vv = S.v[l][p];
                            if (vv[0] != 0.0 || vv[1] != 0.0 || vv[2] != 0.0) {
                                // grad N_l x v (p_pcurl); zero when mu = mu0
                                const double *d = tdN + (g * MN + l) * 3;
                                double gn[3];
                                for (int a = 0; a < 3; ++a) gn[a] = ji[a * 3 + 0] * d[0] + ji[a * 3 + 1] * d[1] + ji[a * 3 + 2] * d[2];
                                pc[0] += vv[2] * gn[1] - vv[1] * gn[2];
                                pc[1] += vv[0] * gn[2] - vv[2] * gn[0];
                                pc[2] += vv[1] * gn[0] - vv[0] * gn[1];
                            }
                        }
                        const cd wH = cscale(H, w);
                        for (int a = 0; a < 3; ++a) {
                            const cd s = cmul({dm3[a].re + pc[a], dm3[a].im}, {0.0, -w32});
                            const cd t = cmul(wH, s);
                            S.srcw[gl][f][p][2 * a] = t.re;
                            S.srcw[gl][f][p][2 * a + 1] = t.im;
                        }
                    }
                }
            }
            __syncthreads();
            // ---- edge basis at the chunk's Gauss points (int_edges, v_fem.f90:38-60)
            for (int t = tid; t < G::GC * ME; t += blockDim.x) {
                const int gl = t / ME, j = t % ME, g = ch * G::GC + gl;
                const double *ji = S.jinv[gl];
                const int dir = edge_dir[j];
                const double L = tL[g * ME + j];
                const double *dl = tdL + (g * ME + j) * 3;
                double vij[3], dni[3];
                for (int a = 0; a < 3; ++a) {
                    vij[a] = ji[a * 3 + dir];
                    dni[a] = ji[a * 3 + 0] * dl[0] + ji[a * 3 + 1] * dl[1] + ji[a * 3 + 2] * dl[2];
                }
                double cvp[6] = {dni[1] * vij[2], dni[2] * vij[1], dni[2] * vij[0], dni[0] * vij[2], dni[0] * vij[1],
                                 dni[1] * vij[0]};
                double cv[G::CW];
                if (GPML) {
                    for (int q = 0; q < 6; ++q) cv[q] = cvp[q];
                } else {
                    for (int a = 0; a < 3; ++a) cv[a] = cvp[2 * a] - cvp[2 * a + 1];
                }
                for (int q = 0; q < G::CW; ++q) S.bc[gl][j][q] = cv[q];
                for (int q = 0; q < G::CW; ++q) {
                    double s = 0.0;
                    for (int r = 0; r < G::CW; ++r) s += S.dk[gl][q][r] * cv[r];
                    S.tc[gl][j][q] = s;
                }
                double ve[3];
                for (int a = 0; a < 3; ++a) ve[a] = L * vij[a];
                for (int a = 0; a < 3; ++a) S.bv[gl][j][a] = ve[a];
                for (int a = 0; a < 3; ++a) S.tv[gl][j][a] = S.dm[gl][a][0] * ve[0] + S.dm[gl][a][1] * ve[1] + S.dm[gl][a][2] * ve[2];
                if (K1e)
                    for (int a = 0; a < 3; ++a)
                        S.tvp[gl][j][a] = S.dmp[gl][a][0] * ve[0] + S.dmp[gl][a][1] * ve[1] + S.dmp[gl][a][2] * ve[2];
            }
            __syncthreads();
            // ---- accumulate K_e, M_e (alocal) and b_e (blocal)
#pragma unroll
            for (int q = 0; q < G::PPT; ++q) {
                const int p = tid + q * 256;
                if (p < G::NPAIR) {
                    // pair index -> (i, j), i <= j
                    int i = (int)((sqrt(8.0 * p + 1.0) - 1.0) * 0.5);
                    while ((i + 1) * (i + 2) / 2 <= p) ++i;
                    while (i * (i + 1) / 2 > p) --i;
                    const int jj = p - i * (i + 1) / 2;  // jj <= i
                    double ks = 0.0, ms = 0.0, mps = 0.0;
                    for (int gl = 0; gl < G::GC; ++gl) {
#pragma unroll
                        for (int r = 0; r < G::CW; ++r) ks += S.bc[gl][i][r] * S.tc[gl][jj][r];
#pragma unroll
                        for (int r = 0; r < 3; ++r) ms += S.bv[gl][i][r] * S.tv[gl][jj][r];
                        if (K1e) {
#pragma unroll
                            for (int r = 0; r < 3; ++r) mps += S.bv[gl][i][r] * S.tvp[gl][jj][r];
                        }
                    }
                    kacc[q] += ks;
                    macc[q] += ms;
                    mpacc[q] += mps;
                }
            }
#pragma unroll
            for (int q = 0; q < BPT; ++q) {
                const int s = tid + q * 256;
                if (s < ME * 2) {
                    const int j = s >> 1, p = s & 1;
                    for (int f = 0; f < nf; ++f) {
                        double re = 0.0, im = 0.0;
                        for (int gl = 0; gl < G::GC; ++gl)
                            for (int a = 0; a < 3; ++a) {
                                re += S.bv[gl][j][a] * S.srcw[gl][f][p][2 * a];
                                im += S.bv[gl][j][a] * S.srcw[gl][f][p][2 * a + 1];
                            }
                        bacc[q][f][0] += re;
                        bacc[q][f][1] += im;
                    }
                }
            }
            __syncthreads();
        }
        if (S.err && tid == 0) atomicMax(errflag, S.err);
        // ---- element matrices into shared memory (reuse bc region)
        double *Ks = &S.bc[0][0][0];
        double *Ms = Ks + ME * ME;
        static_assert(sizeof(S.bc) + sizeof(S.tc) + sizeof(S.bv) + sizeof(S.tv) >= 2 * ME * ME * sizeof(double),
                      "element matrices reuse the per-chunk basis arrays");
#pragma unroll
        for (int q = 0; q < G::PPT; ++q) {
            const int p = tid + q * 256;
            if (p < G::NPAIR) {
                int i = (int)((sqrt(8.0 * p + 1.0) - 1.0) * 0.5);
                while ((i + 1) * (i + 2) / 2 <= p) ++i;
                while (i * (i + 1) / 2 > p) --i;
                const int jj = p - i * (i + 1) / 2;
                Ks[i * ME + jj] = kacc[q];
                Ks[jj * ME + i] = kacc[q];
                Ms[i * ME + jj] = macc[q];
                Ms[jj * ME + i] = macc[q];
            }
        }
        __syncthreads();
        if (Kst) {
            const int64_t so = (e - store_base);
            for (int t = tid; t < ME * ME; t += blockDim.x) {
                Kst[so * ME * ME + t] = Ks[t];
                Mst[so * ME * ME + t] = Ms[t];
            }
#pragma unroll
            for (int q = 0; q < BPT; ++q) {
                const int s = tid + q * 256;
                if (s < ME * 2) {
                    bst[(so * ME * 2 + s) * 2] = bacc[q][0][0];
                    bst[(so * ME * 2 + s) * 2 + 1] = bacc[q][0][1];
                }
            }
            continue;  // parity hook: no scatter
        }
        // ---- scatter into the CSR (assign_aij, global_assembly.f90:43-60; both triangles)
        for (int t = tid; t < ME * ME; t += blockDim.x) {
            const int i = t / ME, j = t % ME;
            const int gi = S.gne[i], gj = S.gne[j];
            if (gi <= 0 || gj <= 0) continue;
            const int64_t lo0 = rowptr[gi - 1], hi0 = rowptr[gi];
            int64_t lo = lo0, hi = hi0 - 1;
            const int target = gj - 1;
            while (lo < hi) {
                const int64_t mid = (lo + hi) >> 1;
                if (col[mid] < target) lo = mid + 1;
                else hi = mid;
            }
            if (col[lo] != target) { atomicMax(errflag, 4); continue; }
            K64[lo] += Ks[t];
            M64[lo] += Ms[t];
        }
        // right-hand side (assign_bi, global_assembly.f90:62-79) minus the Dirichlet lift
        // sum_jm A_e(j, jm) f_boundary(jm) (local_vfem, MoVFEM_3DMT.f90:221-263), which
        // vanishes for the zero-secondary-field model and for GPML.  f_boundary
        // (boundary_conds.f90:188-250) is the primary E_x (E_y) of the boundary node
        // times dx/dxi_dir (dy/dxi_dir) of this element at that node; Jn holds the
        // latter for every Dirichlet DOF not on a z face.
        double *Jn = &S.srcw[0][0][0][0];  // [ME][2], free after the Gauss-point loop
        if (c_ap.lift) {
            for (int jm = tid; jm < ME; jm += blockDim.x) {
                const int bd = -S.gne[jm];
                double j0 = 0.0, j1 = 0.0;
                if (bd > 0 && bd != 3 && bd != 6) {
                    const int nd = edge_node[jm], dir = edge_dir[jm];
                    const double rn[3] = {(double)node_ref(nd, 0), (double)node_ref(nd, 1), (double)node_ref(nd, 2)};
                    for (int l = 0; l < MN; ++l) {
                        double N, g[3];
                        nodal(MN, l, rn, N, g, c_ap.q9 != 0);
                        j0 += g[dir] * S.x[l][0];
                        j1 += g[dir] * S.x[l][1];
                    }
                    if (c_ap.bidx[S.node[nd]] < 0) atomicMax(errflag, 5);
                }
                Jn[2 * jm] = j0;
                Jn[2 * jm + 1] = j1;
            }
            __syncthreads();
        }
#pragma unroll
        for (int q = 0; q < BPT; ++q) {
            const int s = tid + q * 256;
            if (s < ME * 2) {
                const int j = s >> 1, p = s & 1;
                const int gj = S.gne[j];
                if (gj > 0) {
                    for (int f = 0; f < nf; ++f) {
                        double lr = 0.0, li = 0.0;
                        if (c_ap.lift) {
                            const double w = rr32(c_ap.omega[f]);
                            for (int jm = 0; jm < ME; ++jm) {
                                const double jn = Jn[2 * jm + p];
                                if (jn == 0.0) continue;
                                const int32_t bi = c_ap.bidx[S.node[edge_node[jm]]];
                                if (bi < 0) continue;
                                const double2 ep = c_ap.bep[((int64_t)f * c_ap.nb + bi) * 2 + p];
                                // (K + i w M)(j, jm) * ep * jn
                                const double ar = Ks[j * ME + jm], ai = w * Ms[j * ME + jm];
                                lr += (ar * ep.x - ai * ep.y) * jn;
                                li += (ar * ep.y + ai * ep.x) * jn;
                            }
                        }
                        double *dst = rhs + (((int64_t)f * 2 + p) * nne + (gj - 1)) * 2;
                        dst[0] += bacc[q][f][0] - lr;
                        dst[1] += bacc[q][f][1] - li;
                    }
                }
            }
        }
        // diagonals of G^T K G and G^T M G at the element's gradient nodes
        for (int l = tid; l < MN; l += blockDim.x) {
            const int32_t gn = node_gidx[S.node[l]];
            if (gn < 0) continue;
            double kd = 0.0, md = 0.0, ma = 0.0;
            const int cnt = c_glist_n[l];
            for (int a = 0; a < cnt; ++a) {
                const int ia = c_glist_i[l][a];
                if (S.gne[ia] <= 0) continue;
                const double ga = c_glist_v[l][a];
                ma += ga * ga * fabs(Ms[ia * ME + ia]);
                for (int b = 0; b < cnt; ++b) {
                    const int ib = c_glist_i[l][b];
                    if (S.gne[ib] <= 0) continue;
                    const double gb = c_glist_v[l][b];
                    kd += ga * gb * Ks[ia * ME + ib];
                    md += ga * gb * Ms[ia * ME + ib];
                }
            }
            kphi[gn] += kd;
            mphi[gn] += md;
            mabs[gn] += ma;
        }
        __syncthreads();
        if constexpr (ME != 12) {
            if (K1e) {
                // the preconditioner's element mass replaces M_e in shared memory; then the
                // Galerkin element matrices on the 12-edge space of the same cell,
                // P^T K_e P and P^T Mp_e P, and the scatter of Mp_e into the preconditioner's
                // CSR values
#pragma unroll
                for (int q = 0; q < G::PPT; ++q) {
                    const int p = tid + q * 256;
                    if (p < G::NPAIR) {
                        int i = (int)((sqrt(8.0 * p + 1.0) - 1.0) * 0.5);
                        while ((i + 1) * (i + 2) / 2 <= p) ++i;
                        while (i * (i + 1) / 2 > p) --i;
                        const int jj = p - i * (i + 1) / 2;
                        Ms[i * ME + jj] = mpacc[q];
                        Ms[jj * ME + i] = mpacc[q];
                    }
                }
                __syncthreads();
                // optional shift tau diag(K_e) of the preconditioner's mass
                if (c_ap.mg_tau > 0.0)
                    for (int i = tid; i < ME; i += blockDim.x) Ms[i * ME + i] += c_ap.mg_tau * Ks[i * ME + i];
                __syncthreads();
                for (int t = tid; t < 144; t += blockDim.x) {
                    const int a = t / 12, b = t % 12;
                    double k = 0.0, mm = 0.0;
                    for (int p = 0; p < c_ploc.cnt[a]; ++p) {
                        const int i = c_ploc.idx[a][p];
                        const double pa = c_ploc.val[a][p];
                        for (int q = 0; q < c_ploc.cnt[b]; ++q) {
                            const int j = c_ploc.idx[b][q];
                            const double w = pa * c_ploc.val[b][q];
                            k += w * Ks[i * ME + j];
                            mm += w * Ms[i * ME + j];
                        }
                    }
                    K1e[e * 144 + t] = k;
                    M1e[e * 144 + t] = mm;
                }
                for (int t = tid; t < ME * ME; t += blockDim.x) {
                    const int i = t / ME, j = t % ME;
                    const int gi = S.gne[i], gj = S.gne[j];
                    if (gi <= 0 || gj <= 0) continue;
                    int64_t lo = rowptr[gi - 1], hi = rowptr[gi] - 1;
                    while (lo < hi) {
                        const int64_t mid = (lo + hi) >> 1;
                        if (col[mid] < gj - 1) lo = mid + 1;
                        else hi = mid;
                    }
                    if (col[lo] == gj - 1) Mp64[lo] += Ms[t];
                }
                __syncthreads();
            }
        }
    }
}

template <int MN, int ME, int NGP, bool GPML>
static int launch_elements(Ctx *c, MatrixSet &S, const int32_t *elems, int64_t n, double *Kst, double *Mst, double *bst,
                           int64_t store_base, int *errflag) {
    double *K1e = Kst ? nullptr : S.K1e, *M1e = Kst ? nullptr : S.M1e, *Mp64 = Kst ? nullptr : S.Mp64;
    using SM = Smem<MN, ME, NGP, GPML>;
    const size_t smem = sizeof(SM);
    auto kern = element_kernel<MN, ME, NGP, GPML>;
    MVF_CUDA(c, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (n <= 0) return 0;
    const int64_t grid = std::min<int64_t>(n, 152 * 16);
    count_launch();
    kern<<<(unsigned)grid, 256, smem, c->stream>>>(
        elems, n, c->d.xp, c->d.yp, c->d.zp, c->d.sigma, c->d.sigma_f, c->d.mu, c->d.gne, c->d.N, c->d.dN, c->d.L,
        c->d.dL, c->d.gp, c->d.edge_node, c->d.edge_dir, c->d.rowptr, c->d.col, S.K64, S.M64, c->d.rhs, c->nne,
        c->d.node_gidx, S.kphi, S.mphi, S.mabs, Kst, Mst, bst, store_base, errflag, K1e, M1e, Mp64, c->mg_floor);
    MVF_CUDA(c, cudaGetLastError());
    return 0;
}

static int run_elements(Ctx *c, MatrixSet &S, bool gpml, const int32_t *elems, int64_t n, double *Kst, double *Mst,
                        double *bst, int64_t store_base, int *errflag) {
    const int mn = c->T.mn;
    if (mn == 8) return gpml ? launch_elements<8, 12, 8, true>(c, S, elems, n, Kst, Mst, bst, store_base, errflag)
                             : launch_elements<8, 12, 8, false>(c, S, elems, n, Kst, Mst, bst, store_base, errflag);
    if (mn == 20) return gpml ? launch_elements<20, 36, 27, true>(c, S, elems, n, Kst, Mst, bst, store_base, errflag)
                              : launch_elements<20, 36, 27, false>(c, S, elems, n, Kst, Mst, bst, store_base, errflag);
    return gpml ? launch_elements<27, 54, 27, true>(c, S, elems, n, Kst, Mst, bst, store_base, errflag)
                : launch_elements<27, 54, 27, false>(c, S, elems, n, Kst, Mst, bst, store_base, errflag);
}

// FP32 copies of K and M for the inner solver
__global__ void to_f32(const double *__restrict__ a, float *__restrict__ b, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

static void set_params(Ctx *c, AsmParams &ap, int fset, int nfb, const double *omegas, bool gpml, int ifreq) {
    const mvf_mesh &m = c->mesh;
    memset(&ap, 0, sizeof ap);
    ap.nx = m.nx; ap.ny = m.ny; ap.nz = m.nz;
    ap.nny = c->nny; ap.nnz_nodes = c->nnz_nodes; ap.npt = c->npt;
    ap.nf = nfb;
    for (int f = 0; f < nfb; ++f) ap.omega[f] = omegas[f];
    ap.omega_km = omegas[0];
    ap.r32 = (m.quirks & MVF_Q_FP32_CONST) ? 1 : 0;
    ap.have_sigma_f = c->d.sigma_f ? 1 : 0;
    ap.lift = dirichlet_lift(*c) ? 1 : 0;
    ap.q9 = (m.quirks & MVF_Q_LIN_DZETA) ? 1 : 0;
    ap.nb = (int64_t)c->bnode_h.size();
    ap.mg_tau = c->mg_tau;
    ap.mg_abs = c->mg_abs;
    ap.bidx = c->d.bidx;
    ap.bep = c->d.bep;
    (void)fset;
    GpmlParams &g = ap.g;
    g.on = gpml;
    g.sch = m.gpml_sch;
    g.lag = (m.quirks & MVF_Q_GPML_LAG) ? 1 : 0;
    g.ifreq = ifreq;
    g.nextd = m.nextd;
    g.a0 = m.a0; g.b0 = m.b0; g.nn = m.nn;
    if (gpml) {
        const int nord = c->T.nord;
        const int n3[3] = {m.nx + 1, m.ny + 1, m.nz + 1};
        for (int d = 0; d < 3; ++d) {
            g.el_a[d][0] = m.nextd; g.el_a[d][1] = n3[d] - m.nextd;
            g.el_b[d][0] = 1; g.el_b[d][1] = n3[d] - 1;
        }
        // init_gpml (boundary_conds.f90:60-63)
        const int64_t nnx = c->nnx, nny = c->nny, nnz = c->nnz_nodes;
        g.za[0][0] = c->xp_h[m.nextd * (nord - 1)];
        g.za[0][1] = c->xp_h[nnx - 1 - m.nextd * (nord - 1)];
        g.zb[0][0] = c->xp_h[0];
        g.zb[0][1] = c->xp_h[nnx - 1];
        g.za[1][0] = c->yp_h[m.nextd * (nord - 1)];
        g.za[1][1] = c->yp_h[nny - 1 - m.nextd * (nord - 1)];
        g.zb[1][0] = c->yp_h[0];
        g.zb[1][1] = c->yp_h[nny - 1];
        const int64_t id1 = (int64_t)m.nextd * (nord - 1);
        const int64_t id2 = (nnx - 1) * nny * nnz + (nny - 1) * nnz + nnz - 1 - (int64_t)m.nzl_top * (nord - 1);
        g.za[2][0] = c->zp_h[id1];
        g.za[2][1] = c->zp_h[id2];
        g.zb[2][0] = c->zp_h[0];
        g.zb[2][1] = c->zp_h[(nnx - 1) * nny * nnz + (nny - 1) * nnz + nnz - 1];
        const double f1 = (m.quirks & MVF_Q_FP32_CONST) ? (double)(float)1.e-5 : 1.e-5;
        g.omegar0 = 2.0 * PI_D * f1;
        g.omegar1 = 2.0 * PI_D * 1.e3;
    }
}

static int upload_glist(Ctx *c) {
    int n[MVF_MAX_NODES] = {0};
    unsigned char gi[MVF_MAX_NODES][24] = {{0}};
    double gv[MVF_MAX_NODES][24] = {{0}};
    for (int l = 0; l < c->T.mn; ++l)
        for (int j = 0; j < c->T.me; ++j)
            if (c->T.G[j][l] != 0.0) {
                if (n[l] >= 24) return fail(c, MVF_E_ARG, "gradient table overflow");
                gi[l][n[l]] = (unsigned char)j;
                gv[l][n[l]] = c->T.G[j][l];
                n[l]++;
            }
    MVF_CUDA(c, cudaMemcpyToSymbolAsync(c_glist_n, n, sizeof n, 0, cudaMemcpyHostToDevice, c->stream));
    MVF_CUDA(c, cudaMemcpyToSymbolAsync(c_glist_i, gi, sizeof gi, 0, cudaMemcpyHostToDevice, c->stream));
    MVF_CUDA(c, cudaMemcpyToSymbolAsync(c_glist_v, gv, sizeof gv, 0, cudaMemcpyHostToDevice, c->stream));
    return 0;
}

void free_sets(Ctx *c) {
    for (MatrixSet &S : c->sets) {
        void *p[] = {S.K64, S.M64, S.K32, S.M32, S.kphi, S.mphi, S.mabs, S.Kff, S.Mff, S.K1e, S.M1e, S.Mp64};
        for (void *q : p)
            if (q) cudaFree(q);
    }
    c->sets.clear();
}

// Assemble one matrix set and the right-hand sides of its frequencies.
int assemble_set(Ctx *c, MatrixSet &S, bool gpml, int fset) {
    const int64_t nnz = c->nnz;
    MVF_CUDA(c, cudaMalloc((void **)&S.K64, nnz * sizeof(double)));
    MVF_CUDA(c, cudaMalloc((void **)&S.M64, nnz * sizeof(double)));
    MVF_CUDA(c, cudaMalloc((void **)&S.K32, nnz * sizeof(float)));
    MVF_CUDA(c, cudaMalloc((void **)&S.M32, nnz * sizeof(float)));
    MVF_CUDA(c, cudaMalloc((void **)&S.kphi, std::max<int64_t>(c->ngn, 1) * sizeof(double)));
    MVF_CUDA(c, cudaMalloc((void **)&S.mphi, std::max<int64_t>(c->ngn, 1) * sizeof(double)));
    MVF_CUDA(c, cudaMalloc((void **)&S.mabs, std::max<int64_t>(c->ngn, 1) * sizeof(double)));
    MVF_CUDA(c, cudaMemsetAsync(S.K64, 0, nnz * sizeof(double), c->stream));
    MVF_CUDA(c, cudaMemsetAsync(S.M64, 0, nnz * sizeof(double), c->stream));
    MVF_CUDA(c, cudaMemsetAsync(S.kphi, 0, std::max<int64_t>(c->ngn, 1) * sizeof(double), c->stream));
    MVF_CUDA(c, cudaMemsetAsync(S.mphi, 0, std::max<int64_t>(c->ngn, 1) * sizeof(double), c->stream));
    MVF_CUDA(c, cudaMemsetAsync(S.mabs, 0, std::max<int64_t>(c->ngn, 1) * sizeof(double), c->stream));
    if (c->use_patches && c->precond == 0 && !c->mg.empty()) {
        MVF_CUDA(c, cudaMalloc((void **)&S.K1e, (size_t)c->ne * 144 * sizeof(double)));
        MVF_CUDA(c, cudaMalloc((void **)&S.M1e, (size_t)c->ne * 144 * sizeof(double)));
        MVF_CUDA(c, cudaMalloc((void **)&S.Mp64, nnz * sizeof(double)));
        MVF_CUDA(c, cudaMemsetAsync(S.Mp64, 0, nnz * sizeof(double), c->stream));
        PLoc pl;
        p_local(c->T.mn, pl);
        MVF_CUDA(c, cudaMemcpyToSymbolAsync(c_ploc, &pl, sizeof pl, 0, cudaMemcpyHostToDevice, c->stream));
    }
    AsmParams ap;
    set_params(c, ap, fset, S.nfreq, c->omega + S.first_freq, gpml, c->ifreq0 + S.first_freq);
    MVF_CUDA(c, cudaMemcpyToSymbolAsync(c_ap, &ap, sizeof ap, 0, cudaMemcpyHostToDevice, c->stream));
    int rc = upload_glist(c);
    if (rc) return rc;
    int *errflag = nullptr;
    MVF_CUDA(c, cudaMalloc((void **)&errflag, sizeof(int)));
    MVF_CUDA(c, cudaMemsetAsync(errflag, 0, sizeof(int), c->stream));
    // the right-hand-side rows of this set's frequencies
    double *rhs_save = c->d.rhs;
    c->d.rhs = c->d.rhs + (int64_t)S.first_freq * 2 * c->nne * 2;
    for (int col8 = 0; col8 < 8 && !rc; ++col8) {
        const int64_t a = c->color_off[col8], b = c->color_off[col8 + 1];
        rc = run_elements(c, S, gpml, c->d.elem_color + a, b - a, nullptr, nullptr, nullptr, 0, errflag);
    }
    c->d.rhs = rhs_save;
    if (rc) { cudaFree(errflag); return rc; }
    count_launch();
    to_f32<<<1024, 256, 0, c->stream>>>(S.K64, S.K32, nnz);
    count_launch();
    to_f32<<<1024, 256, 0, c->stream>>>(S.M64, S.M32, nnz);
    int herr = 0;
    MVF_CUDA(c, cudaMemcpyAsync(&herr, errflag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MVF_CUDA(c, cudaStreamSynchronize(c->stream));
    cudaFree(errflag);
    if (herr == 1) return fail(c, MVF_E_SINGULAR, "no mu inversion: singular mu tensor (problem.f90:266-271)");
    if (herr == 2) return fail(c, MVF_E_SINGULAR, "no transformation: zero Jacobian (n_fem.f90:374-377)");
    if (herr == 4) return fail(c, MVF_E_STATE, "element entry missing from the CSR pattern");
    if (herr == 5) return fail(c, MVF_E_STATE, "Dirichlet DOF off the x/y boundary planes");
    return 0;
}

int element_matrices(Ctx *c, int64_t e0, int64_t count, int f, double *K, double *M, double *b) {
    if (!c->assembled) return fail(c, MVF_E_STATE, "assemble first");
    if (e0 < 0 || count < 1 || e0 + count > c->ne || f < 0 || f >= c->nfreq) return fail(c, MVF_E_ARG, "bad range");
    const bool gpml = !c->mesh.dirichlet;
    MatrixSet tmp;
    // locate the set of frequency f; recompute with only frequency f on the rhs
    int si = 0;
    for (size_t s = 0; s < c->sets.size(); ++s)
        if (f >= c->sets[s].first_freq && f < c->sets[s].first_freq + c->sets[s].nfreq) si = (int)s;
    tmp = c->sets[si];
    AsmParams ap;
    double om[1] = {c->omega[f]};
    set_params(c, ap, si, 1, om, gpml, c->ifreq0 + f);
    if (ap.have_sigma_f) {
        // per-frequency sigma: point at frequency f's slice
        ap.have_sigma_f = 0;
    }
    MVF_CUDA(c, cudaMemcpyToSymbolAsync(c_ap, &ap, sizeof ap, 0, cudaMemcpyHostToDevice, c->stream));
    int rc = upload_glist(c);
    if (rc) return rc;
    const int me = c->T.me;
    double *dK, *dM, *db;
    int *errflag;
    MVF_CUDA(c, cudaMalloc((void **)&dK, count * me * me * sizeof(double)));
    MVF_CUDA(c, cudaMalloc((void **)&dM, count * me * me * sizeof(double)));
    MVF_CUDA(c, cudaMalloc((void **)&db, count * me * 2 * 2 * sizeof(double)));
    MVF_CUDA(c, cudaMalloc((void **)&errflag, sizeof(int)));
    MVF_CUDA(c, cudaMemsetAsync(errflag, 0, sizeof(int), c->stream));
    double *sig_save = c->d.sigma;
    if (c->d.sigma_f) c->d.sigma = c->d.sigma_f + (int64_t)f * c->npt * 12;
    rc = run_elements(c, tmp, gpml, nullptr, count, dK, dM, db, e0, errflag);
    c->d.sigma = sig_save;
    if (!rc) {
        MVF_CUDA(c, cudaMemcpyAsync(K, dK, count * me * me * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        MVF_CUDA(c, cudaMemcpyAsync(M, dM, count * me * me * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        MVF_CUDA(c, cudaMemcpyAsync(b, db, count * me * 4 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        MVF_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    cudaFree(dK); cudaFree(dM); cudaFree(db); cudaFree(errflag);
    return rc;
}

}  // namespace mvf

using namespace mvf;

// ---------------------------------------------------------------------------
// Primary field of the Dirichlet models 2 (half-space under air) and 3 (layered
// earth) on the boundary, per frequency (bd_setmodel / bd_updatemodel,
// boundary_conds.f90:396-430; wait_recursion :521-553; ezl :558-598; p_pfields
// :436-516).  Heights are depths below ztop in km, as the reference evaluates them.
namespace {
using cplx = std::complex<double>;

struct Primary {
    int nl = 0;
    cplx psig[16], cz[16], ez[16];
    double zl[16] = {0}, dl[16] = {0};
    double pmu = 4.0 * M_PI * 1.e-7;
};

double q32(const Ctx *c, double v) { return (c->mesh.quirks & MVF_Q_FP32_CONST) ? (double)(float)v : v; }

void primary_model(const Ctx *c, double omega, Primary &L) {
    const double eps0 = 8.854187817e-12;
    const cplx I(0.0, 1.0);
    if (c->mesh.inimod == 2) {
        L.nl = 2;
        L.psig[0] = I * q32(c, eps0 * omega);
        L.psig[1] = q32(c, c->mesh.h_sigma) + I * q32(c, eps0 * omega);
        return;
    }
    L.nl = (int)c->l_sigma_h.size();
    L.zl[0] = 0.0;
    for (int i = 0; i + 1 < L.nl; ++i) L.dl[i] = c->l_dz_h[i];
    for (int i = 1; i < L.nl; ++i) L.zl[i] = L.zl[i - 1] - L.dl[i - 1];
    for (int i = 0; i < L.nl; ++i) L.psig[i] = q32(c, c->l_sigma_h[i]) + I * q32(c, eps0 * omega);
    // impedance recursion from the bottom layer up, then the field ratios downwards
    const int nl = L.nl;
    L.cz[nl - 1] = 1.0 / std::sqrt(I * (omega * L.pmu * L.psig[nl - 1]));
    for (int l = nl - 2; l >= 0; --l) {
        const cplx gl = std::sqrt(I * (omega * L.pmu * L.psig[l]));
        const cplx r = (1.0 - gl * L.cz[l + 1]) / (1.0 + gl * L.cz[l + 1]);
        const cplx ex = std::exp(-2.0 * gl * L.dl[l]);
        L.cz[l] = (1.0 - r * ex) / (gl * (1.0 + r * ex));
    }
    L.ez[0] = 1.0;
    for (int l = 0; l + 1 < nl; ++l) {
        const cplx gl = std::sqrt(I * (omega * L.pmu * L.psig[l]));
        L.ez[l + 1] = std::exp(-gl * L.dl[l]) * (L.ez[l] * L.cz[l + 1] * (1.0 + L.cz[l] * gl)) /
                      (L.cz[l] * (1.0 + L.cz[l + 1] * gl));
    }
}

// the layered model's field at height z (ezl, its field branch)
cplx layered_e(const Primary &L, double omega, double z) {
    const cplx I(0.0, 1.0);
    cplx r = 0.0;
    const int nl = L.nl;
    for (int l = 0; l + 1 < nl; ++l) {
        if (z <= L.zl[l] && z > L.zl[l + 1]) {
            const cplx g = std::sqrt(I * (omega * L.pmu * L.psig[l]));
            const cplx rr = (1.0 - g * L.cz[l + 1]) / (1.0 + g * L.cz[l + 1]);
            r = (L.ez[l] / 2.0) * (1.0 + 1.0 / (L.cz[l] * g)) * (1.0 - rr * std::exp(-2.0 * g * (z - L.zl[l + 1]))) *
                std::exp(-g * (L.zl[l] - z));
        }
    }
    if (z <= L.zl[nl - 1]) {
        const cplx g = std::sqrt(I * (omega * L.pmu * L.psig[nl - 1]));
        r = L.ez[nl - 1] * std::exp(-g * (L.zl[nl - 1] - z));
    }
    return r;
}

// (E_x of polarisation 1, E_y of polarisation 2) at a node of height znode
void boundary_field(const Ctx *c, const Primary &L, double omega, double znode, cplx out[2]) {
    const cplx I(0.0, 1.0);
    const double bb0 = 1.e-9, z = (c->mesh.ztop - znode) / 1000.0;
    if (c->mesh.inimod == 2) {
        cplx fp;
        if (znode > c->mesh.ztop) {
            const cplx sa = std::sqrt(I * (omega * L.pmu * L.psig[0]));
            fp = (1.0 / sa) * (1.0 - z * sa);
        } else {
            const cplx sa = std::sqrt(I * (omega * L.pmu * L.psig[1]));
            fp = (1.0 / sa) * std::exp(-z * sa);
        }
        out[0] = (I * q32(c, -2.0 * omega * bb0)) * fp;
        out[1] = (I * q32(c, 2.0 * omega * bb0)) * fp;
    } else {
        const cplx f = znode > c->mesh.ztop ? (L.cz[0] - z) : L.cz[0] * layered_e(L, omega, z);
        out[0] = (I * q32(c, 2.0 * omega * bb0)) * f;
        out[1] = (I * q32(c, -2.0 * omega * bb0)) * f;
    }
}

int boundary_fields(Ctx *c) {
    if (c->d.bep) cudaFree(c->d.bep);
    c->d.bep = nullptr;
    if (!dirichlet_lift(*c)) return 0;
    const int64_t nb = (int64_t)c->bnode_h.size();
    std::vector<double2> h((size_t)c->nfreq * nb * 2);
    for (int f = 0; f < c->nfreq; ++f) {
        Primary L;
        primary_model(c, c->omega[f], L);
        for (int64_t b = 0; b < nb; ++b) {
            cplx ep[2];
            boundary_field(c, L, c->omega[f], c->zp_h[c->bnode_h[b]], ep);
            for (int p = 0; p < 2; ++p) h[((size_t)f * nb + b) * 2 + p] = make_double2(ep[p].real(), ep[p].imag());
        }
    }
    MVF_CUDA(c, cudaMalloc((void **)&c->d.bep, h.size() * sizeof(double2)));
    MVF_CUDA(c, cudaMemcpy(c->d.bep, h.data(), h.size() * sizeof(double2), cudaMemcpyHostToDevice));
    return 0;
}
}  // namespace

extern "C" int mvf_assemble(mvf_ctx *x, int32_t nfreq, const double *omega, const double *sigma_f, int32_t ifreq0) {
    if (!x) return MVF_E_ARG;
    Ctx *c = &x->c;
    if (!c->d.rowptr) return fail(c, MVF_E_STATE, "context not created");
    if (nfreq < 1 || nfreq > MVF_MAX_FREQ || !omega) return fail(c, MVF_E_ARG, "nfreq must be 1..16");
    for (int f = 0; f < nfreq; ++f)
        if (!(omega[f] > 0.0) || !std::isfinite(omega[f])) return fail(c, MVF_E_ARG, "omega must be positive");
    free_sets(c);
    c->assembled = c->solved = false;
    c->nfreq = nfreq;
    c->ifreq0 = ifreq0;
    for (int f = 0; f < nfreq; ++f) c->omega[f] = omega[f];
    if (c->d.sigma_f) { cudaFree(c->d.sigma_f); c->d.sigma_f = nullptr; }
    if (sigma_f) {
        MVF_CUDA(c, cudaMalloc((void **)&c->d.sigma_f, (size_t)nfreq * c->npt * 12 * sizeof(double)));
        MVF_CUDA(c, cudaMemcpy(c->d.sigma_f, sigma_f, (size_t)nfreq * c->npt * 12 * sizeof(double), cudaMemcpyHostToDevice));
    }
    if (c->d.rhs) cudaFree(c->d.rhs);
    if (c->d.x) cudaFree(c->d.x);
    c->d.rhs = c->d.x = nullptr;
    const size_t vb = (size_t)nfreq * 2 * c->nne * 2 * sizeof(double);
    MVF_CUDA(c, cudaMalloc((void **)&c->d.rhs, vb));
    MVF_CUDA(c, cudaMalloc((void **)&c->d.x, vb));
    MVF_CUDA(c, cudaMemsetAsync(c->d.rhs, 0, vb, c->stream));
    MVF_CUDA(c, cudaMemsetAsync(c->d.x, 0, vb, c->stream));
    if (int rc = boundary_fields(c)) return rc;
    const bool gpml = !c->mesh.dirichlet;
    if (!gpml) {
        // K and M do not depend on the frequency without GPML (Im(sigma) is dropped,
        // integration.f90:211-238): one set shared by every frequency
        c->sets.resize(1);
        c->sets[0].first_freq = 0;
        c->sets[0].nfreq = nfreq;
    } else {
        c->sets.resize(nfreq);
        for (int f = 0; f < nfreq; ++f) { c->sets[f].first_freq = f; c->sets[f].nfreq = 1; }
    }
    double *sig_save = c->d.sigma;
    for (size_t s = 0; s < c->sets.size(); ++s) {
        MatrixSet &S = c->sets[s];
        if (gpml && c->d.sigma_f) c->d.sigma = c->d.sigma_f + (int64_t)S.first_freq * c->npt * 12;
        // the sigma_f pointer offsets are per frequency inside the kernel; with one
        // frequency per set the set's slice is selected by shifting the base
        double *sf_save = c->d.sigma_f;
        if (gpml && c->d.sigma_f) c->d.sigma_f = c->d.sigma;
        int rc = assemble_set(c, S, gpml, (int)s);
        c->d.sigma_f = sf_save;
        c->d.sigma = sig_save;
        if (rc) return rc;
    }
    c->assembled = true;
    ++c->asm_gen;
    return 0;
}

extern "C" int mvf_element_matrices(const mvf_ctx *x, int64_t e0, int64_t count, int32_t f, double *K, double *M,
                                    double *b) {
    if (!x || !K || !M || !b) return MVF_E_ARG;
    return element_matrices(const_cast<Ctx *>(&x->c), e0, count, f, K, M, b);
}
