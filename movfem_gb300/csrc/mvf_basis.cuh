// mvf_basis.cuh -- nodal and edge basis of the 8/20/27-node hexahedra.
//
// Same functions as n_fem.f90:138-317 (nodal N_i and dN_i/dxi) and v_fem.f90:78-466
// (the per-edge "mixed-order" scalar factor L and its reference gradient), written
// as products of 1-D factors.  An edge basis function is L(xi) * grad(xi_dir)
// (v_fem.f90:38-44); its curl is grad(L) x grad(xi_dir) (v_fem.f90:49-60).
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define MVF_HD __host__ __device__ __forceinline__
#else
#define MVF_HD inline
#endif

namespace mvf {

// Reference coordinates of the element nodes (n_fem.f90:112-134): 8 corners,
// 12 mid-edge nodes, 4 x/y face centres, 2 z face centres, body centre.
MVF_HD int node_ref(int i, int axis) {
    // packed as three 27-entry tables of {-1,0,1}+1
    const signed char t[3][27] = {
        {1, 1, -1, -1, 1, 1, -1, -1, 1, 0, -1, 0, 1, 0, -1, 0, 1, 1, -1, -1, 1, 0, -1, 0, 0, 0, 0},
        {-1, 1, 1, -1, -1, 1, 1, -1, 0, 1, 0, -1, 0, 1, 0, -1, -1, 1, 1, -1, 0, 1, 0, -1, 0, 0, 0},
        {-1, -1, -1, -1, 1, 1, 1, 1, -1, -1, -1, -1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, -1, 1, 0}};
    return t[axis][i];
}

// 1-D factors: linear hat (1+a t)/2, quadratic Lagrange a t (1+a t)/2 (a=+-1) and
// the bubble 1-t^2.
MVF_HD void lin1(int a, double t, double &f, double &df) { f = 0.5 * (1.0 + a * t); df = 0.5 * a; }
MVF_HD void quad1(int a, double t, double &f, double &df) {
    if (a == 0) { f = 1.0 - t * t; df = -2.0 * t; }
    else { f = 0.5 * a * t * (1.0 + a * t); df = 0.5 * a * (1.0 + 2.0 * a * t); }
}

// Nodal shape function i of an mn-node hexahedron and its reference gradient.
// lin_dzeta_quirk: the 8-node dN/dzeta is written (1+nr1)(1+nr2*eta)nr3/8 in the
// reference (n_fem.f90:193) instead of (1+nr1*xi)(1+nr2*eta)nr3/8.
MVF_HD void nodal(int mn, int i, const double t[3], double &N, double g[3], bool lin_dzeta_quirk) {
    const int a = node_ref(i, 0), b = node_ref(i, 1), c = node_ref(i, 2);
    if (mn == 8) {
        double fx, dx, fy, dy, fz, dz;
        lin1(a, t[0], fx, dx); lin1(b, t[1], fy, dy); lin1(c, t[2], fz, dz);
        N = fx * fy * fz;
        g[0] = dx * fy * fz; g[1] = fx * dy * fz;
        g[2] = lin_dzeta_quirk ? 0.5 * (1.0 + a) * fy * dz : fx * fy * dz;
        return;
    }
    if (mn == 20) {
        if (i < 8) {
            // (1+a xi)(1+b eta)(1+c zeta)(a xi + b eta + c zeta - 2)/8
            const double p = 1.0 + a * t[0], q = 1.0 + b * t[1], r = 1.0 + c * t[2];
            const double s = a * t[0] + b * t[1] + c * t[2] - 2.0;
            N = p * q * r * s * 0.125;
            g[0] = a * q * r * (s + p) * 0.125;
            g[1] = b * p * r * (s + q) * 0.125;
            g[2] = c * p * q * (s + r) * 0.125;
            return;
        }
        // mid-edge: bubble along the axis with zero coordinate, (1+n t) on the others, /4
        double f[3], d[3];
        for (int k = 0; k < 3; ++k) {
            const int n = node_ref(i, k);
            if (n == 0) { f[k] = 1.0 - t[k] * t[k]; d[k] = -2.0 * t[k]; }
            else { f[k] = 1.0 + n * t[k]; d[k] = n; }
        }
        N = 0.25 * f[0] * f[1] * f[2];
        g[0] = 0.25 * d[0] * f[1] * f[2]; g[1] = 0.25 * f[0] * d[1] * f[2]; g[2] = 0.25 * f[0] * f[1] * d[2];
        return;
    }
    double fx, dx, fy, dy, fz, dz;
    quad1(a, t[0], fx, dx); quad1(b, t[1], fy, dy); quad1(c, t[2], fz, dz);
    N = fx * fy * fz;
    g[0] = dx * fy * fz; g[1] = fx * dy * fz; g[2] = fx * fy * dz;
}

// Scalar factor L of the edge basis attached to node i and direction dir (0..2).
MVF_HD void edge_factor(int mn, int i, int dir, const double t[3], double &L, double g[3]) {
    double f[3], d[3];
    if (mn == 8) {
        for (int k = 0; k < 3; ++k) {
            if (k == dir) { f[k] = 1.0; d[k] = 0.0; }
            else lin1(node_ref(i, k), t[k], f[k], d[k]);
        }
    } else if (mn == 20) {
        if (i < 8) {
            // prod_{k != dir}(1 + a_k t_k) * (sum_k a_k t_k - 1) / 8
            const int a[3] = {node_ref(i, 0), node_ref(i, 1), node_ref(i, 2)};
            const double s = a[0] * t[0] + a[1] * t[1] + a[2] * t[2] - 1.0;
            double p[3];
            for (int k = 0; k < 3; ++k) p[k] = (k == dir) ? 1.0 : 1.0 + a[k] * t[k];
            const double P = p[0] * p[1] * p[2];
            L = P * s * 0.125;
            for (int k = 0; k < 3; ++k) {
                double dp = 0.0;
                if (k != dir) {
                    dp = a[k];
                    for (int q = 0; q < 3; ++q) if (q != k) dp *= p[q];
                }
                g[k] = (dp * s + P * a[k]) * 0.125;
            }
            return;
        }
        for (int k = 0; k < 3; ++k) {
            const int n = node_ref(i, k);
            if (n == 0) { f[k] = 1.0 - t[k] * t[k]; d[k] = -2.0 * t[k]; }
            else if (k == dir) { f[k] = 1.0; d[k] = 0.0; }
            else { f[k] = 1.0 + n * t[k]; d[k] = n; }
        }
        f[0] *= 0.5; d[0] *= 0.5;
    } else {
        for (int k = 0; k < 3; ++k) {
            const int n = node_ref(i, k);
            if (k == dir) lin1(n, t[k], f[k], d[k]);
            else quad1(n, t[k], f[k], d[k]);
        }
    }
    L = f[0] * f[1] * f[2];
    g[0] = d[0] * f[1] * f[2]; g[1] = f[0] * d[1] * f[2]; g[2] = f[0] * f[1] * d[2];
}

// Edge DOF -> (node, direction), 1-based as mx_edge_dir (v_fem.f90:488-506).
struct EdgeTable {
    int me;
    const signed char *node;
    const signed char *dir;
};

}  // namespace mvf
