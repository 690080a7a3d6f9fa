// mvf_setup.cu -- context creation: tables, DOF numbering, CSR pattern, discrete gradient.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

#include "mvf_internal.cuh"

namespace mvf {

int fail(Ctx *c, int code, const std::string &msg) {
    if (c) c->err = msg;
    return code;
}

int cuda_fail(Ctx *c, cudaError_t e, const char *what) {
    char buf[512];
    snprintf(buf, sizeof buf, "CUDA error %d (%s) in %s", (int)e, cudaGetErrorString(e), what);
    if (c) c->err = buf;
    return e == cudaErrorMemoryAllocation ? MVF_E_NOMEM : MVF_E_CUDA;
}

// Edge DOF -> (node, direction), 1-based: the mx_edge_dir tables of v_fem.f90:488-506.
static const signed char EDGE12[2][12] = {{4, 4, 8, 3, 4, 8, 3, 7, 1, 1, 5, 2}, {3, 2, 2, 3, 1, 1, 1, 1, 3, 2, 2, 3}};
static const signed char EDGE36[2][36] = {
    {4, 8, 4, 3, 8, 7, 3, 7, 4, 1, 8, 5, 3, 2, 7, 6, 1, 5, 1, 2, 5, 6, 2, 6, 12, 20, 12, 16, 10, 17, 11, 20, 11, 15, 19, 9},
    {3, 3, 2, 2, 2, 2, 3, 3, 1, 1, 1, 1, 1, 1, 1, 1, 3, 3, 2, 2, 2, 2, 3, 3, 3, 2, 2, 2, 3, 2, 3, 1, 1, 1, 1, 3}};
static const signed char EDGE54[2][54] = {
    {4, 8, 4, 20, 8, 11, 15, 3, 19, 7, 3, 7, 4, 20, 8, 11, 15, 3, 19, 7, 12, 16, 12, 10, 16, 14, 10,
     14, 1, 17, 5, 9, 13, 2, 18, 6, 1, 5, 1, 17, 5, 9, 13, 2, 18, 6, 2, 6, 25, 26, 24, 22, 23, 21},
    {3, 3, 2, 2, 2, 3, 3, 2, 2, 2, 3, 3, 1, 1, 1, 1, 1, 1, 1, 1, 3, 3, 2, 2, 2, 2, 3,
     3, 1, 1, 1, 1, 1, 1, 1, 1, 3, 3, 2, 2, 2, 3, 3, 2, 2, 2, 3, 3, 3, 3, 2, 2, 1, 1}};

static double f32(double v) { return (double)(float)v; }

// Cholesky solve of the small SPD system A x = b (n <= 54), in place.
static bool chol_solve(std::vector<double> &A, std::vector<double> &b, int n) {
    for (int j = 0; j < n; ++j) {
        double s = A[j * n + j];
        for (int k = 0; k < j; ++k) s -= A[j * n + k] * A[j * n + k];
        if (s <= 0) return false;
        A[j * n + j] = std::sqrt(s);
        for (int i = j + 1; i < n; ++i) {
            double t = A[i * n + j];
            for (int k = 0; k < j; ++k) t -= A[i * n + k] * A[j * n + k];
            A[i * n + j] = t / A[j * n + j];
        }
    }
    for (int i = 0; i < n; ++i) {
        double t = b[i];
        for (int k = 0; k < i; ++k) t -= A[i * n + k] * b[k];
        b[i] = t / A[i * n + i];
    }
    for (int i = n - 1; i >= 0; --i) {
        double t = b[i];
        for (int k = i + 1; k < n; ++k) t -= A[k * n + i] * b[k];
        b[i] = t / A[i * n + i];
    }
    return true;
}

void build_tables(int mn, int quirks, OrderTables &T) {
    T.mn = mn;
    T.me = mn == 8 ? 12 : mn == 20 ? 36 : 54;
    T.nord = mn == 8 ? 2 : 3;
    for (int j = 0; j < T.me; ++j) {
        int nd, dr;
        if (mn == 8) { nd = EDGE12[0][j]; dr = EDGE12[1][j]; }
        else if (mn == 20) { nd = EDGE36[0][j]; dr = EDGE36[1][j]; }
        else { nd = EDGE54[0][j]; dr = EDGE54[1][j]; }
        T.edge_node[j] = nd - 1;
        T.edge_dir[j] = dr - 1;
    }
    // Face maps.  A DOF lies on the +a face when its node has coordinate +1 on axis a
    // and its direction is not a; across that face it is the DOF with the same
    // direction whose node is the mirror image (coordinate -1 on axis a).  This gives
    // the neighbour tables of c_gne12/36/54 and shr_nzindx12/36/54
    // (global_assembly.f90:231-1906) and the face lists of edge_bdary
    // (boundary_conds.f90:262-390).  Face order z, y, x as the reference.
    const int axis_of_face[3] = {2, 1, 0};
    for (int f = 0; f < 3; ++f) {
        const int a = axis_of_face[f];
        int cnt = 0;
        for (int j = 0; j < T.me; ++j) {
            const int nd = T.edge_node[j];
            if (node_ref(nd, a) != 1 || T.edge_dir[j] == a) continue;
            int mate = -1;
            for (int k = 0; k < T.me; ++k) {
                const int nk = T.edge_node[k];
                if (T.edge_dir[k] != T.edge_dir[j] || node_ref(nk, a) != -1) continue;
                bool same = true;
                for (int q = 0; q < 3; ++q)
                    if (q != a && node_ref(nk, q) != node_ref(nd, q)) same = false;
                if (same) mate = k;
            }
            T.face_src[f][cnt] = j;
            T.face_dst[f][cnt] = mate;
            ++cnt;
        }
        T.face_cnt = cnt;
    }
    // Gauss rule (integration.f90:25-55,267-496): 2^3 for the 12-edge element,
    // 3^3 otherwise, k fastest; abscissae and 3-point weights are default-real literals.
    const bool r32 = (quirks & MVF_Q_FP32_CONST) != 0;
    double p[3], w[3];
    int n;
    if (T.me == 12) {
        n = 2;
        p[1] = r32 ? f32(0.577350269189625764509148780502) : 0.577350269189625764509148780502;
        p[0] = -p[1];
        w[0] = w[1] = 1.0;
    } else {
        n = 3;
        p[2] = r32 ? f32(0.774596669241483377035853079956) : 0.774596669241483377035853079956;
        p[0] = -p[2];
        p[1] = 0.0;
        w[0] = w[2] = r32 ? f32(0.555555555555555555555555555556) : 5.0 / 9.0;
        w[1] = r32 ? f32(0.888888888888888888888888888889) : 8.0 / 9.0;
    }
    T.ngp = n * n * n;
    int g = 0;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j)
            for (int k = 0; k < n; ++k) {
                T.gp[g][0] = p[i]; T.gp[g][1] = p[j]; T.gp[g][2] = p[k];
                T.gp[g][3] = w[i] * w[j] * w[k];
                ++g;
            }
    const bool q9 = (quirks & MVF_Q_LIN_DZETA) != 0;
    T.N.assign(T.ngp * mn, 0.0);
    T.dN.assign(T.ngp * mn * 3, 0.0);
    T.L.assign(T.ngp * T.me, 0.0);
    T.dL.assign(T.ngp * T.me * 3, 0.0);
    for (g = 0; g < T.ngp; ++g) {
        for (int l = 0; l < mn; ++l) nodal(mn, l, T.gp[g], T.N[g * mn + l], &T.dN[(g * mn + l) * 3], q9);
        for (int j = 0; j < T.me; ++j)
            edge_factor(mn, T.edge_node[j], T.edge_dir[j], T.gp[g], T.L[g * T.me + j], &T.dL[(g * T.me + j) * 3]);
    }
    // Discrete gradient: coefficients with grad_xi N_n = sum_j G[j][n] L_j e_dir(j) on
    // the reference cube (the edge space contains the gradients of the nodal space;
    // the coefficients are geometry independent because both sides transform with
    // J^-1).  Least squares over sample points; entries are multiples of 1/8.
    {
        const double s[4] = {-0.83, -0.29, 0.37, 0.91};
        const int me = T.me;
        std::vector<double> BtB(me * me, 0.0);
        std::vector<double> rows;  // [192][me]
        std::vector<std::array<double, 3>> pts;
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b)
                for (int c = 0; c < 4; ++c) pts.push_back({s[a], s[b], s[c]});
        const int np = (int)pts.size();
        rows.assign((size_t)np * 3 * me, 0.0);
        for (int q = 0; q < np; ++q)
            for (int j = 0; j < me; ++j) {
                double Lv, gL[3];
                edge_factor(mn, T.edge_node[j], T.edge_dir[j], pts[q].data(), Lv, gL);
                rows[((size_t)q * 3 + T.edge_dir[j]) * me + j] = Lv;
            }
        for (int r = 0; r < np * 3; ++r)
            for (int i = 0; i < me; ++i)
                for (int j = 0; j < me; ++j) BtB[i * me + j] += rows[(size_t)r * me + i] * rows[(size_t)r * me + j];
        for (int nn = 0; nn < mn; ++nn) {
            std::vector<double> A = BtB, rhs(me, 0.0);
            for (int q = 0; q < np; ++q) {
                double Nv, gN[3];
                nodal(mn, nn, pts[q].data(), Nv, gN, false);
                for (int k = 0; k < 3; ++k)
                    for (int j = 0; j < me; ++j) rhs[j] += rows[((size_t)q * 3 + k) * me + j] * gN[k];
            }
            chol_solve(A, rhs, me);
            for (int j = 0; j < me; ++j) T.G[j][nn] = std::round(rhs[j] * 8.0) / 8.0;
        }
    }
}

// DOF numbering (c_gne12/36/54, global_assembly.f90:231-475 with edge_bdary,
// boundary_conds.f90:262-390): shared DOFs are inherited from the -z, -y, -x
// neighbours in that order; in Dirichlet mode, a DOF on the domain boundary gets the
// negative number of the first boundary face (x-, y-, z-, x+, y+, z+) it lies on; every
// other new DOF is numbered in element order.
int32_t number_grid(const OrderTables &T, int nx, int ny, int nz, bool dirichlet, std::vector<int32_t> &gne) {
    const int me = T.me;
    gne.assign((size_t)nx * ny * nz * me, 0);
    int32_t next = 0;
    std::vector<char> face_of[6];  // membership per boundary face
    for (int f = 0; f < 6; ++f) face_of[f].assign(me, 0);
    // boundary lists: x-, y-, z- are the dst sets of faces x, y, z; x+, y+, z+ the src sets
    const int fidx[6] = {2, 1, 0, 2, 1, 0};
    for (int f = 0; f < 6; ++f)
        for (int k = 0; k < T.face_cnt; ++k) face_of[f][f < 3 ? T.face_dst[fidx[f]][k] : T.face_src[fidx[f]][k]] = 1;
    for (int ie = 0; ie < nx; ++ie)
        for (int je = 0; je < ny; ++je)
            for (int ke = 0; ke < nz; ++ke) {
                const int64_t e = ((int64_t)ie * ny + je) * nz + ke;
                int32_t *row = &gne[(size_t)e * me];
                char inherited[MVF_MAX_ME] = {0};
                const int64_t nb[3] = {ke > 0 ? e - 1 : -1, je > 0 ? e - nz : -1, ie > 0 ? e - (int64_t)ny * nz : -1};
                for (int f = 0; f < 3; ++f) {
                    if (nb[f] < 0) continue;
                    const int32_t *prow = &gne[(size_t)nb[f] * me];
                    for (int k = 0; k < T.face_cnt; ++k) {
                        row[T.face_dst[f][k]] = prow[T.face_src[f][k]];
                        inherited[T.face_dst[f][k]] = 1;
                    }
                }
                const bool onb[6] = {ie == 0, je == 0, ke == 0, ie == nx - 1, je == ny - 1, ke == nz - 1};
                for (int j = 0; j < me; ++j) {
                    int face = 0;
                    if (dirichlet)
                        for (int f = 0; f < 6 && !face; ++f)
                            if (onb[f] && face_of[f][j]) face = f + 1;
                    if (face) row[j] = -face;
                    else if (!inherited[j]) row[j] = ++next;
                }
            }
    int32_t nne = 0;
    for (int32_t v : gne) nne = std::max(nne, v);
    return nne;
}

static int32_t number_dofs(const Ctx &c, std::vector<int32_t> &gne) {
    return number_grid(c.T, c.mesh.nx, c.mesh.ny, c.mesh.nz, c.mesh.dirichlet != 0, gne);
}

// Full symmetric CSR pattern: row r holds every free DOF that shares an element with r.
void pattern_from_gne(const std::vector<int32_t> &gne, int me, int64_t ne, int32_t n, std::vector<int64_t> &rowptr,
                      std::vector<int32_t> &col) {
    std::vector<int64_t> deg(n + 1, 0);
    for (int64_t e = 0; e < ne; ++e)
        for (int j = 0; j < me; ++j) {
            const int32_t g = gne[(size_t)e * me + j];
            if (g > 0) deg[g]++;
        }
    std::vector<int64_t> ip(n + 1, 0);
    for (int32_t r = 0; r < n; ++r) ip[r + 1] = ip[r] + deg[r + 1];
    std::vector<int64_t> elist(ip[n]);
    std::vector<int64_t> fill(ip.begin(), ip.end() - 1);
    for (int64_t e = 0; e < ne; ++e)
        for (int j = 0; j < me; ++j) {
            const int32_t g = gne[(size_t)e * me + j];
            if (g > 0) elist[fill[g - 1]++] = e;
        }
    rowptr.assign(n + 1, 0);
    std::vector<std::vector<int32_t>> rows_local;
#pragma omp parallel
    {
        std::vector<int32_t> buf;
#pragma omp for schedule(static)
        for (int32_t r = 0; r < n; ++r) {
            buf.clear();
            for (int64_t k = ip[r]; k < ip[r + 1]; ++k) {
                const int32_t *row = &gne[(size_t)elist[k] * me];
                for (int j = 0; j < me; ++j)
                    if (row[j] > 0) buf.push_back(row[j] - 1);
            }
            std::sort(buf.begin(), buf.end());
            rowptr[r + 1] = std::unique(buf.begin(), buf.end()) - buf.begin();
        }
    }
    for (int32_t r = 0; r < n; ++r) rowptr[r + 1] += rowptr[r];
    col.assign(rowptr[n], 0);
#pragma omp parallel
    {
        std::vector<int32_t> buf;
#pragma omp for schedule(static)
        for (int32_t r = 0; r < n; ++r) {
            buf.clear();
            for (int64_t k = ip[r]; k < ip[r + 1]; ++k) {
                const int32_t *row = &gne[(size_t)elist[k] * me];
                for (int j = 0; j < me; ++j)
                    if (row[j] > 0) buf.push_back(row[j] - 1);
            }
            std::sort(buf.begin(), buf.end());
            auto end = std::unique(buf.begin(), buf.end());
            std::copy(buf.begin(), end, col.begin() + rowptr[r]);
        }
    }
}

static void build_pattern(const Ctx &c, std::vector<int64_t> &rowptr, std::vector<int32_t> &col) {
    pattern_from_gne(c.gne_h, c.T.me, c.ne, c.nne, rowptr, col);
}

template <class T>
static int upload(Ctx *c, T **dst, const T *src, size_t n) {
    MVF_CUDA(c, cudaMalloc((void **)dst, std::max<size_t>(n, 1) * sizeof(T)));
    if (n) MVF_CUDA(c, cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
    return 0;
}

int64_t element_node(const Ctx &c, int ie, int je, int ke, int l) {
    const int nord = c.T.nord;
    const int64_t ii = (int64_t)ie * (nord - 1) + (node_ref(l, 0) + 1) * (nord - 1) / 2;
    const int64_t jj = (int64_t)je * (nord - 1) + (node_ref(l, 1) + 1) * (nord - 1) / 2;
    const int64_t kk = (int64_t)ke * (nord - 1) + (node_ref(l, 2) + 1) * (nord - 1) / 2;
    return (ii * c.nny + jj) * c.nnz_nodes + kk;
}

// Discrete gradient G (free DOFs x gradient nodes) and its transpose.  Gradient
// nodes are the grid nodes the element uses; in Dirichlet mode nodes on the outer
// boundary are left out so that G maps into the free DOFs exactly.
static int build_gradient(Ctx *c) {
    const OrderTables &T = c->T;
    const int me = T.me, mn = T.mn;
    std::vector<int32_t> gidx(c->npt, -1);
    int32_t ngn = 0;
    auto on_boundary = [&](int64_t id) {
        const int64_t i = id / (c->nny * c->nnz_nodes), j = (id / c->nnz_nodes) % c->nny, k = id % c->nnz_nodes;
        return i == 0 || j == 0 || k == 0 || i == c->nnx - 1 || j == c->nny - 1 || k == c->nnz_nodes - 1;
    };
    std::vector<char> row_done(c->nne, 0);
    std::vector<std::vector<std::pair<int32_t, float>>> rows(c->nne);
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
                        if (T.G[j][l] == 0.0) continue;
                        if (c->mesh.dirichlet && on_boundary(nodes[l])) continue;
                        if (gidx[nodes[l]] < 0) gidx[nodes[l]] = ngn++;
                        rows[g - 1].push_back({gidx[nodes[l]], (float)T.G[j][l]});
                    }
                }
            }
    c->ngn = ngn;
    std::vector<int64_t> gr(c->nne + 1, 0), gtr(ngn + 1, 0);
    for (int32_t r = 0; r < c->nne; ++r) gr[r + 1] = gr[r] + (int64_t)rows[r].size();
    std::vector<int32_t> gc(gr[c->nne]);
    std::vector<float> gv(gr[c->nne]);
    for (int32_t r = 0; r < c->nne; ++r) {
        std::sort(rows[r].begin(), rows[r].end());
        for (size_t k = 0; k < rows[r].size(); ++k) {
            gc[gr[r] + k] = rows[r][k].first;
            gv[gr[r] + k] = rows[r][k].second;
            gtr[rows[r][k].first + 1]++;
        }
    }
    for (int32_t n = 0; n < ngn; ++n) gtr[n + 1] += gtr[n];
    std::vector<int32_t> gtc(gr[c->nne]);
    std::vector<float> gtv(gr[c->nne]);
    std::vector<int64_t> fill(gtr.begin(), gtr.end() - 1);
    for (int32_t r = 0; r < c->nne; ++r)
        for (int64_t k = gr[r]; k < gr[r + 1]; ++k) {
            gtc[fill[gc[k]]] = r;
            gtv[fill[gc[k]]++] = gv[k];
        }
    int rc;
    if ((rc = upload(c, &c->d.grow, gr.data(), gr.size()))) return rc;
    if ((rc = upload(c, &c->d.gcol, gc.data(), gc.size()))) return rc;
    if ((rc = upload(c, &c->d.gval, gv.data(), gv.size()))) return rc;
    if ((rc = upload(c, &c->d.gtrow, gtr.data(), gtr.size()))) return rc;
    if ((rc = upload(c, &c->d.gtcol, gtc.data(), gtc.size()))) return rc;
    if ((rc = upload(c, &c->d.gtval, gtv.data(), gtv.size()))) return rc;
    if ((rc = upload(c, &c->d.node_gidx, gidx.data(), gidx.size()))) return rc;
    return 0;
}

static int create(Ctx *c, const mvf_mesh *m, int device) {
    if (!m || !m->xp || !m->yp || !m->zp || !m->sigma || !m->mu) return fail(c, MVF_E_ARG, "null mesh array");
    if (m->nodes_per_elem != 8 && m->nodes_per_elem != 20 && m->nodes_per_elem != 27)
        return fail(c, MVF_E_ARG, "nodes_per_elem must be 8, 20 or 27");
    if (m->nx < 1 || m->ny < 1 || m->nz < 1) return fail(c, MVF_E_ARG, "empty mesh");
    if (m->dirichlet && (m->inimod < 1 || m->inimod > 3)) return fail(c, MVF_E_ARG, "inimod must be 1, 2 or 3");
    if (m->dirichlet && m->inimod == 3 &&
        (m->nlayers < 1 || m->nlayers > 16 || !m->l_sigma || (m->nlayers > 1 && !m->l_dz)))
        return fail(c, MVF_E_ARG, "inimod 3 needs 1..16 layers with l_sigma[nlayers] and l_dz[nlayers-1]");
    if (!m->dirichlet && (m->nzl_top < 0 || m->nextd < 0)) return fail(c, MVF_E_ARG, "bad GPML zone sizes");
    c->mesh = *m;
    {
        const int nord0 = m->nodes_per_elem == 8 ? 2 : 3;
        const int64_t nnx0 = (int64_t)m->nx * (nord0 - 1) + 1, nny0 = (int64_t)m->ny * (nord0 - 1) + 1;
        const int64_t npt0 = nnx0 * nny0 * ((int64_t)m->nz * (nord0 - 1) + 1);
        c->xp_h.assign(m->xp, m->xp + nnx0);
        c->yp_h.assign(m->yp, m->yp + nny0);
        c->zp_h.assign(m->zp, m->zp + npt0);
        // the caller's arrays need not outlive this call
        c->mesh.xp = c->xp_h.data();
        c->mesh.yp = c->yp_h.data();
        c->mesh.zp = c->zp_h.data();
        c->mesh.sigma = nullptr;
        c->mesh.mu = nullptr;
        if (m->dirichlet && m->inimod == 3) {
            c->l_sigma_h.assign(m->l_sigma, m->l_sigma + m->nlayers);
            if (m->nlayers > 1) c->l_dz_h.assign(m->l_dz, m->l_dz + m->nlayers - 1);
        }
        c->mesh.l_sigma = nullptr;
        c->mesh.l_dz = nullptr;
    }
    int ndev = 0;
    MVF_CUDA(c, cudaGetDeviceCount(&ndev));
    if (ndev < 1) return fail(c, MVF_E_CUDA, "no CUDA device");
    if (device >= 0) MVF_CUDA(c, cudaSetDevice(device));
    MVF_CUDA(c, cudaGetDevice(&c->device));
    {
        // the element and receiver kernels keep per-thread tables on the stack: make
        // sure the per-thread stack covers them (the default is 1 KB)
        size_t stack = 0;
        MVF_CUDA(c, cudaDeviceGetLimit(&stack, cudaLimitStackSize));
        if (stack < 4096) MVF_CUDA(c, cudaDeviceSetLimit(cudaLimitStackSize, 4096));
    }
    MVF_CUDA(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    MVF_CUDA(c, cudaMalloc((void **)&c->d.wsp, 2 * 32 * sizeof(double)));
    build_tables(m->nodes_per_elem, m->quirks, c->T);
    const int nord = c->T.nord;
    c->nnx = (int64_t)m->nx * (nord - 1) + 1;
    c->nny = (int64_t)m->ny * (nord - 1) + 1;
    c->nnz_nodes = (int64_t)m->nz * (nord - 1) + 1;
    c->npt = c->nnx * c->nny * c->nnz_nodes;
    c->ne = (int64_t)m->nx * m->ny * m->nz;
    // material checks (problem.f90:260-271): singular sigma or mu stops the reference
    for (int64_t i = 0; i < c->npt; ++i) {
        const double *a = m->mu + i * 6;
        const double d = a[0] * (a[3] * a[5] - a[4] * a[4]) + a[1] * (a[2] * a[4] - a[1] * a[5]) +
                         a[2] * (a[1] * a[4] - a[3] * a[2]);
        if (d == 0.0 || !std::isfinite(d)) return fail(c, MVF_E_SINGULAR, "singular mu tensor at node " + std::to_string(i));
        for (int k = 0; k < 12; ++k)
            if (!std::isfinite(m->sigma[i * 12 + k])) return fail(c, MVF_E_ARG, "non-finite sigma at node " + std::to_string(i));
    }
    c->nne = number_dofs(*c, c->gne_h);
    if (c->nne <= 0) return fail(c, MVF_E_ARG, "no free DOFs");
    std::vector<int64_t> rowptr;
    std::vector<int32_t> col;
    build_pattern(*c, rowptr, col);
    c->nnz = rowptr[c->nne];
    int64_t low = 0;
    for (int32_t r = 0; r < c->nne; ++r)
        for (int64_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
            if (col[k] <= r) ++low;
    c->nnz_lower = low;
    int rc;
    if ((rc = upload(c, &c->d.rowptr, rowptr.data(), rowptr.size()))) return rc;
    if ((rc = upload(c, &c->d.col, col.data(), col.size()))) return rc;
    if ((rc = upload(c, &c->d.gne, c->gne_h.data(), c->gne_h.size()))) return rc;
    if (dirichlet_lift(*c)) {
        // nodes on the x and y boundary planes carry the prescribed primary field of
        // the Dirichlet DOFs on faces 1, 2, 4, 5 (f_boundary skips the z faces 3, 6)
        std::vector<int32_t> bidx(c->npt, -1);
        c->bnode_h.clear();
        for (int64_t i = 0; i < c->nnx; ++i)
            for (int64_t j = 0; j < c->nny; ++j) {
                if (i != 0 && i != c->nnx - 1 && j != 0 && j != c->nny - 1) continue;
                for (int64_t k = 0; k < c->nnz_nodes; ++k) {
                    const int64_t id = (i * c->nny + j) * c->nnz_nodes + k;
                    bidx[id] = (int32_t)c->bnode_h.size();
                    c->bnode_h.push_back(id);
                }
            }
        if ((rc = upload(c, &c->d.bidx, bidx.data(), bidx.size()))) return rc;
    }
    // element colouring: 2x2x2 parity classes share no DOF or node
    std::vector<int32_t> byc;
    byc.reserve(c->ne);
    c->color_off.assign(9, 0);
    for (int col8 = 0; col8 < 8; ++col8) {
        c->color_off[col8] = (int64_t)byc.size();
        for (int ie = col8 & 1; ie < m->nx; ie += 2)
            for (int je = (col8 >> 1) & 1; je < m->ny; je += 2)
                for (int ke = (col8 >> 2) & 1; ke < m->nz; ke += 2)
                    byc.push_back((int32_t)(((int64_t)ie * m->ny + je) * m->nz + ke));
    }
    c->color_off[8] = (int64_t)byc.size();
    if ((rc = upload(c, &c->d.elem_color, byc.data(), byc.size()))) return rc;
    if ((rc = upload(c, &c->d.xp, m->xp, (size_t)c->nnx))) return rc;
    if ((rc = upload(c, &c->d.yp, m->yp, (size_t)c->nny))) return rc;
    if ((rc = upload(c, &c->d.zp, m->zp, (size_t)c->npt))) return rc;
    if ((rc = upload(c, &c->d.sigma, m->sigma, (size_t)c->npt * 12))) return rc;
    if ((rc = upload(c, &c->d.mu, m->mu, (size_t)c->npt * 6))) return rc;
    const OrderTables &T = c->T;
    if ((rc = upload(c, &c->d.N, T.N.data(), T.N.size()))) return rc;
    if ((rc = upload(c, &c->d.dN, T.dN.data(), T.dN.size()))) return rc;
    if ((rc = upload(c, &c->d.L, T.L.data(), T.L.size()))) return rc;
    if ((rc = upload(c, &c->d.dL, T.dL.data(), T.dL.size()))) return rc;
    if ((rc = upload(c, &c->d.gp, &T.gp[0][0], (size_t)MVF_MAX_GP * 4))) return rc;
    {
        std::vector<double> gl((size_t)T.me * T.mn);
        for (int j = 0; j < T.me; ++j)
            for (int l = 0; l < T.mn; ++l) gl[j * T.mn + l] = T.G[j][l];
        if ((rc = upload(c, &c->d.Gloc, gl.data(), gl.size()))) return rc;
        std::vector<int32_t> en(T.edge_node, T.edge_node + T.me), ed(T.edge_dir, T.edge_dir + T.me);
        if ((rc = upload(c, &c->d.edge_node, en.data(), en.size()))) return rc;
        if ((rc = upload(c, &c->d.edge_dir, ed.data(), ed.size()))) return rc;
    }
    if ((rc = build_gradient(c))) return rc;
    // the 36- and 54-DOF elements are preconditioned with vertex patches
    c->use_patches = c->T.mn != 8;
    if (c->use_patches && (rc = patch_setup(c))) return rc;
    if (c->use_patches && c->precond == 0 && (rc = mg_setup(c))) return rc;
    return 0;
}

static void release(Ctx *c) {
    free_sets(c);
    mg_release(c);
    surf_release(c);
    void *ptrs[] = {c->d.xp, c->d.yp, c->d.zp, c->d.sigma, c->d.sigma_f, c->d.mu, c->d.gne, c->d.elem_color,
                    c->d.N, c->d.dN, c->d.L, c->d.dL, c->d.gp, c->d.Gloc, c->d.edge_node, c->d.edge_dir,
                    c->d.rowptr, c->d.col, c->d.grow, c->d.gcol, c->d.gval, c->d.gtrow, c->d.gtcol, c->d.gtval,
                    c->d.node_gidx, c->d.rhs, c->d.x, c->d.guess, c->d.bidx, c->d.bep, c->d.wsp, c->d.Ke, c->d.Me, c->d.be, c->d.patch_ptr,
                    c->d.patch_ioff, c->d.patch_dof};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    c->d = Device{};
    if (c->stream) cudaStreamDestroy(c->stream);
    c->stream = nullptr;
}

}  // namespace mvf

using namespace mvf;

extern "C" int mvf_create(mvf_ctx **out, const mvf_mesh *mesh, int32_t device) {
    if (!out) return MVF_E_ARG;
    mvf_ctx *x = new mvf_ctx();
    int rc = create(&x->c, mesh, device);
    if (rc) {
        // keep the context so the caller can read the message, with device memory freed
        release(&x->c);
    }
    *out = x;
    return rc;
}

extern "C" void mvf_destroy(mvf_ctx *x) {
    if (!x) return;
    release(&x->c);
    delete x;
}

extern "C" const char *mvf_last_error(const mvf_ctx *x) { return x ? x->c.err.c_str() : map_last_error(); }

extern "C" int mvf_sizes(const mvf_ctx *x, int32_t *nne, int64_t *nnz_full, int64_t *nnz_lower, int32_t *me,
                         int64_t *ne) {
    if (!x) return MVF_E_ARG;
    const Ctx &c = x->c;
    if (!c.d.rowptr) return MVF_E_STATE;
    if (nne) *nne = c.nne;
    if (nnz_full) *nnz_full = c.nnz;
    if (nnz_lower) *nnz_lower = c.nnz_lower;
    if (me) *me = c.T.me;
    if (ne) *ne = c.ne;
    return 0;
}

extern "C" int mvf_numbering(const mvf_ctx *x, int32_t *gne) {
    if (!x || !gne) return MVF_E_ARG;
    const Ctx &c = x->c;
    if (c.gne_h.empty()) return MVF_E_STATE;
    const int me = c.T.me;
    for (int64_t e = 0; e < c.ne; ++e)
        for (int j = 0; j < me; ++j) gne[(size_t)j * c.ne + e] = c.gne_h[(size_t)e * me + j];
    return 0;
}

extern "C" int mvf_set_sigma(mvf_ctx *x, const double *sigma) {
    if (!x || !sigma) return MVF_E_ARG;
    Ctx *c = &x->c;
    if (!c->d.sigma) return fail(c, MVF_E_STATE, "context not created");
    MVF_CUDA(c, cudaMemcpy(c->d.sigma, sigma, (size_t)c->npt * 12 * sizeof(double), cudaMemcpyHostToDevice));
    return 0;
}
