// TEST INFRASTRUCTURE ONLY -- CPU oracle (see oracle.hpp).
// Geometry info, global DOF numbering, per-element global<->local transforms and
// global CSR assembly.  Restates src/BuildSpace.cpp:436-1214 and
// src/Discretize.cpp:522-593, 1297-1395.
#include "oracle.hpp"
#include <cmath>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <algorithm>
#include <numeric>
#include <stdexcept>

namespace tsem_oracle {

static const int kFacePoint[12] = {1, 2, 3, 0, 2, 3, 0, 1, 3, 0, 1, 2};
static const int kFaceEdge[12] = {5, 4, 3, 5, 2, 1, 4, 2, 0, 3, 1, 0};
static const int kEdgeStart[6] = {0, 0, 0, 1, 1, 2};
static const int kEdgeEnd[6] = {1, 2, 3, 2, 3, 3};

// ------------------------------------------------------------- face table I/O
// Same record layout as the reference reader, src/BuildSpace.cpp:1704-1771.
bool FaceTable::load(const std::string& path) {
    std::ifstream in(path);
    if (!in) return false;
    in >> M_tab;
    nf_tab = (M_tab - 2) * (M_tab - 3) / 2 + M_tab - 2;
    edge.assign(6, {});
    face.assign(6, {});
    for (int v = 0; v < 6; ++v) {
        edge[v].resize(nf_tab);
        face[v].resize(nf_tab);
        for (int d = 0; d < nf_tab; ++d)
            for (int e = 0; e < 3; ++e) {
                int cnt; in >> cnt;
                for (int k = 0; k < cnt; ++k) { int i; double x; in >> i >> x; edge[v][d][e].push_back({i, x}); }
            }
        for (int d = 0; d < nf_tab; ++d) {
            int cnt; in >> cnt;
            for (int k = 0; k < cnt; ++k) { int i; double x; in >> i >> x; face[v][d].push_back({i, x}); }
        }
    }
    return (bool)in;
}

// ------------------------------------------------------------------- CSR
int64_t Csr::find(int r, int c) const {
    if (col[rowptr[r]] == c) return rowptr[r];
    auto b = col.begin() + rowptr[r] + 1, e = col.begin() + rowptr[r + 1];
    auto it = std::lower_bound(b, e, c);
    if (it == e || *it != c) return -1;
    return it - col.begin();
}
void Csr::vmult(const double* x, double* y) const {
#pragma omp parallel for schedule(static)
    for (int r = 0; r < n; ++r) {
        double s = 0;
        for (int64_t p = rowptr[r]; p < rowptr[r + 1]; ++p) s += val[p] * x[col[p]];
        y[r] = s;
    }
}

int Space::geo_first_dof(int dim, int idx) const {
    int t = idx;
    for (int d = 0; d < dim; ++d) t += n_geo[d];
    return location_actualdof[location_geometry[t]];
}

void Space::build(const Mesh& m, int order, const FaceTable& ft, int quad_q) {
    mesh = &m;
    M = order;
    lb.init(M);
    n_loc = lb.n_loc;
    ref.build(lb);
    quad.build(quad_q);
    if (ft.M_tab < M) throw std::runtime_error("face table order too low");
    n_geo[0] = m.nv; n_geo[1] = m.ne; n_geo[2] = m.nf; n_geo[3] = m.nt;
    n_ele = m.nt;
    n_geo_total = m.nv + m.ne + m.nf + m.nt;
    for (int d = 0; d <= 3; ++d) n_dof_geo[d] = binom_ref(M - 1, d);  // BuildSpace.cpp:448-449
    n_dof = 0;
    for (int d = 0; d <= 3; ++d) n_dof += n_geo[d] * n_dof_geo[d];

    // ---------------------------------------------- geometry info, :471-633
    const int E = n_ele;
    ele_node.assign(4 * E, -1); ele_edge.assign(6 * E, -1); ele_face.assign(4 * E, -1);
    type_edge.assign(6 * E, -1); type_face.assign(4 * E, -1); type_face_inv.assign(4 * E, -1);
    edge_node.assign(2 * m.ne, -1);
    face_node.assign(3 * m.nf, -1); face_edge.assign(3 * m.nf, -1);
    face_same.assign(3 * m.nf, 1);
    std::vector<char> seen_edge(m.ne, 0), seen_face(m.nf, 0);
    for (int e = 0; e < E; ++e) {
        int* nd = &ele_node[4 * e];
        int* ed = &ele_edge[6 * e];
        for (int k = 0; k < 4; ++k) nd[k] = m.tet_v[4 * e + k];
        // edges from the faces opposite P3, P2, P1
        {
            int f = m.tet_f[4 * e + 3];
            for (int j = 0; j < 3; ++j) {
                int v = m.face_v[3 * f + j], eg = m.face_e[3 * f + j];
                if (v == nd[0]) ed[3] = eg;
                if (v == nd[1]) ed[1] = eg;
                if (v == nd[2]) ed[0] = eg;
            }
            f = m.tet_f[4 * e + 2];
            for (int j = 0; j < 3; ++j) {
                int v = m.face_v[3 * f + j], eg = m.face_e[3 * f + j];
                if (v == nd[0]) ed[4] = eg;
                if (v == nd[1]) ed[2] = eg;
            }
            f = m.tet_f[4 * e + 1];
            for (int j = 0; j < 3; ++j)
                if (m.face_v[3 * f + j] == nd[0]) ed[5] = m.face_e[3 * f + j];
        }
        for (int k = 0; k < 4; ++k) ele_face[4 * e + k] = m.tet_f[4 * e + k];
        for (int k = 0; k < 6; ++k) {
            int g = ed[k];
            if (!seen_edge[g]) {
                edge_node[2 * g] = nd[kEdgeStart[k]];
                edge_node[2 * g + 1] = nd[kEdgeEnd[k]];
                type_edge[6 * e + k] = 0;
                seen_edge[g] = 1;
            } else {
                type_edge[6 * e + k] = (edge_node[2 * g] == nd[kEdgeStart[k]]) ? 0 : 1;
            }
        }
        for (int k = 0; k < 4; ++k) {
            int f = ele_face[4 * e + k];
            if (!seen_face[f]) {
                for (int j = 0; j < 3; ++j) {
                    face_node[3 * f + j] = nd[kFacePoint[3 * k + j]];
                    face_edge[3 * f + j] = ed[kFaceEdge[3 * k + j]];
                }
                if (edge_node[2 * face_edge[3 * f + 0]] != nd[kFacePoint[3 * k + 1]]) face_same[3 * f + 0] = 0;
                if (edge_node[2 * face_edge[3 * f + 1]] != nd[kFacePoint[3 * k + 0]]) face_same[3 * f + 1] = 0;
                if (edge_node[2 * face_edge[3 * f + 2]] != nd[kFacePoint[3 * k + 0]]) face_same[3 * f + 2] = 0;
                type_face[4 * e + k] = 0;
                type_face_inv[4 * e + k] = 0;
                seen_face[f] = 1;
            } else {
                int o[3] = {-1, -1, -1};
                for (int a = 0; a < 3; ++a)
                    for (int b = 0; b < 3; ++b)
                        if (nd[kFacePoint[3 * k + a]] == face_node[3 * f + b]) o[a] = b;
                int code = 100 * o[0] + 10 * o[1] + o[2];
                int t = -1, ti = -1;
                switch (code) {
                case 12: t = 0; ti = 0; break;
                case 21: t = 1; ti = 1; break;
                case 102: t = 2; ti = 2; break;
                case 120: t = 3; ti = 4; break;
                case 201: t = 4; ti = 3; break;
                case 210: t = 5; ti = 5; break;
                default: throw std::runtime_error("face permutation not found");
                }
                type_face[4 * e + k] = t;
                type_face_inv[4 * e + k] = ti;
            }
        }
    }
    // |T| = |det J| / 6, :636-646
    volume.assign(E, 0.0);
    for (int e = 0; e < E; ++e) {
        const double* p0 = &m.xyz[3 * ele_node[4 * e]];
        double d[3][3];
        for (int k = 0; k < 3; ++k) {
            const double* pk = &m.xyz[3 * ele_node[4 * e + k + 1]];
            for (int j = 0; j < 3; ++j) d[j][k] = pk[j] - p0[j];
        }
        double det = d[0][0] * (d[1][1] * d[2][2] - d[1][2] * d[2][1]) - d[0][1] * (d[1][0] * d[2][2] - d[1][2] * d[2][0])
                     + d[0][2] * (d[1][0] * d[2][1] - d[1][1] * d[2][0]);
        volume[e] = std::fabs(det / 6.0);
    }

    // ------------------------------------------ DOF numbering, :895-948
    std::vector<double> w(n_geo_total);
    for (int v = 0; v < m.nv; ++v) w[v] = m.femdof_v[v];
    for (int g = 0; g < m.ne; ++g) w[m.nv + g] = m.femdof_e[g];
    for (int f = 0; f < m.nf; ++f) {
        double s = 0.0;
        for (int j = 0; j < 3; ++j) s += w[m.face_v[3 * f + j]];
        w[m.nv + m.ne + f] = s / 3;
    }
    for (int t = 0; t < m.nt; ++t) {
        double s = 0.0;
        for (int j = 0; j < 4; ++j) s += w[m.tet_v[4 * t + j]];
        w[m.nv + m.ne + m.nf + t] = s / 4;
    }
    // the reference's insertion sort only swaps on strict '<': a stable sort
    std::vector<int> order(n_geo_total);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return w[a] < w[b]; });
    auto dim_of = [&](int t) { return t < m.nv ? 0 : t < m.nv + m.ne ? 1 : t < m.nv + m.ne + m.nf ? 2 : 3; };
    location_geometry.assign(n_geo_total, 0);
    location_actualdof.assign(n_geo_total, 0);
    for (int i = 0; i < n_geo_total; ++i) location_geometry[order[i]] = i;
    for (int i = 1; i < n_geo_total; ++i) location_actualdof[i] = location_actualdof[i - 1] + n_dof_geo[dim_of(order[i - 1])];

    // ----------------------------------- transform global -> local, :1016-1110
    const int ndE = M - 1;
    const int ndF = (M - 2) * (M - 3) / 2 + M - 2;
    auto N = [](int a, int b, int c) { return MultiIndexTable::number(a, b, c); };
    std::vector<int> edge_loc(6 * ndE), face_loc(4 * std::max(ndF, 1));
    for (int l = 2; l <= M; ++l) {
        edge_loc[ndE * 0 + l - 2] = N(l, 0, 0);
        edge_loc[ndE * 1 + l - 2] = N(0, l, 0);
        edge_loc[ndE * 2 + l - 2] = N(0, 0, l);
        edge_loc[ndE * 3 + l - 2] = N(1, l - 1, 0);
        edge_loc[ndE * 4 + l - 2] = N(1, 0, l - 1);
        edge_loc[ndE * 5 + l - 2] = N(0, 1, l - 1);
    }
    for (int l1 = 2; l1 <= M; ++l1)
        for (int l2 = 1; l2 <= M - l1; ++l2) {
            int d = (l1 + l2 - 3) * (l1 + l2 - 2) / 2 + l2 - 1;
            face_loc[ndF * 0 + d] = N(1, l1 - 1, l2);
            face_loc[ndF * 1 + d] = N(0, l1, l2);
            face_loc[ndF * 2 + d] = N(l1, 0, l2);
            face_loc[ndF * 3 + d] = N(l1, l2, 0);
        }
    std::vector<std::vector<std::vector<std::pair<int, double>>>> T(E, std::vector<std::vector<std::pair<int, double>>>(n_loc));
    for (int e = 0; e < E; ++e) {
        auto& Te = T[e];
        for (int k = 0; k < 4; ++k) Te[k] = {{geo_first_dof(0, ele_node[4 * e + k]), 1.0}};
        for (int k = 0; k < 6; ++k) {
            int start = geo_first_dof(1, ele_edge[6 * e + k]);
            for (int l = 2; l <= M; ++l) {
                double s = (type_edge[6 * e + k] == 1 && l % 2 == 1) ? -1.0 : 1.0;
                Te[edge_loc[ndE * k + l - 2]] = {{start + l - 2, s}};
            }
        }
        for (int k = 0; k < 4; ++k) {
            int f = ele_face[4 * e + k];
            int fstart = geo_first_dof(2, f);
            int var = type_face_inv[4 * e + k];
            for (int d = 0; d < ndF; ++d) {
                std::vector<std::pair<int, double>> dep;
                for (int j = 0; j < 3; ++j) {
                    int estart = geo_first_dof(1, face_edge[3 * f + j]);
                    for (auto& pr : ft.edge[var][d][j]) {
                        double v = pr.second;
                        if (!face_same[3 * f + j] && pr.first % 2 == 1) v = -v;
                        dep.push_back({estart + pr.first, v});
                    }
                }
                for (auto& pr : ft.face[var][d]) dep.push_back({fstart + pr.first, pr.second});
                Te[face_loc[ndF * k + d]] = dep;
            }
        }
        const int nI = n_dof_geo[3];
        int istart = geo_first_dof(3, e);
        for (int d = 0; d < nI && M >= 4; ++d) {
            auto a = lb.mi.num2idx[d];
            Te[N(a[0] + 2, a[1] + 1, a[2] + 1)] = {{istart + d, 1.0}};
        }
    }
    max_dep = 1;
    for (int e = 0; e < E; ++e)
        for (int i = 0; i < n_loc; ++i) max_dep = std::max(max_dep, (int)T[e][i].size());
    t_n.assign((size_t)E * n_loc, 0);
    t_ind.assign((size_t)E * n_loc * max_dep, 0);
    t_val.assign((size_t)E * n_loc * max_dep, 0.0);
    for (int e = 0; e < E; ++e)
        for (int i = 0; i < n_loc; ++i) {
            size_t b = ((size_t)e * n_loc + i);
            t_n[b] = (int)T[e][i].size();
            for (int j = 0; j < t_n[b]; ++j) {
                t_ind[b * max_dep + j] = T[e][i][j].first;
                t_val[b * max_dep + j] = T[e][i][j].second;
            }
        }
    for (int d = 0; d < 3; ++d) flag_bm[d].assign(n_geo[d], 0);
    if ((int)m.mark_v.size() == m.nv) flag_bm[0] = m.mark_v;
    if ((int)m.mark_e.size() == m.ne) flag_bm[1] = m.mark_e;
    if ((int)m.mark_f.size() == m.nf) flag_bm[2] = m.mark_f;
}

void Space::gather(int e, const double* u, double* loc) const {
    for (int i = 0; i < n_loc; ++i) {
        size_t b = (size_t)e * n_loc + i;
        double s = 0;
        for (int j = 0; j < t_n[b]; ++j) s += u[t_ind[b * max_dep + j]] * t_val[b * max_dep + j];
        loc[i] = s;
    }
}

// src/Miscellaneous.cpp:557-587
void Space::sum_dof(std::vector<int>& out) const {
    out.assign(n_dof, 0);
    for (int v = 0; v < n_geo[0]; ++v) out[geo_first_dof(0, v)] = 1;
    for (int g = 0; g < n_geo[1]; ++g) {
        int p = geo_first_dof(1, g);
        for (int l = 2; l <= M; ++l) out[p + l - 2] = l;
    }
    for (int f = 0; f < n_geo[2]; ++f) {
        int p = geo_first_dof(2, f);
        for (int l1 = 2; l1 <= M; ++l1)
            for (int l2 = 1; l2 <= M - l1; ++l2) out[p + (l1 + l2 - 2) * (l1 + l2 - 3) / 2 + l2 - 1] = l1 + l2;
    }
    for (int t = 0; t < n_geo[3]; ++t) {
        int p = geo_first_dof(3, t);
        for (int l1 = 2; l1 <= M; ++l1)
            for (int l2 = 1; l2 <= M - l1; ++l2)
                for (int l3 = 1; l3 <= M - l1 - l2; ++l3)
                    out[p + MultiIndexTable::number(l1 - 2, l2 - 1, l3 - 1)] = l1 + l2 + l3;
    }
}

// ------------------------------------------------------------- assembly
// Global pattern: diagonal plus, for every element and every pattern entry (r, c)
// of the element matrices, all products of the transform dependencies of r and c.
static void build_pattern(const Space& S, const std::vector<const RefSparse*>& mats, Csr& A) {
    const int n = S.n_dof, nl = S.n_loc, md = S.max_dep;
    // union of the element patterns
    std::vector<std::vector<int>> pu(nl);
    for (const RefSparse* R : mats)
        for (int r = 0; r < nl; ++r) pu[r].insert(pu[r].end(), R->cols[r].begin(), R->cols[r].end());
    for (int r = 0; r < nl; ++r) {
        std::sort(pu[r].begin(), pu[r].end());
        pu[r].erase(std::unique(pu[r].begin(), pu[r].end()), pu[r].end());
    }
    std::vector<std::vector<int>> rows(n);
    std::vector<size_t> clean(n, 1);   // size after the last deduplication of each row
    for (int i = 0; i < n; ++i) rows[i].push_back(i);
    auto dedup = [](std::vector<int>& row) {
        std::sort(row.begin(), row.end());
        row.erase(std::unique(row.begin(), row.end()), row.end());
    };
    for (int e = 0; e < S.n_ele; ++e) {
        for (int r = 0; r < nl; ++r) {
            size_t br = (size_t)e * nl + r;
            for (int a = 0; a < S.t_n[br]; ++a) {
                const int g = S.t_ind[br * md + a];
                auto& row = rows[g];
                for (int c : pu[r]) {
                    size_t bc = (size_t)e * nl + c;
                    for (int b = 0; b < S.t_n[bc]; ++b) row.push_back(S.t_ind[bc * md + b]);
                }
                if (row.size() > 4 * clean[g] + 256) { dedup(row); clean[g] = row.size(); }
            }
        }
    }
#pragma omp parallel for schedule(dynamic, 256)
    for (int i = 0; i < n; ++i) dedup(rows[i]);
    A.n = n;
    A.rowptr.assign(n + 1, 0);
    for (int i = 0; i < n; ++i) A.rowptr[i + 1] = A.rowptr[i] + (int64_t)rows[i].size();
    A.col.assign(A.rowptr[n], 0);
    A.val.assign(A.rowptr[n], 0.0);
    for (int i = 0; i < n; ++i) {
        int64_t p = A.rowptr[i];
        A.col[p++] = i;  // diagonal first (deal.II square convention)
        for (int c : rows[i]) if (c != i) A.col[p++] = c;
        std::vector<int>().swap(rows[i]);
    }
}

static void scatter(const Space& S, const RefSparse& R, int e, double scale, Csr& A) {
    const int nl = S.n_loc, md = S.max_dep;
    for (int r = 0; r < nl; ++r) {
        size_t br = (size_t)e * nl + r;
        for (size_t q = 0; q < R.cols[r].size(); ++q) {
            int c = R.cols[r][q];
            double v = R.vals[r][q] * scale;
            size_t bc = (size_t)e * nl + c;
            for (int a = 0; a < S.t_n[br]; ++a) {
                int gr = S.t_ind[br * md + a];
                double va = v * S.t_val[br * md + a];
                for (int b = 0; b < S.t_n[bc]; ++b) {
                    int64_t p = A.find(gr, S.t_ind[bc * md + b]);
                    A.val[p] += va * S.t_val[bc * md + b];
                }
            }
        }
    }
}

void Space::assemble_mass(Csr& A) const {
    build_pattern(*this, {&ref.mass}, A);
    for (int e = 0; e < n_ele; ++e) scatter(*this, ref.mass, e, 6 * volume[e], A);
}

// dihedral weights, src/Discretize.cpp:1357-1372
static void dihedral(const Space& S, int e, double g[6]) {
    const double* X = S.mesh->xyz.data();
    auto P = [&](int k) { return &X[3 * S.ele_node[4 * e + k]]; };
    for (int k = 0; k < 6; ++k) g[k] = 0;
    for (int i1 = 0; i1 <= 2; ++i1)
        for (int i2 = i1 + 1; i2 <= 3; ++i2) {
            int s = (i1 == 0) ? (i2 % 2 + 1) : 0;
            int t = 6 - i1 - i2 - s;
            const double *p1 = P(i1), *p2 = P(i2), *ps = P(s), *pe = P(t);
            double a[3], b[3], c[3];
            for (int j = 0; j < 3; ++j) { a[j] = pe[j] - ps[j]; b[j] = p1[j] - ps[j]; c[j] = p2[j] - ps[j]; }
            double u[3] = {a[1] * b[2] - a[2] * b[1], -a[0] * b[2] + a[2] * b[0], a[0] * b[1] - a[1] * b[0]};
            double v[3] = {a[1] * c[2] - a[2] * c[1], -a[0] * c[2] + a[2] * c[0], a[0] * c[1] - a[1] * c[0]};
            double cf = 0.25 * (u[0] * v[0] + u[1] * v[1] + u[2] * v[2]);
            // reference-matrix index of the pair: (2,0,0),(1,1,0),(1,0,1),(0,2,0),(0,1,1),(0,0,2)
            int k;
            if (i1 == 0) k = (i2 == 1) ? 0 : (i2 == 2 ? 3 : 5);
            else if (i1 == 1) k = (i2 == 2) ? 1 : 2;
            else k = 4;
            g[k] = cf;
        }
}

void Space::assemble_stiff(Csr& A) const {
    build_pattern(*this, {&ref.stiff[0], &ref.stiff[1], &ref.stiff[2], &ref.stiff[3], &ref.stiff[4], &ref.stiff[5]}, A);
    for (int e = 0; e < n_ele; ++e) {
        double g[6];
        dihedral(*this, e, g);
        double coef = 2.0 / (3 * volume[e]);
        for (int k = 0; k < 6; ++k) {
            if (std::fabs(g[k]) < 1e-12) continue;
            scatter(*this, ref.stiff[k], e, coef * g[k], A);
        }
    }
}

}  // namespace tsem_oracle
