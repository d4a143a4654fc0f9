// Host construction of the TSEM space (see space.hpp).
#include "space.hpp"
#include "jacobi.cuh"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <stdexcept>
#include <string>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace tsem {

namespace {
// local face k is opposite vertex k; vertex order and the edges opposite those
// vertices as the reference lists them (src/BuildSpace.cpp:505-512)
const int kFacePt[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
const int kFaceEd[4][3] = {{5, 4, 3}, {5, 2, 1}, {4, 2, 0}, {3, 1, 0}};
const int kEdgeA[6] = {0, 0, 0, 1, 1, 2};
const int kEdgeB[6] = {1, 2, 3, 2, 3, 3};

void require(bool ok, const std::string& msg) {
    if (!ok) throw std::invalid_argument(msg);
}
int binom(int n, int k) {
    if (k < 0 || n < k) return 0;
    long v = 1;
    for (int i = 1; i <= k; ++i) v = v * (n - k + i) / i;
    return (int)v;
}
}  // namespace

void SpaceHost::build(const MeshInput& in, int order) {
    require(order >= 1 && order <= 16, "polynomial order must be in [1, 16]");
    M = order;
    nv = in.nv; ne = in.ne; nf = in.nf; nt = in.nt;
    require(nv > 0 && ne > 0 && nf > 0 && nt > 0, "empty mesh");
    require(in.xyz && in.edge_v && in.face_v && in.face_e && in.tet_v && in.tet_f && in.femdof_v && in.femdof_e,
            "missing mesh array");
    lt.build(M);
    n_loc = lt.n_loc;
    pat.build(lt);
    ftab.derive(M);
    ndE = binom(M - 1, 1); ndF = binom(M - 1, 2); ndI = binom(M - 1, 3);
    xyz.assign(in.xyz, in.xyz + 3 * (size_t)nv);
    auto marks = [](const int* p, int n, std::vector<int>& out) { out.assign(n, 0); if (p) out.assign(p, p + n); };
    marks(in.mark_v, nv, mark_v); marks(in.mark_e, ne, mark_e); marks(in.mark_f, nf, mark_f);

    // ---- input validation: the AFEPack relations the reference relies on
    for (int i = 0; i < 2 * ne; ++i) require(in.edge_v[i] >= 0 && in.edge_v[i] < nv, "edge vertex out of range");
    for (int i = 0; i < 3 * nf; ++i) {
        require(in.face_v[i] >= 0 && in.face_v[i] < nv, "face vertex out of range");
        require(in.face_e[i] >= 0 && in.face_e[i] < ne, "face edge out of range");
    }
    for (int f = 0; f < nf; ++f)
        for (int k = 0; k < 3; ++k) {
            int e = in.face_e[3 * f + k], a = in.face_v[3 * f + (k + 1) % 3], b = in.face_v[3 * f + (k + 2) % 3];
            int u = in.edge_v[2 * e], w = in.edge_v[2 * e + 1];
            require((u == a && w == b) || (u == b && w == a), "face edge k must join the face vertices other than k");
        }
    for (int t = 0; t < nt; ++t)
        for (int k = 0; k < 4; ++k) {
            int v = in.tet_v[4 * t + k], f = in.tet_f[4 * t + k];
            require(v >= 0 && v < nv && f >= 0 && f < nf, "tetrahedron index out of range");
            for (int j = 0; j < 3; ++j) require(in.face_v[3 * f + j] != v, "tetrahedron face k must not contain vertex k");
        }

    // ---- geometry information, src/BuildSpace.cpp:471-646
    const int E = nt;
    ele_node.assign(4 * (size_t)E, -1); ele_edge.assign(6 * (size_t)E, -1); ele_face.assign(4 * (size_t)E, -1);
    type_edge.assign(6 * (size_t)E, 0); type_face.assign(4 * (size_t)E, 0); type_face_inv.assign(4 * (size_t)E, 0);
    edge_node.assign(2 * (size_t)ne, -1); face_node.assign(3 * (size_t)nf, -1); face_edge.assign(3 * (size_t)nf, -1);
    face_same.assign(3 * (size_t)nf, 1);
    volume.assign(E, 0.0);
    std::vector<uint8_t> seen_e(ne, 0), seen_f(nf, 0);
    for (int e = 0; e < E; ++e) {
        int* nd = &ele_node[4 * (size_t)e];
        int* ed = &ele_edge[6 * (size_t)e];
        for (int k = 0; k < 4; ++k) nd[k] = in.tet_v[4 * (size_t)e + k];
        for (int k = 0; k < 4; ++k) ele_face[4 * (size_t)e + k] = in.tet_f[4 * (size_t)e + k];
        // local edges from the faces opposite P3, P2 and P1
        {
            const int f3 = in.tet_f[4 * (size_t)e + 3], f2 = in.tet_f[4 * (size_t)e + 2], f1 = in.tet_f[4 * (size_t)e + 1];
            for (int j = 0; j < 3; ++j) {
                const int v = in.face_v[3 * f3 + j], g = in.face_e[3 * f3 + j];
                if (v == nd[0]) ed[3] = g;
                else if (v == nd[1]) ed[1] = g;
                else if (v == nd[2]) ed[0] = g;
            }
            for (int j = 0; j < 3; ++j) {
                const int v = in.face_v[3 * f2 + j], g = in.face_e[3 * f2 + j];
                if (v == nd[0]) ed[4] = g;
                else if (v == nd[1]) ed[2] = g;
            }
            for (int j = 0; j < 3; ++j)
                if (in.face_v[3 * f1 + j] == nd[0]) ed[5] = in.face_e[3 * f1 + j];
            for (int k = 0; k < 6; ++k) require(ed[k] >= 0, "tetrahedron faces do not share the expected edges");
        }
        for (int k = 0; k < 6; ++k) {
            const int g = ed[k];
            if (!seen_e[g]) {
                seen_e[g] = 1;
                edge_node[2 * g] = nd[kEdgeA[k]];
                edge_node[2 * g + 1] = nd[kEdgeB[k]];
            } else {
                type_edge[6 * (size_t)e + k] = edge_node[2 * g] == nd[kEdgeA[k]] ? 0 : 1;
            }
        }
        for (int k = 0; k < 4; ++k) {
            const int f = ele_face[4 * (size_t)e + k];
            if (!seen_f[f]) {
                seen_f[f] = 1;
                for (int j = 0; j < 3; ++j) {
                    face_node[3 * f + j] = nd[kFacePt[k][j]];
                    face_edge[3 * f + j] = ed[kFaceEd[k][j]];
                }
                // edge opposite face vertex 0 runs v1 -> v2, the other two start at v0
                face_same[3 * f + 0] = edge_node[2 * face_edge[3 * f + 0]] == nd[kFacePt[k][1]];
                face_same[3 * f + 1] = edge_node[2 * face_edge[3 * f + 1]] == nd[kFacePt[k][0]];
                face_same[3 * f + 2] = edge_node[2 * face_edge[3 * f + 2]] == nd[kFacePt[k][0]];
            } else {
                int o[3];
                for (int a = 0; a < 3; ++a) {
                    o[a] = -1;
                    for (int b = 0; b < 3; ++b)
                        if (nd[kFacePt[k][a]] == face_node[3 * f + b]) o[a] = b;
                    require(o[a] >= 0, "face shared by two tetrahedra with different vertices");
                }
                // local vertex a sits at global position o[a]
                static const int code_t[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
                static const int t_of[6] = {0, 1, 2, 3, 4, 5}, ti_of[6] = {0, 1, 2, 4, 3, 5};
                for (int c = 0; c < 6; ++c)
                    if (o[0] == code_t[c][0] && o[1] == code_t[c][1] && o[2] == code_t[c][2]) {
                        type_face[4 * (size_t)e + k] = (int8_t)t_of[c];
                        type_face_inv[4 * (size_t)e + k] = (int8_t)ti_of[c];
                    }
            }
        }
        const double* p0 = &xyz[3 * (size_t)nd[0]];
        double d[3][3];
        for (int k = 0; k < 3; ++k)
            for (int j = 0; j < 3; ++j) d[j][k] = xyz[3 * (size_t)nd[k + 1] + j] - p0[j];
        const double det = d[0][0] * (d[1][1] * d[2][2] - d[1][2] * d[2][1]) - d[0][1] * (d[1][0] * d[2][2] - d[1][2] * d[2][0]) +
                           d[0][2] * (d[1][0] * d[2][1] - d[1][1] * d[2][0]);
        require(std::fabs(det) > 0, "degenerate tetrahedron");
        volume[e] = std::fabs(det / 6.0);
    }

    // ---- DOF numbering: stable sort of all geometries by weight, :895-948
    const int64_t ng = (int64_t)nv + ne + nf + nt;
    std::vector<double> w(ng);
    {
        std::vector<uint8_t> used((size_t)nv + ne, 0);
        for (int i = 0; i < nv; ++i) {
            int v = in.femdof_v[i];
            require(v >= 0 && v < nv + ne && !used[v], "femdof numbers must be a permutation of 0..nv+ne-1");
            used[v] = 1;
            w[i] = v;
        }
        for (int i = 0; i < ne; ++i) {
            int v = in.femdof_e[i];
            require(v >= 0 && v < nv + ne && !used[v], "femdof numbers must be a permutation of 0..nv+ne-1");
            used[v] = 1;
            w[nv + i] = v;
        }
    }
    for (int f = 0; f < nf; ++f) {
        double s = 0.0;
        for (int j = 0; j < 3; ++j) s += w[in.face_v[3 * f + j]];
        w[(size_t)nv + ne + f] = s / 3;
    }
    for (int t = 0; t < nt; ++t) {
        double s = 0.0;
        for (int j = 0; j < 4; ++j) s += w[in.tet_v[4 * (size_t)t + j]];
        w[(size_t)nv + ne + nf + t] = s / 4;
    }
    std::vector<int> order_(ng);
    std::iota(order_.begin(), order_.end(), 0);
    std::stable_sort(order_.begin(), order_.end(), [&](int a, int b) { return w[a] < w[b]; });
    const int ndg[4] = {1, ndE, ndF, ndI};
    auto dim_of = [&](int64_t g) { return g < nv ? 0 : g < nv + ne ? 1 : g < (int64_t)nv + ne + nf ? 2 : 3; };
    location_geometry.assign(ng, 0);
    location_actualdof.assign(ng, 0);
    for (int64_t i = 0; i < ng; ++i) location_geometry[order_[i]] = (int)i;
    int64_t acc = 0;
    for (int64_t i = 0; i < ng; ++i) {
        require(acc < (int64_t)1 << 31, "too many DOFs for 32-bit column indices");
        location_actualdof[i] = (int)acc;
        acc += ndg[dim_of(order_[i])];
    }
    n_dof = acc;
    vdof.resize(nv); edof.resize(ne); fdof.resize(nf); tdof.resize(nt);
    for (int i = 0; i < nv; ++i) vdof[i] = location_actualdof[location_geometry[i]];
    for (int i = 0; i < ne; ++i) edof[i] = location_actualdof[location_geometry[(size_t)nv + i]];
    for (int i = 0; i < nf; ++i) fdof[i] = location_actualdof[location_geometry[(size_t)nv + ne + i]];
    for (int i = 0; i < nt; ++i) tdof[i] = location_actualdof[location_geometry[(size_t)nv + ne + nf + i]];

    // ---- transforms global -> local, src/BuildSpace.cpp:1016-1110
    std::vector<int> edge_loc(6 * std::max(ndE, 1)), face_loc(4 * std::max(ndF, 1));
    for (int l = 2; l <= M; ++l) {
        edge_loc[0 * ndE + l - 2] = mi_number(l, 0, 0);
        edge_loc[1 * ndE + l - 2] = mi_number(0, l, 0);
        edge_loc[2 * ndE + l - 2] = mi_number(0, 0, l);
        edge_loc[3 * ndE + l - 2] = mi_number(1, l - 1, 0);
        edge_loc[4 * ndE + l - 2] = mi_number(1, 0, l - 1);
        edge_loc[5 * ndE + l - 2] = mi_number(0, 1, l - 1);
    }
    for (int l1 = 2; l1 <= M; ++l1)
        for (int l2 = 1; l2 <= M - l1; ++l2) {
            const int d = face_dof_index(l1, l2);
            face_loc[0 * ndF + d] = mi_number(1, l1 - 1, l2);
            face_loc[1 * ndF + d] = mi_number(0, l1, l2);
            face_loc[2 * ndF + d] = mi_number(l1, 0, l2);
            face_loc[3 * ndF + d] = mi_number(l1, l2, 0);
        }
    max_dep = 1;
    for (int v = 0; v < 6; ++v)
        for (int d = 0; d < ndF; ++d)
            max_dep = std::max(max_dep, (int)(ftab.edge[v][d].size() + ftab.face[v][d].size()));
    t_n.assign((size_t)E * n_loc, 0);
    t_ind.assign((size_t)E * n_loc * max_dep, 0);
    t_val.assign((size_t)E * n_loc * max_dep, 0.0);
#pragma omp parallel for schedule(static)
    for (int e = 0; e < E; ++e) {
        auto put = [&](int loc, int g, double v) {
            size_t b = (size_t)e * n_loc + loc;
            int j = t_n[b]++;
            t_ind[b * max_dep + j] = g;
            t_val[b * max_dep + j] = v;
        };
        for (int k = 0; k < 4; ++k) put(k, vdof[ele_node[4 * (size_t)e + k]], 1.0);
        for (int k = 0; k < 6; ++k) {
            const int s = edof[ele_edge[6 * (size_t)e + k]];
            const bool rev = type_edge[6 * (size_t)e + k] == 1;
            for (int l = 2; l <= M; ++l) put(edge_loc[k * ndE + l - 2], s + l - 2, (rev && (l & 1)) ? -1.0 : 1.0);
        }
        for (int k = 0; k < 4; ++k) {
            const int f = ele_face[4 * (size_t)e + k];
            const int var = type_face_inv[4 * (size_t)e + k];
            for (int d = 0; d < ndF; ++d) {
                const int loc = face_loc[k * ndF + d];
                for (auto& t : ftab.edge[var][d]) {
                    double v = t.v;
                    if (!face_same[3 * f + t.k] && (t.idx & 1)) v = -v;
                    put(loc, edof[face_edge[3 * f + t.k]] + t.idx, v);
                }
                for (auto& t : ftab.face[var][d]) put(loc, fdof[f] + t.idx, t.v);
            }
        }
        for (int d = 0; d < ndI; ++d) {
            auto a = mi_index(d);
            put(mi_number(a[0] + 2, a[1] + 1, a[2] + 1), tdof[e] + d, 1.0);
        }
    }
    // ---- polynomial degree per DOF
    sum_dof.assign(n_dof, 0);
    for (int i = 0; i < nv; ++i) sum_dof[vdof[i]] = 1;
    for (int i = 0; i < ne; ++i)
        for (int l = 2; l <= M; ++l) sum_dof[edof[i] + l - 2] = l;
    for (int i = 0; i < nf; ++i)
        for (int l1 = 2; l1 <= M; ++l1)
            for (int l2 = 1; l2 <= M - l1; ++l2) sum_dof[fdof[i] + face_dof_index(l1, l2)] = l1 + l2;
    for (int i = 0; i < nt; ++i)
        for (int d = 0; d < ndI; ++d) {
            auto a = mi_index(d);
            sum_dof[tdof[i] + d] = a[0] + a[1] + a[2] + 4;
        }
}

void SpaceHost::closure(int e, int* out) const {
    int c = 0;
    for (int k = 0; k < 4; ++k) out[c++] = vdof[ele_node[4 * (size_t)e + k]];
    for (int k = 0; k < 6; ++k)
        for (int i = 0; i < ndE; ++i) out[c++] = edof[ele_edge[6 * (size_t)e + k]] + i;
    for (int k = 0; k < 4; ++k)
        for (int i = 0; i < ndF; ++i) out[c++] = fdof[ele_face[4 * (size_t)e + k]] + i;
    for (int i = 0; i < ndI; ++i) out[c++] = tdof[e] + i;
}

void PatternCandidates::build(const SpaceHost& S) {
    const int64_t ng = (int64_t)S.nv + S.ne + S.nf + S.nt;
    // elements around every geometry
    std::vector<int64_t> cnt(ng + 1, 0);
    auto gid_v = [&](int i) { return (int64_t)i; };
    auto gid_e = [&](int i) { return (int64_t)S.nv + i; };
    auto gid_f = [&](int i) { return (int64_t)S.nv + S.ne + i; };
    auto gid_t = [&](int i) { return (int64_t)S.nv + S.ne + S.nf + i; };
    for (int e = 0; e < S.nt; ++e) {
        for (int k = 0; k < 4; ++k) cnt[gid_v(S.ele_node[4 * (size_t)e + k]) + 1]++;
        for (int k = 0; k < 6; ++k) cnt[gid_e(S.ele_edge[6 * (size_t)e + k]) + 1]++;
        for (int k = 0; k < 4; ++k) cnt[gid_f(S.ele_face[4 * (size_t)e + k]) + 1]++;
        cnt[gid_t(e) + 1]++;
    }
    for (int64_t g = 0; g < ng; ++g) cnt[g + 1] += cnt[g];
    std::vector<int> inc(cnt[ng]);
    {
        std::vector<int64_t> pos(cnt.begin(), cnt.end() - 1);
        for (int e = 0; e < S.nt; ++e) {
            for (int k = 0; k < 4; ++k) inc[pos[gid_v(S.ele_node[4 * (size_t)e + k])]++] = e;
            for (int k = 0; k < 6; ++k) inc[pos[gid_e(S.ele_edge[6 * (size_t)e + k])]++] = e;
            for (int k = 0; k < 4; ++k) inc[pos[gid_f(S.ele_face[4 * (size_t)e + k])]++] = e;
            inc[pos[gid_t(e)]++] = e;
        }
    }
    // sorted union of the closures of those elements
    std::vector<std::vector<int>> lists(ng);
#pragma omp parallel
    {
        std::vector<int> buf(S.n_loc);
        std::vector<int> acc;
#pragma omp for schedule(dynamic, 256)
        for (int64_t g = 0; g < ng; ++g) {
            acc.clear();
            for (int64_t q = cnt[g]; q < cnt[g + 1]; ++q) {
                S.closure(inc[q], buf.data());
                acc.insert(acc.end(), buf.begin(), buf.end());
            }
            std::sort(acc.begin(), acc.end());
            acc.erase(std::unique(acc.begin(), acc.end()), acc.end());
            lists[g] = acc;
        }
    }
    geo_start.assign(ng + 1, 0);
    for (int64_t g = 0; g < ng; ++g) geo_start[g + 1] = geo_start[g] + (int64_t)lists[g].size();
    cand.resize(geo_start[ng]);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t g = 0; g < ng; ++g) std::copy(lists[g].begin(), lists[g].end(), cand.begin() + geo_start[g]);
    row_geo.assign(S.n_dof, -1);
    for (int i = 0; i < S.nv; ++i) row_geo[S.vdof[i]] = (int)gid_v(i);
    for (int i = 0; i < S.ne; ++i)
        for (int k = 0; k < S.ndE; ++k) row_geo[S.edof[i] + k] = (int)gid_e(i);
    for (int i = 0; i < S.nf; ++i)
        for (int k = 0; k < S.ndF; ++k) row_geo[S.fdof[i] + k] = (int)gid_f(i);
    for (int i = 0; i < S.nt; ++i)
        for (int k = 0; k < S.ndI; ++k) row_geo[S.tdof[i] + k] = (int)gid_t(i);
}

}  // namespace tsem
