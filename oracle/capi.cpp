// TEST INFRASTRUCTURE ONLY -- C entry points of the CPU oracle, bound with ctypes
// by oracle/__init__.py.  Used only by tests/, __graft_entry__.smoke() and the
// CPU-baseline leg of bench.py.
#include "oracle.hpp"
#include "physics.hpp"
#include "solver.hpp"
#include <cstring>
#include <string>
#include <exception>
#include <stdexcept>
#include <memory>
#include <omp.h>

using namespace tsem_oracle;

namespace {
thread_local std::string g_err;
struct SpaceH {
    Mesh mesh;
    FaceTable table;
    Space space;
    FaceBases fb;
};
}  // namespace

#define OR_TRY(expr) try { expr; } catch (const std::exception& ex) { g_err = ex.what(); return -1; }

extern "C" {

const char* or_last_error() { return g_err.c_str(); }

// OpenMP threads of the parallel loops (the SpMV and the assembly); the GS sweeps
// are sequential like the reference's
void or_set_threads(int n) { omp_set_num_threads(n > 0 ? n : 1); }
int or_get_threads() { return omp_get_max_threads(); }

void* or_space_create(int nv, const double* xyz, int ne, const int* edge_v, int nf, const int* face_v, const int* face_e,
                      int nt, const int* tet_v, const int* tet_f, const int* mark_v, const int* mark_e, const int* mark_f,
                      const int* femdof_v, const int* femdof_e, int M, const char* table_path, int quad_q) {
    try {
        if (M < 4) throw std::runtime_error("the oracle restates the reference for p >= 4 only");
        std::unique_ptr<SpaceH> hp(new SpaceH());
        SpaceH* h = hp.get();
        Mesh& m = h->mesh;
        m.nv = nv; m.ne = ne; m.nf = nf; m.nt = nt;
        m.xyz.assign(xyz, xyz + 3 * nv);
        m.edge_v.assign(edge_v, edge_v + 2 * ne);
        m.face_v.assign(face_v, face_v + 3 * nf);
        m.face_e.assign(face_e, face_e + 3 * nf);
        m.tet_v.assign(tet_v, tet_v + 4 * nt);
        m.tet_f.assign(tet_f, tet_f + 4 * nt);
        if (mark_v) m.mark_v.assign(mark_v, mark_v + nv);
        if (mark_e) m.mark_e.assign(mark_e, mark_e + ne);
        if (mark_f) m.mark_f.assign(mark_f, mark_f + nf);
        m.femdof_v.assign(femdof_v, femdof_v + nv);
        m.femdof_e.assign(femdof_e, femdof_e + ne);
        if (!h->table.load(table_path)) throw std::runtime_error("cannot read face table");
        h->space.build(h->mesh, M, h->table, quad_q);
        h->fb.build(h->space);
        return hp.release();
    } catch (const std::exception& ex) {
        g_err = ex.what();
        return nullptr;
    }
}

void or_space_free(void* h) { delete (SpaceH*)h; }

// n_dof, n_loc, max_dep, n_ele, nq3, nq2, nq1, n_geo[4], n_dof_geo[4]
void or_space_info(void* hh, int* out) {
    auto& S = ((SpaceH*)hh)->space;
    out[0] = S.n_dof; out[1] = S.n_loc; out[2] = S.max_dep; out[3] = S.n_ele;
    out[4] = (int)S.quad.w3.size(); out[5] = (int)S.quad.w2.size(); out[6] = (int)S.quad.w1.size();
    for (int d = 0; d < 4; ++d) { out[7 + d] = S.n_geo[d]; out[11 + d] = S.n_dof_geo[d]; }
}

void or_space_geometry(void* hh, int* type_edge, int* type_face, int* type_face_inv, int* edge_node, int* face_node,
                       int* face_edge, unsigned char* face_same, double* volume, int* ele_edge) {
    auto& S = ((SpaceH*)hh)->space;
    std::memcpy(type_edge, S.type_edge.data(), sizeof(int) * S.type_edge.size());
    std::memcpy(type_face, S.type_face.data(), sizeof(int) * S.type_face.size());
    std::memcpy(type_face_inv, S.type_face_inv.data(), sizeof(int) * S.type_face_inv.size());
    std::memcpy(edge_node, S.edge_node.data(), sizeof(int) * S.edge_node.size());
    std::memcpy(face_node, S.face_node.data(), sizeof(int) * S.face_node.size());
    std::memcpy(face_edge, S.face_edge.data(), sizeof(int) * S.face_edge.size());
    std::memcpy(face_same, S.face_same.data(), S.face_same.size());
    std::memcpy(volume, S.volume.data(), sizeof(double) * S.volume.size());
    std::memcpy(ele_edge, S.ele_edge.data(), sizeof(int) * S.ele_edge.size());
}

void or_space_numbering(void* hh, int* location_geometry, int* location_actualdof) {
    auto& S = ((SpaceH*)hh)->space;
    std::memcpy(location_geometry, S.location_geometry.data(), sizeof(int) * S.location_geometry.size());
    std::memcpy(location_actualdof, S.location_actualdof.data(), sizeof(int) * S.location_actualdof.size());
}

void or_space_transform(void* hh, int* t_n, int* t_ind, double* t_val) {
    auto& S = ((SpaceH*)hh)->space;
    std::memcpy(t_n, S.t_n.data(), sizeof(int) * S.t_n.size());
    std::memcpy(t_ind, S.t_ind.data(), sizeof(int) * S.t_ind.size());
    std::memcpy(t_val, S.t_val.data(), sizeof(double) * S.t_val.size());
}

// include/Correspondence.h:64-109: number -> multi-index for every number of order M,
// and the number of each of those multi-indices back again
void or_multiindex(int M, int* alpha, int* number) {
    MultiIndexTable t;
    t.init(M);
    for (int i = 0; i < t.n; ++i) {
        const auto& a = t.num2idx[i];
        for (int c = 0; c < 3; ++c) alpha[3 * i + c] = a[c];
        number[i] = MultiIndexTable::number(a[0], a[1], a[2]);
    }
}

void or_sum_dof(void* hh, int* out) {
    std::vector<int> s;
    ((SpaceH*)hh)->space.sum_dof(s);
    std::memcpy(out, s.data(), sizeof(int) * s.size());
}

// which: 0 mass, 1..6 stiffness k = which-1; basis: 0 Jacobi basis, 1 actual basis.
// dense is n x n row-major (n = n_loc, or C(M+2,3) for the Jacobi stiffness)
int or_refmat(void* hh, int which, int basis, double* dense, unsigned char* pattern) {
    auto& R = ((SpaceH*)hh)->space.ref;
    const RefSparse* S = nullptr;
    if (which == 0) S = basis ? &R.mass : &R.mass_jac;
    else S = basis ? &R.stiff[which - 1] : &R.stiff_jac[which - 1];
    const int n = S->n;
    if (dense) std::memset(dense, 0, sizeof(double) * n * n);
    if (pattern) std::memset(pattern, 0, (size_t)n * n);
    for (int r = 0; r < n; ++r)
        for (size_t q = 0; q < S->cols[r].size(); ++q) {
            if (dense) dense[(size_t)r * n + S->cols[r][q]] = S->vals[r][q];
            if (pattern) pattern[(size_t)r * n + S->cols[r][q]] = 1;
        }
    return n;
}

void or_basis_values(void* hh, const double* pt, double* out) { ((SpaceH*)hh)->space.lb.basis_values(pt, out); }
void or_basis_gradients(void* hh, const double* pt, double* out) { ((SpaceH*)hh)->space.lb.basis_gradients(pt, out); }
void or_jacobi_values(void* hh, const double* pt, double* out) { ((SpaceH*)hh)->space.lb.jacobi_values(pt, out); }

void or_quadrature(void* hh, double* x3, double* w3, double* b2, double* w2, double* x1, double* w1) {
    auto& Q = ((SpaceH*)hh)->space.quad;
    for (size_t i = 0; i < Q.w3.size(); ++i) { for (int j = 0; j < 3; ++j) x3[3 * i + j] = Q.x3[i][j]; w3[i] = Q.w3[i]; }
    for (size_t i = 0; i < Q.w2.size(); ++i) { for (int j = 0; j < 3; ++j) b2[3 * i + j] = Q.b2[i][j]; w2[i] = Q.w2[i]; }
    for (size_t i = 0; i < Q.w1.size(); ++i) { x1[i] = Q.x1[i]; w1[i] = Q.w1[i]; }
}

void or_element_qpoints(void* hh, double* out) {
    auto& S = ((SpaceH*)hh)->space;
    std::vector<double> p;
    const size_t nq = S.quad.w3.size();
    for (int e = 0; e < S.n_ele; ++e) {
        element_qpoints(S, e, p);
        std::memcpy(out + (size_t)e * nq * 3, p.data(), sizeof(double) * nq * 3);
    }
}

int64_t or_boundary_points(void* hh, int dim, double* out) {
    std::vector<double> p;
    boundary_points(((SpaceH*)hh)->space, dim, p);
    if (out) std::memcpy(out, p.data(), sizeof(double) * p.size());
    return (int64_t)p.size() / 3;
}

void or_rhs(void* hh, const double* f_qp, double* rhs) { calc_rhs(((SpaceH*)hh)->space, f_qp, rhs); }

void* or_assemble_potential(void* hh, const double* v_qp) {
    auto* A = new Csr();
    try {
        assemble_potential(((SpaceH*)hh)->space, v_qp, *A);
    } catch (const std::exception& ex) { g_err = ex.what(); delete A; return nullptr; }
    return A;
}

void or_errors(void* hh, const double* sol, const double* u_qp, const double* gu_qp, double* out) {
    calc_errors(((SpaceH*)hh)->space, sol, u_qp, gu_qp, out, out + 1);
}

void or_density(void* hh, const double* states, int k, const double* occ, double* out) {
    calc_density(((SpaceH*)hh)->space, states, k, occ, out);
}

double or_density_l2_difference(void* hh, const double* u, const double* v, int k, const double* occ) {
    return calc_density_l2_difference(((SpaceH*)hh)->space, u, v, k, occ);
}

// ------------------------------------------------------------------ CSR
void* or_assemble(void* hh, int which) {
    auto* A = new Csr();
    try {
        if (which == 0) ((SpaceH*)hh)->space.assemble_stiff(*A);
        else ((SpaceH*)hh)->space.assemble_mass(*A);
    } catch (const std::exception& ex) { g_err = ex.what(); delete A; return nullptr; }
    return A;
}
void* or_csr_import(int n, const int64_t* rowptr, const int* col, const double* val) {
    auto* A = new Csr();
    A->n = n;
    A->rowptr.assign(rowptr, rowptr + n + 1);
    A->col.assign(col, col + rowptr[n]);
    A->val.assign(val, val + rowptr[n]);
    return A;
}
void* or_csr_copy(void* a) { return new Csr(*(Csr*)a); }
void or_csr_free(void* a) { delete (Csr*)a; }
int64_t or_csr_nnz(void* a) { return ((Csr*)a)->rowptr.back(); }
int or_csr_n(void* a) { return ((Csr*)a)->n; }
void or_csr_export(void* a, int64_t* rowptr, int* col, double* val) {
    Csr& A = *(Csr*)a;
    if (rowptr) std::memcpy(rowptr, A.rowptr.data(), sizeof(int64_t) * A.rowptr.size());
    if (col) std::memcpy(col, A.col.data(), sizeof(int) * A.col.size());
    if (val) std::memcpy(val, A.val.data(), sizeof(double) * A.val.size());
}
void or_csr_vmult(void* a, const double* x, double* y) { ((Csr*)a)->vmult(x, y); }

int or_dirichlet(void* hh, void* a, double* rhs, const double* vb0, const double* vb1, const double* vb2, int modify,
                 int flag) {
    auto* h = (SpaceH*)hh;
    OR_TRY(impose_dirichlet(h->space, h->fb, *(Csr*)a, rhs, vb0, vb1, vb2, modify != 0, flag));
    return 0;
}
int or_neumann(void* hh, double* rhs, const double* g2, int flag) {
    auto* h = (SpaceH*)hh;
    OR_TRY(impose_neumann(h->space, h->fb, rhs, g2, flag));
    return 0;
}
int or_zero_bc(void* hh, void* a, double* rhs, int flag) {
    OR_TRY(impose_zero_bc(((SpaceH*)hh)->space, (Csr*)a, rhs, flag));
    return 0;
}
// read_quad_info (src/QuadInfo.cpp:13-60): a tabulated rule replaces the built one
int or_space_set_quadrature(void* hh, int n1, const double* x1, const double* w1, int n2, const double* b2,
                            const double* w2, int n3, const double* x3, const double* w3) {
    auto* h = (SpaceH*)hh;
    try {
        Quadrature& Q = h->space.quad;
        Q.q = 0;
        Q.x1.assign(x1, x1 + n1);
        Q.w1.assign(w1, w1 + n1);
        Q.b2.resize(n2);
        Q.w2.assign(w2, w2 + n2);
        for (int p = 0; p < n2; ++p) Q.b2[p] = {b2[3 * p], b2[3 * p + 1], b2[3 * p + 2]};
        Q.x3.resize(n3);
        Q.w3.assign(w3, w3 + n3);
        for (int p = 0; p < n3; ++p) Q.x3[p] = {x3[3 * p], x3[3 * p + 1], x3[3 * p + 2]};
        h->fb = FaceBases();
        h->fb.build(h->space);
    } catch (const std::exception& ex) {
        g_err = ex.what();
        return -1;
    }
    return 0;
}
int or_interpolation(void* hh, const double* u_v, const double* u_e, const double* u_f, const double* u_qp,
                     double* out) {
    auto* h = (SpaceH*)hh;
    OR_TRY(calc_interpolation(h->space, h->fb, u_v, u_e, u_f, u_qp, out));
    return 0;
}

// ------------------------------------------------------------------ solvers
void* or_pmg_create(void* a, int p, const int* sum_dof, int step) {
    auto* P = new PMG();
    std::vector<int> s(sum_dof, sum_dof + ((Csr*)a)->n);
    P->init(*(Csr*)a, p, s, step);
    return P;
}
void or_pmg_free(void* p) { delete (PMG*)p; }
int or_pmg_levels(void* p, int* n_dof_layer) {
    auto* P = (PMG*)p;
    if (n_dof_layer) for (int i = 0; i <= P->n_project; ++i) n_dof_layer[i] = P->n_dof_layer[i];
    return P->n_project;
}
void* or_pmg_level_matrix(void* p, int level) { return &((PMG*)p)->A[level]; }
void or_pmg_core_at(void* p, int level, int* out) {
    auto* P = (PMG*)p;
    std::memcpy(out, P->core_at[level].data(), sizeof(int) * P->core_at[level].size());
}
void or_pmg_vcycle(void* p, double* x, const double* r, int smooth) { ((PMG*)p)->vcycle(x, r, smooth); }

void or_gs(void* a, double* x, const double* r, int steps, int dir) {
    if (dir == 0) gs_forward(*(Csr*)a, x, r, steps);
    else if (dir == 1) gs_backward(*(Csr*)a, x, r, steps);
    else gs_symmetric(*(Csr*)a, x, r, steps);
}

// stats: iterations, residual_l1, init_l1, residual_l2, status
int or_pcg(void* a, double* x, const double* b, double tol, double rel_tol, int max_step, int flag, void* pmg, int smooth,
           double omega, double* stats) {
    try {
        PcgStats s = solve_pcg(*(Csr*)a, x, b, tol, rel_tol, max_step, flag, (PMG*)pmg, smooth, omega);
        if (stats) { stats[0] = s.iterations; stats[1] = s.residual_l1; stats[2] = s.init_l1; stats[3] = s.residual_l2; stats[4] = s.status; }
        return s.iterations;
    } catch (const std::exception& ex) { g_err = ex.what(); return -1; }
}

double or_inverse_power(void* a, void* b, double* x, double tol, int max_step, int* iters) {
    return solve_inverse_power(*(Csr*)a, *(Csr*)b, x, tol, max_step, iters);
}

int or_lobpcg(void* a, void* b, int k, double* X, double* lambda, double tol, int max_it, int precond, void* pmg, int smooth,
              double* stats) {
    try {
        LobpcgStats s = solve_lobpcg(*(Csr*)a, *(Csr*)b, k, X, lambda, tol, max_it, precond, (PMG*)pmg, smooth);
        if (stats) { stats[0] = s.iterations; stats[1] = s.residual; stats[2] = s.status; }
        return s.status;
    } catch (const std::exception& ex) { g_err = ex.what(); return -1; }
}

// theta[r], C[m][r] (row-major); returns r
int or_rayleigh_ritz(int m, const double* ga, const double* gb, double* theta, double* c) {
    std::vector<double> GA(ga, ga + (size_t)m * m), GB(gb, gb + (size_t)m * m), T, C;
    const int r = rayleigh_ritz(m, GA, GB, T, C);
    std::memcpy(theta, T.data(), sizeof(double) * r);
    std::memcpy(c, C.data(), sizeof(double) * (size_t)m * r);
    return r;
}

void or_sym_eig(int n, const double* a, double* w, double* v) {
    std::vector<double> A(a, a + (size_t)n * n), W, V;
    sym_eig(n, A, W, V);
    std::memcpy(w, W.data(), sizeof(double) * n);
    std::memcpy(v, V.data(), sizeof(double) * n * n);
}

}  // extern "C"
