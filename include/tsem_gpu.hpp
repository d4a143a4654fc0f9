/* C++ call surface shaped like TSEMLib's TSEM<double> (include/TetrahedralSEM.h:29-331)
 * and TSEMSolver<double> (include/TSEMSolver.h:57-98), header-only, over the C ABI
 * of tsem_gpu.h.  AFEPack's RegularMesh / FEMSpace are replaced by tsem_gpu::Mesh
 * (plain arrays), deal.II's SparseMatrix by tsem_gpu::SparseMatrix (a device CSR
 * with the same diagonal-first rows) and Vector<double> by std::vector<double>.
 * Errors are thrown as tsem_gpu::Error carrying the tsem_status. */
#ifndef TSEM_GPU_HPP
#define TSEM_GPU_HPP

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <map>
#include <tuple>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "tsem_gpu.h"

namespace tsem_gpu {

using Vector = std::vector<double>;

struct Error : std::runtime_error {
    tsem_status status;
    Error(tsem_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline tsem_status check(tsem_status rc, bool allow_solver_status = false) {
    if (rc == TSEM_OK) return rc;
    if (allow_solver_status && (rc == TSEM_MAXIT || rc == TSEM_BREAKDOWN)) return rc;
    throw Error(rc, tsem_last_error());
}

/* Multiindex<3> and Correspondence<3> (include/Multiindex.h,
 * include/Correspondence.h:64-109): the numbering of the multi-indices |alpha| <= M
 * that numbers the Jacobi basis (by total degree, then alpha1 + alpha2, then
 * alpha2), with the reference's method names; the table comes from the library
 * (tsem_multiindex). */
struct Multiindex {
    int index[3] = {0, 0, 0};
    int sum() const { return index[0] + index[1] + index[2]; }
    int n_nonzero() const { return (index[0] != 0) + (index[1] != 0) + (index[2] != 0); }
};

class Correspondence {
   public:
    Correspondence() = default;
    explicit Correspondence(int order_truncate) { init(order_truncate); }
    void init(int order_truncate) {
        if (order_truncate < 0 || order_truncate > 40) throw Error(TSEM_INVALID, "order must be in [0, 40]");
        M_ = order_truncate;
        const int n = (M_ + 1) * (M_ + 2) * (M_ + 3) / 6;
        alpha_.assign(3 * (size_t)n, 0);
        check(tsem_multiindex(M_, alpha_.data(), nullptr));
        const int w = M_ + 1;
        lookup_.assign((size_t)w * w * w, -1);
        begin_.assign(M_ + 2, n);
        for (int i = n - 1; i >= 0; --i) {
            const int32_t* a = &alpha_[3 * (size_t)i];
            lookup_[((size_t)a[0] * w + a[1]) * w + a[2]] = i;
            begin_[a[0] + a[1] + a[2]] = i;
        }
    }
    /* the number of a multi-index with |alpha| <= M */
    int index2number(const Multiindex& a) const {
        if (a.index[0] < 0 || a.index[1] < 0 || a.index[2] < 0 || a.sum() > M_)
            throw Error(TSEM_INVALID, "multi-index outside the truncation order");
        const int w = M_ + 1;
        return lookup_[((size_t)a.index[0] * w + a.index[1]) * w + a.index[2]];
    }
    Multiindex number2index(int number) const {
        if (number < 0 || number >= n_index()) throw Error(TSEM_INVALID, "number outside the table");
        Multiindex a;
        for (int c = 0; c < 3; ++c) a.index[c] = alpha_[3 * (size_t)number + c];
        return a;
    }
    int n_index() const { return (int)(alpha_.size() / 3); }
    /* first number of |alpha| = order, and the first of |alpha| = order + 1 */
    int n_index_begin(int order) const { return begin_.at(order); }
    int n_index_end(int order) const { return begin_.at(order + 1); }

   private:
    int M_ = 0;
    std::vector<int32_t> alpha_, lookup_, begin_;
};

/* Mesh with the AFEPack relations the space needs.  from_tets() numbers edges and
 * faces by first appearance while walking the tetrahedra (edges E01 E02 E03 E12
 * E13 E23, face k opposite vertex k) and gives the P2 DOF order of a walk over
 * each tetrahedron's vertices then edges; a caller holding AFEPack's own order
 * overwrites femdof_v / femdof_e. */
struct Mesh {
    std::vector<double> xyz;
    std::vector<int32_t> edge_v, face_v, face_e, tet_v, tet_f;
    std::vector<int32_t> mark_v, mark_e, mark_f, femdof_v, femdof_e;

    int32_t nv() const { return (int32_t)(xyz.size() / 3); }
    int32_t ne() const { return (int32_t)(edge_v.size() / 2); }
    int32_t nf() const { return (int32_t)(face_v.size() / 3); }
    int32_t nt() const { return (int32_t)(tet_v.size() / 4); }

    static Mesh from_tets(std::vector<double> xyz, const std::vector<int32_t>& tets) {
        static const int ea[6] = {0, 0, 0, 1, 1, 2}, eb[6] = {1, 2, 3, 2, 3, 3};
        static const int fp[4][3] = {{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}};
        Mesh m;
        m.xyz = std::move(xyz);
        m.tet_v = tets;
        const int32_t nt = m.nt();
        std::map<std::pair<int32_t, int32_t>, int32_t> edges;
        std::map<std::array<int32_t, 3>, int32_t> faces;
        std::vector<int32_t> tet_e((size_t)nt * 6);
        m.tet_f.resize((size_t)nt * 4);
        for (int32_t t = 0; t < nt; ++t) {
            const int32_t* v = &tets[(size_t)t * 4];
            for (int k = 0; k < 6; ++k) {
                const int32_t a = v[ea[k]], b = v[eb[k]];
                auto key = std::make_pair(std::min(a, b), std::max(a, b));
                auto it = edges.find(key);
                if (it == edges.end()) {
                    it = edges.emplace(key, m.ne()).first;
                    m.edge_v.push_back(a);
                    m.edge_v.push_back(b);
                }
                tet_e[(size_t)t * 6 + k] = it->second;
            }
            for (int k = 0; k < 4; ++k) {
                std::array<int32_t, 3> fv = {v[fp[k][0]], v[fp[k][1]], v[fp[k][2]]};
                std::array<int32_t, 3> key = fv;
                std::sort(key.begin(), key.end());
                auto it = faces.find(key);
                if (it == faces.end()) {
                    it = faces.emplace(key, m.nf()).first;
                    m.face_v.insert(m.face_v.end(), fv.begin(), fv.end());
                }
                m.tet_f[(size_t)t * 4 + k] = it->second;
            }
        }
        m.face_e.resize(m.face_v.size());
        for (int32_t f = 0; f < m.nf(); ++f)
            for (int k = 0; k < 3; ++k) {
                const int32_t a = m.face_v[(size_t)f * 3 + (k + 1) % 3], b = m.face_v[(size_t)f * 3 + (k + 2) % 3];
                m.face_e[(size_t)f * 3 + k] = edges.at(std::make_pair(std::min(a, b), std::max(a, b)));
            }
        m.femdof_v.assign(m.nv(), -1);
        m.femdof_e.assign(m.ne(), -1);
        int32_t next = 0;
        for (int32_t t = 0; t < nt; ++t) {
            for (int k = 0; k < 4; ++k) {
                int32_t& d = m.femdof_v[tets[(size_t)t * 4 + k]];
                if (d < 0) d = next++;
            }
            for (int k = 0; k < 6; ++k) {
                int32_t& d = m.femdof_e[tet_e[(size_t)t * 6 + k]];
                if (d < 0) d = next++;
            }
        }
        m.mark_v.assign(m.nv(), 0);
        m.mark_e.assign(m.ne(), 0);
        m.mark_f.assign(m.nf(), 0);
        return m;
    }

    tsem_mesh desc() const {
        tsem_mesh d;
        d.nv = nv(); d.ne = ne(); d.nf = nf(); d.nt = nt();
        d.xyz = xyz.data(); d.edge_v = edge_v.data(); d.face_v = face_v.data(); d.face_e = face_e.data();
        d.tet_v = tet_v.data(); d.tet_f = tet_f.data();
        d.mark_v = mark_v.empty() ? nullptr : mark_v.data();
        d.mark_e = mark_e.empty() ? nullptr : mark_e.data();
        d.mark_f = mark_f.empty() ? nullptr : mark_f.data();
        d.femdof_v = femdof_v.data(); d.femdof_e = femdof_e.data();
        return d;
    }
};

/* deal.II SparseMatrix<double> counterpart: a device CSR, diagonal first in each row */
class SparseMatrix {
   public:
    SparseMatrix() = default;
    explicit SparseMatrix(tsem_csr h) : h_(h) {}
    SparseMatrix(const SparseMatrix& o) : h_(nullptr) {
        if (o.h_) check(tsem_csr_copy(o.h_, &h_));
    }
    SparseMatrix& operator=(const SparseMatrix& o) {
        if (this != &o) {
            reset();
            if (o.h_) check(tsem_csr_copy(o.h_, &h_));
        }
        return *this;
    }
    SparseMatrix(SparseMatrix&& o) noexcept : h_(o.h_) { o.h_ = nullptr; }
    SparseMatrix& operator=(SparseMatrix&& o) noexcept {
        if (this != &o) { reset(); h_ = o.h_; o.h_ = nullptr; }
        return *this;
    }
    ~SparseMatrix() { reset(); }

    tsem_csr handle() const { return h_; }
    int64_t m() const { int64_t n = 0, z = 0; check(tsem_csr_info(h_, &n, &z)); return n; }
    int64_t n_nonzero_elements() const { int64_t n = 0, z = 0; check(tsem_csr_info(h_, &n, &z)); return z; }
    /* dst = A src (SparseMatrix::vmult) */
    void vmult(Vector& dst, const Vector& src) const {
        dst.resize(src.size());
        check(tsem_csr_spmv(h_, src.data(), dst.data(), 0, nullptr));
    }
    void export_csr(std::vector<int64_t>& rowptr, std::vector<int32_t>& col, Vector& val) const {
        int64_t n = 0, z = 0;
        check(tsem_csr_info(h_, &n, &z));
        rowptr.resize(n + 1); col.resize(z); val.resize(z);
        check(tsem_csr_export(h_, rowptr.data(), col.data(), val.data()));
    }

   private:
    void reset() { if (h_) tsem_csr_destroy(h_); h_ = nullptr; }
    tsem_csr h_ = nullptr;
};

/* TSEM<double>: the space of order M on a mesh with its stiffness and mass matrices */
class TSEM {
   public:
    int n_dof_total = 0, n_element = 0, n_index = 0;
    std::array<int, 3> n_q_point{};   // 1-D, 2-D, 3-D rule sizes
    SparseMatrix stiff_matrix, mass_matrix;

    /* TSEM(M, qinfo_order, mesh, fem_space) (include/TetrahedralSEM.h:199-201) */
    TSEM(int polynomial_order, int qinfo_order, const Mesh& mesh) : mesh_(mesh) {
        tsem_mesh d = mesh_.desc();
        check(tsem_space_create(&d, polynomial_order, qinfo_order, &h_));
        int64_t info[15] = {0};
        check(tsem_space_info(h_, info));
        n_dof_total = (int)info[0];
        n_index = (int)info[1];
        n_element = (int)info[2];
        n_q_point = {(int)info[6], (int)info[5], (int)info[4]};
        build_stiff_matrix();
        build_mass_matrix();
    }
    TSEM(const TSEM&) = delete;
    TSEM& operator=(const TSEM&) = delete;
    ~TSEM() { if (h_) tsem_space_destroy(h_); }
    tsem_space handle() const { return h_; }

    void build_stiff_matrix() { tsem_csr a = nullptr; check(tsem_assemble(h_, 0, &a)); stiff_matrix = SparseMatrix(a); }
    void build_mass_matrix() { tsem_csr a = nullptr; check(tsem_assemble(h_, 1, &a)); mass_matrix = SparseMatrix(a); }

    std::vector<int32_t> calc_sum_dof() const {
        std::vector<int32_t> s(n_dof_total);
        check(tsem_space_sum_dof(h_, s.data()));
        return s;
    }

    /* calc_rhs(rhs, fem_space, f) (src/Discretize.cpp:1397-1463): f at the element quadrature points */
    template <class F>
    void calc_rhs(Vector& rhs, F&& f) const {
        const std::vector<double> q = element_qpoints();
        std::vector<double> fv(q.size() / 3);
        for (size_t i = 0; i < fv.size(); ++i) fv[i] = f(&q[3 * i]);
        rhs.assign(n_dof_total, 0.0);
        check(tsem_rhs(h_, fv.data(), rhs.data()));
    }
    /* impose_boundary_condition(rhs, mesh, g, flag): Neumann load (src/Discretize.cpp:2011-2063) */
    template <class G>
    void impose_boundary_condition(Vector& rhs, G&& g, int flag_boundary) const {
        std::vector<double> gv = boundary_values(g, 2, [&](int m) { return m == flag_boundary; });
        check(tsem_neumann(h_, rhs.data(), gv.data(), flag_boundary));
    }
    /* impose_boundary_condition(A, rhs, mesh, u, modify, flag): Dirichlet (src/Discretize.cpp:1683-2008) */
    template <class U>
    void impose_boundary_condition(SparseMatrix& A, Vector& rhs, U&& u, bool flag_modify_matrix, int flag_boundary) const {
        auto on = [&](int m) { return flag_boundary == -2 || (flag_boundary == -1 ? m != 0 : m == flag_boundary); };
        std::vector<double> vb[3];
        for (int d = 0; d < 3; ++d) vb[d] = boundary_values(u, d, on);
        check(tsem_dirichlet(h_, A.handle(), rhs.data(), vb[0].data(), vb[1].data(), vb[2].data(),
                             flag_modify_matrix ? 1 : 0, flag_boundary));
    }
    /* u at the boundary points of the geometries `on` selects, zero at the others (the
     * Dirichlet and Neumann kernels read only the selected ones) */
    template <class U, class On>
    std::vector<double> boundary_values(U&& u, int dim, On&& on) const {
        const std::vector<double> pts = boundary_points(dim);
        int64_t ng = 0;
        check(tsem_geometry_marks(h_, dim, nullptr, &ng));
        std::vector<int32_t> marks((size_t)ng);
        check(tsem_geometry_marks(h_, dim, marks.data(), &ng));
        std::vector<double> v(pts.size() / 3, 0.0);
        const size_t per = ng > 0 ? v.size() / (size_t)ng : 0;
        for (size_t g = 0; g < (size_t)ng; ++g)
            if (on(marks[g]))
                for (size_t i = g * per; i < (g + 1) * per; ++i) v[i] = u(&pts[3 * i]);
        return v;
    }
    /* impose_zero_boundary_condition (src/Discretize.cpp:1466-1569) */
    void impose_zero_boundary_condition(SparseMatrix& A, int flag_boundary = 1) const {
        check(tsem_zero_bc(h_, A.handle(), nullptr, flag_boundary));
    }
    void impose_zero_boundary_condition(Vector& v, int flag_boundary = 1) const {
        check(tsem_zero_bc(h_, nullptr, v.data(), flag_boundary));
    }
    /* {calc_l2_error, calc_l2_error_gradient} (src/CalcError.cpp:64-266) against u and grad u */
    template <class U, class GU>
    std::pair<double, double> calc_errors(const Vector& sol, U&& u, GU&& grad_u) const {
        const std::vector<double> q = element_qpoints();
        const size_t nq = q.size() / 3;
        std::vector<double> uq(nq), gq(3 * nq);
        for (size_t i = 0; i < nq; ++i) { uq[i] = u(&q[3 * i]); grad_u(&q[3 * i], &gq[3 * i]); }
        double out[2] = {0, 0};
        check(tsem_errors(h_, sol.data(), uq.data(), gq.data(), out));
        return {out[0], out[1]};
    }

    std::vector<double> element_qpoints() const {
        std::vector<double> q((size_t)n_element * n_q_point[2] * 3);
        check(tsem_element_qpoints(h_, q.data()));
        return q;
    }
    std::vector<double> boundary_points(int dim) const {
        int64_t cnt = 0;
        check(tsem_boundary_points(h_, dim, nullptr, &cnt));
        std::vector<double> p((size_t)cnt * 3);
        check(tsem_boundary_points(h_, dim, p.data(), &cnt));
        return p;
    }

   private:
    Mesh mesh_;                 // the space keeps pointers into the mesh arrays
    tsem_space h_ = nullptr;
};

/* TSEMSolver<double>: PCG (flags 0 none, 1 Jacobi, 4 p-multigrid) and LOBPCG */
class TSEMSolver {
   public:
    tsem_stats last_stats{};

    TSEMSolver() = default;
    TSEMSolver(const TSEMSolver&) = delete;
    TSEMSolver& operator=(const TSEMSolver&) = delete;
    ~TSEMSolver() { clear(); }

    /* init_PMG (src/TSEMSolver.cpp:36-135); smoother 0 = exact Gauss-Seidel, 1 = Chebyshev */
    void init_PMG(const SparseMatrix& A, int polynomial_order, const std::vector<int32_t>& sum_dof, int order_step = 1,
                  int smoother = 0) {
        clear();
        pmg_A_ = A.handle();
        p_ = polynomial_order;
        sum_dof_ = sum_dof;
        step_ = order_step;
        smoother_ = smoother;
    }
    /* solve_PCG (src/TSEMSolver.cpp:1776-1929): x in/out; returns the status */
    tsem_status solve_PCG(const SparseMatrix& A, Vector& x, const Vector& r, double tol = 1.0e-8,
                          unsigned max_step = 100000, unsigned flag_preconditioner = 1, unsigned ite_step = 1,
                          double var = 1, double tol_rel = 0.0) {
        const bool sor = flag_preconditioner == 2 || flag_preconditioner == 3;
        tsem_solver sv = solver(A.handle(), (int)flag_preconditioner,
                                flag_preconditioner == 4 ? (int)var : (sor ? (int)ite_step : 1), tol, tol_rel,
                                (int)max_step, sor ? var : 0.0);
        x.resize(r.size(), 0.0);
        return check(tsem_solve_pcg(sv, r.data(), x.data(), &last_stats), true);
    }
    /* solve_CG (src/TSEMSolver.cpp:1698-1773) */
    tsem_status solve_CG(const SparseMatrix& A, Vector& x, const Vector& r, double tol = 1.0e-8,
                         unsigned max_step = 100000) {
        return solve_PCG(A, x, r, tol, max_step, 0);
    }
    /* solve_PMG (src/TSEMSolver.cpp:1446-1536): stationary V-cycles on x until ||A x - r||_1 < tol */
    tsem_status solve_PMG(Vector& x, const Vector& r, double tol = 1.0e-8, unsigned max_step = 100000,
                          unsigned smooth_step = 2) {
        if (!pmg_A_) throw Error(TSEM_INVALID, "init_PMG must precede solve_PMG");
        tsem_solver sv = solver(pmg_A_, 4, (int)smooth_step, 0.0, 0.0, 1);
        x.resize(r.size(), 0.0);
        return check(tsem_solve_pmg(sv, r.data(), x.data(), tol, (int)max_step, &last_stats), true);
    }
    /* solve_InversePower (src/TSEMSolver.cpp:2042-2068): x <- A^-1 B x, B-normalised,
     * until x^T A x changes by less than tol; returns that Rayleigh quotient */
    double solve_InversePower(Vector& x, const SparseMatrix& A, const SparseMatrix& B,
                              bool Flag_Output_Intermediate = false, double tol = 1.0e-8, unsigned max_step = 1000) {
        (void)Flag_Output_Intermediate;
        Vector rhs, tmp;
        B.vmult(rhs, x);
        double e_last = 0.0, e_now = 0.0;
        for (unsigned it = 0; it < max_step; ++it) {
            solve_PCG(A, x, rhs, tol * 1.0e-2, max_step * 100);
            B.vmult(rhs, x);
            double c = 0.0;
            for (size_t i = 0; i < x.size(); ++i) c += rhs[i] * x[i];
            const double f = 1.0 / std::sqrt(c);
            for (size_t i = 0; i < x.size(); ++i) { x[i] *= f; rhs[i] *= f; }
            A.vmult(tmp, x);
            e_now = 0.0;
            for (size_t i = 0; i < x.size(); ++i) e_now += tmp[i] * x[i];
            if (it > 0 && std::fabs(e_now - e_last) < tol) break;
            e_last = e_now;
        }
        return e_now;
    }
    /* solve_LOBPCG (src/TSEMSolver.cpp:2225-2406): the block x in/out (M-orthonormal
     * Ritz vectors), eigenvalues returned; stop on the relative residual tol of the
     * first n_want (0 = all) pairs */
    std::vector<double> solve_LOBPCG(TSEM& tsem, std::vector<Vector>& x, const SparseMatrix& A, const SparseMatrix& B,
                                     bool Flag_Output_Intermediate = false, double tol = 1.0e-8,
                                     unsigned max_step = 1000, int n_want = 0, int smooth_step = 2) {
        (void)tsem;
        (void)Flag_Output_Intermediate;
        const int k = (int)x.size();
        const size_t n = x.empty() ? 0 : x[0].size();
        const bool pmg = pmg_A_ && pmg_A_ == A.handle();
        tsem_solver sv = solver(A.handle(), pmg ? 4 : 1, pmg ? smooth_step : 1, 0.0, 0.0, 1);
        std::vector<double> X(n * k), lam(k);
        for (int j = 0; j < k; ++j) std::copy(x[j].begin(), x[j].end(), X.begin() + (size_t)j * n);
        check(tsem_solve_lobpcg(sv, B.handle(), k, n_want > 0 ? n_want : k, X.data(), lam.data(), tol, (int)max_step,
                                &last_stats),
              true);
        for (int j = 0; j < k; ++j) std::copy(X.begin() + (size_t)j * n, X.begin() + (size_t)(j + 1) * n, x[j].begin());
        return lam;
    }

   private:
    struct Key {
        tsem_csr A; int precond, smooth; double tol, tol_rel; int max_step; double omega;
        bool operator<(const Key& o) const {
            return std::tie(A, precond, smooth, tol, tol_rel, max_step, omega) <
                   std::tie(o.A, o.precond, o.smooth, o.tol, o.tol_rel, o.max_step, o.omega);
        }
    };
    tsem_solver solver(tsem_csr A, int precond, int smooth, double tol, double tol_rel, int max_step,
                       double omega = 0.0) {
        const Key key{A, precond, smooth, tol, tol_rel, max_step, omega};
        auto it = solvers_.find(key);
        if (it != solvers_.end()) return it->second;
        if (precond == 4 && pmg_A_ != A) throw Error(TSEM_INVALID, "init_PMG must precede flag_preconditioner 4");
        tsem_solver_opts o{};
        o.precond = precond;
        o.pmg_order_step = step_;
        o.smooth_steps = smooth;
        o.smoother = smoother_;
        o.tol_abs_l1 = tol;
        o.tol_rel = tol_rel;
        o.max_iter = max_step;
        o.omega = omega;
        tsem_solver sv = nullptr;
        check(tsem_solver_create(A, precond == 4 ? sum_dof_.data() : nullptr, p_, &o, &sv));
        solvers_[key] = sv;
        return sv;
    }
    void clear() {
        for (auto& kv : solvers_) tsem_solver_destroy(kv.second);
        solvers_.clear();
    }
    std::map<Key, tsem_solver> solvers_;
    tsem_csr pmg_A_ = nullptr;
    int p_ = 1, step_ = 1, smoother_ = 0;
    std::vector<int32_t> sum_dof_;
};

}  // namespace tsem_gpu

#endif /* TSEM_GPU_HPP */
