// TEST INFRASTRUCTURE ONLY -- CPU oracle (see oracle.hpp).
// Gauss-Seidel smoothers, p-multigrid, PCG, inverse power and block LOBPCG.
// Restates src/TSEMSolver.cpp:36-135 (init_PMG), :207-245/:345-383 (injection),
// :573-656 (principal coarse matrices), :924-1077 (GS sweeps), :1120-1183
// (V-cycle), :1776-1929 (PCG), :2042-2068 (inverse power).  The block LOBPCG
// follows :2225-2406 in structure (Rayleigh-Ritz on [X, W, P]) but solves the
// full 3k x 3k projected problem, which the reference's dsygvx call does not.
#include "oracle.hpp"
#include "solver.hpp"
#include <cmath>
#include <algorithm>
#include <stdexcept>

namespace tsem_oracle {

// src/TSEMSolver.cpp:924-937
void gs_forward(const Csr& A, double* x, const double* r, int steps) {
    for (int s = 0; s < steps; ++s)
        for (int row = 0; row < A.n; ++row) {
            double v = r[row];
            for (int64_t p = A.rowptr[row] + 1; p < A.rowptr[row + 1]; ++p) v -= x[A.col[p]] * A.val[p];
            x[row] = v / A.val[A.rowptr[row]];
        }
}
// :991-1004
void gs_backward(const Csr& A, double* x, const double* r, int steps) {
    for (int s = 0; s < steps; ++s)
        for (int row = A.n - 1; row >= 0; --row) {
            double v = r[row];
            for (int64_t p = A.rowptr[row] + 1; p < A.rowptr[row + 1]; ++p) v -= x[A.col[p]] * A.val[p];
            x[row] = v / A.val[A.rowptr[row]];
        }
}
// :1058-1077
void gs_symmetric(const Csr& A, double* x, const double* r, int steps) {
    for (int s = 0; s < steps; ++s) {
        gs_forward(A, x, r, 1);
        gs_backward(A, x, r, 1);
    }
}

// src/TSEMSolver.cpp:36-135 with n_order_each_layer = order_step
void PMG::init(const Csr& fine, int p, const std::vector<int>& sum_dof, int s) {
    n_project = (p + s - 1) / s - 1 + ((p - 1) % s == 0 ? 0 : 1);
    std::vector<int> order(n_project + 1);
    order[0] = p;
    order[n_project] = 1;
    for (int i = 1; i < n_project; ++i) order[i] = order[i - 1] - s;
    const int n = fine.n;
    n_dof_layer.assign(n_project + 1, 0);
    n_dof_layer[0] = n;
    core_at.assign(n_project, {});
    A.assign(n_project + 1, Csr());
    A[0] = fine;
    // global dof -> position on each coarse level (-1 when absent)
    std::vector<std::vector<int>> pos(n_project + 1, std::vector<int>(n, -1));
    for (int i = 0; i < n; ++i) pos[0][i] = i;
    for (int ip = 0; ip < n_project; ++ip) {
        int nf = 0, nc = 0;
        core_at[ip].assign(n_dof_layer[ip], -1);
        for (int i = 0; i < n; ++i) {
            bool f = sum_dof[i] <= order[ip], c = sum_dof[i] <= order[ip + 1];
            if (f) {
                if (c) { core_at[ip][nf] = nc; pos[ip + 1][i] = nc; ++nc; }
                ++nf;
            }
        }
        n_dof_layer[ip + 1] = nc;
        // principal submatrix of the finest matrix, :573-656
        Csr& C = A[ip + 1];
        C.n = nc;
        C.rowptr.assign(nc + 1, 0);
        std::vector<int> glob(nc);
        for (int i = 0; i < n; ++i) if (pos[ip + 1][i] >= 0) glob[pos[ip + 1][i]] = i;
        for (int r = 0; r < nc; ++r) {
            int g = glob[r];
            int64_t cnt = 0;
            for (int64_t q = fine.rowptr[g]; q < fine.rowptr[g + 1]; ++q) if (pos[ip + 1][fine.col[q]] >= 0) ++cnt;
            C.rowptr[r + 1] = C.rowptr[r] + cnt;
        }
        C.col.resize(C.rowptr[nc]);
        C.val.resize(C.rowptr[nc]);
        for (int r = 0; r < nc; ++r) {
            int g = glob[r];
            int64_t o = C.rowptr[r];
            for (int64_t q = fine.rowptr[g]; q < fine.rowptr[g + 1]; ++q) {
                int cc = pos[ip + 1][fine.col[q]];
                if (cc >= 0) { C.col[o] = cc; C.val[o] = fine.val[q]; ++o; }
            }
        }
    }
}

// src/TSEMSolver.cpp:1120-1183 with ite_step = 1
void PMG::vcycle(double* x, const double* r, int smooth) const {
    std::vector<std::vector<double>> xs(n_project + 1), rs(n_project + 1);
    rs[0].assign(r, r + A[0].n);
    for (int i = 1; i <= n_project; ++i) { xs[i].assign(A[i].n, 0.0); rs[i].assign(A[i].n, 0.0); }
    auto X = [&](int i) { return i == 0 ? x : xs[i].data(); };
    std::vector<double> v;
    for (int i = 0; i < n_project; ++i) {
        gs_forward(A[i], X(i), rs[i].data(), smooth);
        v.assign(A[i].n, 0.0);
        A[i].vmult(X(i), v.data());
        for (int j = 0; j < A[i].n; ++j) v[j] = rs[i][j] - v[j];
        for (int j = 0; j < A[i].n; ++j) if (core_at[i][j] >= 0) rs[i + 1][core_at[i][j]] = v[j];
        std::fill(xs[i + 1].begin(), xs[i + 1].end(), 0.0);
    }
    gs_symmetric(A[n_project], X(n_project), rs[n_project].data(), (smooth + 1) / 2);
    for (int i = n_project - 1; i >= 0; --i) {
        double* xi = X(i);
        const double* xc = X(i + 1);
        for (int j = 0; j < A[i].n; ++j) if (core_at[i][j] >= 0) xi[j] += xc[core_at[i][j]];
        gs_backward(A[i], xi, rs[i].data(), smooth);
    }
}

static double l1norm(const std::vector<double>& v) { double s = 0; for (double a : v) s += std::fabs(a); return s; }
static double l2norm(const double* v, int n) { double s = 0; for (int i = 0; i < n; ++i) s += v[i] * v[i]; return std::sqrt(s); }

// ite_SOR / ite_SSOR (src/TSEMSolver.cpp:1288-1345): lexicographic sweeps with relaxation
static void sor_sweep(const Csr& A, double* x, const double* r, double omega, bool forward) {
    const int n = A.n;
    for (int k = 0; k < n; ++k) {
        const int row = forward ? k : n - 1 - k;
        double c = r[row];
        for (int64_t p = A.rowptr[row] + 1; p < A.rowptr[row + 1]; ++p) c -= x[A.col[p]] * A.val[p];
        x[row] = (1 - omega) * x[row] + omega * c / A.val[A.rowptr[row]];
    }
}

// src/TSEMSolver.cpp:1776-1929 (flags 0, 1, 2, 3, 4); flags 2, 3: omega and `smooth` sweeps
PcgStats solve_pcg(const Csr& A, double* x, const double* b, double tol, double rel_tol, int max_step, int flag,
                   const PMG* pmg, int smooth, double omega) {
    const int n = A.n;
    std::vector<double> tmp(n), rk(n), yk(x, x + n), pk(n);
    A.vmult(x, rk.data());
    for (int i = 0; i < n; ++i) rk[i] -= b[i];
    auto precond = [&]() {
        if (flag == 0) yk = rk;
        else if (flag == 1) for (int i = 0; i < n; ++i) yk[i] = rk[i] / A.val[A.rowptr[i]];
        else if (flag == 2 || flag == 3) {
            for (int it = 0; it < smooth; ++it) {
                sor_sweep(A, yk.data(), rk.data(), omega, true);
                if (flag == 3) sor_sweep(A, yk.data(), rk.data(), omega, false);
            }
        }
        else if (flag == 4) pmg->vcycle(yk.data(), rk.data(), smooth);
        else throw std::runtime_error("unsupported preconditioner");
    };
    precond();
    for (int i = 0; i < n; ++i) pk[i] = -yk[i];
    PcgStats st;
    double res = l1norm(rk);
    st.init_l1 = res;
    const double bnorm = l2norm(b, n);
    auto done = [&]() {
        if (rel_tol > 0) return l2norm(rk.data(), n) <= rel_tol * bnorm;
        return res < tol;
    };
    double rty = 0;
    for (int i = 0; i < n; ++i) rty += rk[i] * yk[i];
    int it = 0;
    while (!done()) {
        A.vmult(pk.data(), tmp.data());
        double pap = 0;
        for (int i = 0; i < n; ++i) pap += pk[i] * tmp[i];
        double alpha = rty / pap;
        for (int i = 0; i < n; ++i) x[i] += alpha * pk[i];
        for (int i = 0; i < n; ++i) rk[i] += alpha * tmp[i];
        std::fill(yk.begin(), yk.end(), 0.0);
        precond();
        double rty_next = 0;
        for (int i = 0; i < n; ++i) rty_next += rk[i] * yk[i];
        double beta = rty_next / rty;
        for (int i = 0; i < n; ++i) pk[i] = pk[i] * beta - yk[i];
        res = l1norm(rk);
        ++it;
        if (it > max_step) break;
        rty = rty_next;
    }
    st.iterations = it;
    st.residual_l1 = res;
    st.residual_l2 = l2norm(rk.data(), n);
    st.status = done() ? 0 : 1;
    return st;
}

// src/TSEMSolver.cpp:2042-2068
double solve_inverse_power(const Csr& A, const Csr& B, double* x, double tol, int max_step, int* iters) {
    const int n = A.n;
    std::vector<double> rhs(n), tmp(n);
    B.vmult(x, rhs.data());
    double e_last = 0, e_now = 0;
    int it = 0;
    for (; it < max_step; ++it) {
        solve_pcg(A, x, rhs.data(), tol * 1e-2, 0, max_step * 100, 1, nullptr, 0);
        B.vmult(x, rhs.data());
        double c = 0;
        for (int i = 0; i < n; ++i) c += rhs[i] * x[i];
        double s = std::sqrt(c);
        for (int i = 0; i < n; ++i) { x[i] /= s; rhs[i] /= s; }
        A.vmult(x, tmp.data());
        e_now = 0;
        for (int i = 0; i < n; ++i) e_now += tmp[i] * x[i];
        if (it > 0 && std::fabs(e_now - e_last) < tol) break;
        e_last = e_now;
    }
    if (iters) *iters = it;
    return e_now;
}

// symmetric eigen-decomposition by cyclic Jacobi rotations (ascending order)
void sym_eig(int n, std::vector<double> a, std::vector<double>& w, std::vector<double>& v) {
    v.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) v[(size_t)i * n + i] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0, tot = 0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                tot += a[(size_t)i * n + j] * a[(size_t)i * n + j];
                if (i != j) off += a[(size_t)i * n + j] * a[(size_t)i * n + j];
            }
        if (off <= 1e-30 * tot || off == 0) break;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) {
                double apq = a[(size_t)p * n + q];
                if (std::fabs(apq) < 1e-300) continue;
                double app = a[(size_t)p * n + p], aqq = a[(size_t)q * n + q];
                double th = (aqq - app) / (2 * apq);
                double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1));
                double c = 1 / std::sqrt(t * t + 1), s = t * c;
                for (int k = 0; k < n; ++k) {
                    double akp = a[(size_t)k * n + p], akq = a[(size_t)k * n + q];
                    a[(size_t)k * n + p] = c * akp - s * akq;
                    a[(size_t)k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    double apk = a[(size_t)p * n + k], aqk = a[(size_t)q * n + k];
                    a[(size_t)p * n + k] = c * apk - s * aqk;
                    a[(size_t)q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    double vkp = v[(size_t)k * n + p], vkq = v[(size_t)k * n + q];
                    v[(size_t)k * n + p] = c * vkp - s * vkq;
                    v[(size_t)k * n + q] = s * vkp + c * vkq;
                }
            }
    }
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](int i, int j) { return a[(size_t)i * n + i] < a[(size_t)j * n + j]; });
    w.assign(n, 0.0);
    std::vector<double> vs((size_t)n * n);
    for (int j = 0; j < n; ++j) {
        w[j] = a[(size_t)idx[j] * n + idx[j]];
        for (int k = 0; k < n; ++k) vs[(size_t)k * n + j] = v[(size_t)k * n + idx[j]];
    }
    v.swap(vs);
}

// Rayleigh-Ritz on the columns of S (n x m, column-major blocks): returns the m'
// Ritz pairs of the B-orthonormalised span, ascending; coefficients C (m x m').
int rayleigh_ritz(int m, const std::vector<double>& GA0, const std::vector<double>& GB0, std::vector<double>& theta,
                         std::vector<double>& C) {
    // unit B-norm scaling of the basis before the rank test
    std::vector<double> dsc(m), GA(GA0), GB(GB0);
    for (int i = 0; i < m; ++i) dsc[i] = GB0[(size_t)i * m + i] > 0 ? 1.0 / std::sqrt(GB0[(size_t)i * m + i]) : 0.0;
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j) { GA[(size_t)i * m + j] *= dsc[i] * dsc[j]; GB[(size_t)i * m + j] *= dsc[i] * dsc[j]; }
    std::vector<double> wb, U;
    sym_eig(m, GB, wb, U);
    double mx = 0;
    for (double x : wb) mx = std::max(mx, std::fabs(x));
    std::vector<int> keep;
    for (int j = 0; j < m; ++j) if (wb[j] > 1e-13 * mx) keep.push_back(j);
    const int r = (int)keep.size();
    // Q = U_keep D^{-1/2}
    std::vector<double> Q((size_t)m * r);
    for (int a = 0; a < r; ++a)
        for (int i = 0; i < m; ++i) Q[(size_t)i * r + a] = U[(size_t)i * m + keep[a]] / std::sqrt(wb[keep[a]]);
    std::vector<double> H((size_t)r * r, 0.0);
    for (int a = 0; a < r; ++a)
        for (int b = 0; b < r; ++b) {
            double s = 0;
            for (int i = 0; i < m; ++i)
                for (int j = 0; j < m; ++j) s += Q[(size_t)i * r + a] * GA[(size_t)i * m + j] * Q[(size_t)j * r + b];
            H[(size_t)a * r + b] = s;
        }
    for (int a = 0; a < r; ++a)
        for (int b = 0; b < a; ++b) { double s = 0.5 * (H[(size_t)a * r + b] + H[(size_t)b * r + a]); H[(size_t)a * r + b] = H[(size_t)b * r + a] = s; }
    std::vector<double> Y;
    sym_eig(r, H, theta, Y);
    C.assign((size_t)m * r, 0.0);
    for (int i = 0; i < m; ++i)
        for (int b = 0; b < r; ++b) {
            double s = 0;
            for (int a = 0; a < r; ++a) s += Q[(size_t)i * r + a] * Y[(size_t)a * r + b];
            C[(size_t)i * r + b] = s * dsc[i];
        }
    return r;
}

// Block LOBPCG for the k smallest pairs of A x = lambda B x.  X is n x k column
// blocks (X[j*n + i]).  precond: 1 Jacobi, 4 p-MG V-cycle (one cycle from zero).
LobpcgStats solve_lobpcg(const Csr& A, const Csr& B, int k, double* X, double* lambda, double tol, int max_it,
                         int precond, const PMG* pmg, int smooth) {
    const int n = A.n;
    LobpcgStats st;
    std::vector<double> AX((size_t)n * k), BX((size_t)n * k), W((size_t)n * k), AW((size_t)n * k), BW((size_t)n * k);
    std::vector<double> P, AP, BP;
    auto dot = [&](const double* a, const double* b) { double s = 0; for (int i = 0; i < n; ++i) s += a[i] * b[i]; return s; };
    auto apply = [&](const Csr& M_, const double* src, double* dst, int cols) {
        for (int j = 0; j < cols; ++j) M_.vmult(src + (size_t)j * n, dst + (size_t)j * n);
    };
    // initial Rayleigh-Ritz on X
    apply(A, X, AX.data(), k);
    apply(B, X, BX.data(), k);
    {
        std::vector<double> GA((size_t)k * k), GB((size_t)k * k), th, C;
        for (int a = 0; a < k; ++a)
            for (int b = 0; b < k; ++b) {
                GA[(size_t)a * k + b] = dot(X + (size_t)a * n, AX.data() + (size_t)b * n);
                GB[(size_t)a * k + b] = dot(X + (size_t)a * n, BX.data() + (size_t)b * n);
            }
        int r = rayleigh_ritz(k, GA, GB, th, C);
        if (r < k) throw std::runtime_error("initial block is rank deficient");
        std::vector<double> nx((size_t)n * k, 0.0), nax((size_t)n * k, 0.0), nbx((size_t)n * k, 0.0);
        for (int b = 0; b < k; ++b)
            for (int a = 0; a < k; ++a) {
                double c = C[(size_t)a * r + b];
                for (int i = 0; i < n; ++i) {
                    nx[(size_t)b * n + i] += c * X[(size_t)a * n + i];
                    nax[(size_t)b * n + i] += c * AX[(size_t)a * n + i];
                    nbx[(size_t)b * n + i] += c * BX[(size_t)a * n + i];
                }
            }
        std::copy(nx.begin(), nx.end(), X);
        AX.swap(nax); BX.swap(nbx);
        for (int j = 0; j < k; ++j) lambda[j] = th[j];
    }
    int np = 0;  // columns held in P
    int it = 0;
    for (; it < max_it; ++it) {
        // residuals and convergence
        double worst = 0;
        for (int j = 0; j < k; ++j) {
            double* w = W.data() + (size_t)j * n;
            for (int i = 0; i < n; ++i) w[i] = AX[(size_t)j * n + i] - lambda[j] * BX[(size_t)j * n + i];
            double rn = std::sqrt(dot(w, w)) / (std::fabs(lambda[j]) * std::sqrt(dot(BX.data() + (size_t)j * n, BX.data() + (size_t)j * n)));
            worst = std::max(worst, rn);
        }
        st.residual = worst;
        if (worst < tol) break;
        // precondition
        for (int j = 0; j < k; ++j) {
            double* w = W.data() + (size_t)j * n;
            if (precond == 1) {
                for (int i = 0; i < n; ++i) w[i] /= A.val[A.rowptr[i]];
            } else {
                std::vector<double> r(w, w + n), z(n, 0.0);
                pmg->vcycle(z.data(), r.data(), smooth);
                std::copy(z.begin(), z.end(), w);
            }
        }
        // W -= X (BX^T W): the preconditioned residuals B-orthogonal to X (B-orthonormal
        // after the Rayleigh-Ritz step), so that the Gram matrices need not resolve W's
        // small part outside span(X) next to its large part inside it
        {
            std::vector<double> c((size_t)k * k);
            for (int a = 0; a < k; ++a)
                for (int j = 0; j < k; ++j) c[(size_t)a * k + j] = dot(BX.data() + (size_t)a * n, W.data() + (size_t)j * n);
            for (int j = 0; j < k; ++j) {
                double* w = W.data() + (size_t)j * n;
                for (int a = 0; a < k; ++a) {
                    const double ca = c[(size_t)a * k + j];
                    const double* xa = X + (size_t)a * n;
                    for (int i = 0; i < n; ++i) w[i] -= ca * xa[i];
                }
            }
        }
        apply(A, W.data(), AW.data(), k);
        apply(B, W.data(), BW.data(), k);
        const int m = 2 * k + np;
        std::vector<const double*> S(m), AS(m), BS(m);
        for (int j = 0; j < k; ++j) {
            S[j] = X + (size_t)j * n; AS[j] = AX.data() + (size_t)j * n; BS[j] = BX.data() + (size_t)j * n;
            S[k + j] = W.data() + (size_t)j * n; AS[k + j] = AW.data() + (size_t)j * n; BS[k + j] = BW.data() + (size_t)j * n;
        }
        for (int j = 0; j < np; ++j) {
            S[2 * k + j] = P.data() + (size_t)j * n; AS[2 * k + j] = AP.data() + (size_t)j * n; BS[2 * k + j] = BP.data() + (size_t)j * n;
        }
        std::vector<double> GA((size_t)m * m), GB((size_t)m * m), th, C;
        for (int a = 0; a < m; ++a)
            for (int b = a; b < m; ++b) {
                GA[(size_t)a * m + b] = GA[(size_t)b * m + a] = dot(S[a], AS[b]);
                GB[(size_t)a * m + b] = GB[(size_t)b * m + a] = dot(S[a], BS[b]);
            }
        int r = rayleigh_ritz(m, GA, GB, th, C);
        if (r < k) { st.status = 2; break; }
        std::vector<double> nx((size_t)n * k, 0.0), nax((size_t)n * k, 0.0), nbx((size_t)n * k, 0.0);
        std::vector<double> np_((size_t)n * k, 0.0), nap((size_t)n * k, 0.0), nbp((size_t)n * k, 0.0);
        for (int b = 0; b < k; ++b)
            for (int a = 0; a < m; ++a) {
                double c = C[(size_t)a * r + b];
                for (int i = 0; i < n; ++i) {
                    nx[(size_t)b * n + i] += c * S[a][i];
                    nax[(size_t)b * n + i] += c * AS[a][i];
                    nbx[(size_t)b * n + i] += c * BS[a][i];
                }
                if (a >= k)
                    for (int i = 0; i < n; ++i) {
                        np_[(size_t)b * n + i] += c * S[a][i];
                        nap[(size_t)b * n + i] += c * AS[a][i];
                        nbp[(size_t)b * n + i] += c * BS[a][i];
                    }
            }
        std::copy(nx.begin(), nx.end(), X);
        AX.swap(nax); BX.swap(nbx);
        P.swap(np_);
        // A P and B P recomputed from P: combined like P they lose their relative
        // accuracy when P is small (cancellation), and the Gram matrices of the
        // next step would no longer describe the same vectors
        AP.assign((size_t)n * k, 0.0); BP.assign((size_t)n * k, 0.0);
        apply(A, P.data(), AP.data(), k);
        apply(B, P.data(), BP.data(), k);
        np = k;
        for (int j = 0; j < k; ++j) lambda[j] = th[j];
    }
    st.iterations = it;
    if (st.status == 0 && st.residual >= tol) st.status = 1;
    return st;
}

}  // namespace tsem_oracle
