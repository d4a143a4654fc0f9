// TEST INFRASTRUCTURE ONLY -- CPU oracle (see oracle.hpp).
// Right-hand sides, boundary conditions and error norms.
// Restates src/BuildSpace.cpp:53-170 (2-D/1-D and interpolation bases),
// src/Discretize.cpp:1397-1463 (rhs), :1466-1569 (zero BC), :1683-1776 (Dirichlet
// by modal projection), :2011-2063 (Neumann), src/CalcError.cpp:64-266 (errors),
// src/PointInfo.cpp:60-91 and src/CalcError.cpp:703-735 (densities).
#include <map>
#include "oracle.hpp"
#include "physics.hpp"
#include <cmath>
#include <algorithm>

namespace tsem_oracle {

static void jac_run(int al, int be, double x, int kmax, double* J) {
    J[0] = 1.0;
    if (kmax < 1) return;
    J[1] = jacobi_gen(al, be, 1, x);
    for (int k = 1; k < kmax; ++k)
        J[k + 1] = ((x - coef_a(al, be, 2, k)) * J[k] - coef_a(al, be, 3, k) * J[k - 1]) / coef_a(al, be, 1, k);
}

void FaceBases::build(const Space& S) {
    const int M = S.M;
    const Quadrature& Q = S.quad;
    nq1 = (int)Q.x1.size();
    nq2 = (int)Q.w2.size();
    ndE = M - 1;
    ndF = (M - 2) * (M - 3) / 2 + M - 2;
    interp1.assign((size_t)nq1 * ndE, 0.0);
    for (int p = 0; p < nq1; ++p) {
        const double xp = 2 * Q.x1[p] - 1;
        std::vector<double> J(M + 1);
        jac_run(1, 1, xp, M - 2, J.data());
        for (int l = 0; l < ndE; ++l) interp1[(size_t)p * ndE + l] = J[l];
    }
    face_val.assign((size_t)nq2 * ndF, 0.0);
    interp2.assign((size_t)nq2 * ndF, 0.0);
    add0.assign((size_t)nq2 * ndE, 0.0);
    add1.assign((size_t)nq2 * ndE, 0.0);
    for (int p = 0; p < nq2; ++p) {
        const double x = Q.b2[p][0], y = Q.b2[p][1];
        const double xi = 2 * x / (1 - y) - 1, eta = 2 * y - 1;
        std::vector<double> Jx(M + 2), Je(M + 2);
        // face basis values, src/BuildSpace.cpp:53-71
        jac_run(-1, -1, xi, M, Jx.data());
        Jx[1] = xi;
        for (int l1 = 2; l1 <= M; ++l1) {
            jac_run(2 * l1 - 1, -1, eta, M, Je.data());
            for (int l2 = 1; l2 <= M - l1; ++l2) {
                int d = (l1 + l2 - 2) * (l1 + l2 - 3) / 2 + l2 - 1;
                face_val[(size_t)p * ndF + d] = 2 * std::pow(1 - y, l1) * Jx[l1] * Je[l2];
            }
        }
        // interpolation bases, src/BuildSpace.cpp:113-143
        std::vector<double> Ix(M + 1), Ie(M + 2);
        jac_run(1, 1, xi, M - 2, Ix.data());
        for (int l1 = 2; l1 <= M; ++l1) {
            jac_run(2 * l1 - 1, 1, eta, M - l1, Ie.data());
            for (int l2 = 1; l2 <= M - l1; ++l2) {
                int d = (l1 + l2 - 2) * (l1 + l2 - 3) / 2 + l2 - 1;
                interp2[(size_t)p * ndF + d] = std::pow(1 - eta, l1 - 2) * Ix[l1 - 2] * Ie[l2 - 1];
            }
        }
        std::vector<double> Je1(M + 1);
        jac_run(1, 1, eta, M - 2, Je1.data());
        for (int l = 2; l <= M; ++l) {
            add0[(size_t)p * ndE + l - 2] = std::pow(1 - y, l - 2) * Ix[l - 2];
            add1[(size_t)p * ndE + l - 2] = Je1[l - 2];
        }
    }
}

// physical coordinates of the 3-D quadrature points of element e
void element_qpoints(const Space& S, int e, std::vector<double>& out) {
    const double* X = S.mesh->xyz.data();
    const double* p0 = &X[3 * S.ele_node[4 * e]];
    const double* p1 = &X[3 * S.ele_node[4 * e + 1]];
    const double* p2 = &X[3 * S.ele_node[4 * e + 2]];
    const double* p3 = &X[3 * S.ele_node[4 * e + 3]];
    const int nq = (int)S.quad.w3.size();
    out.resize((size_t)nq * 3);
    for (int q = 0; q < nq; ++q) {
        const auto& r = S.quad.x3[q];
        for (int j = 0; j < 3; ++j)
            out[3 * q + j] = p0[j] + r[0] * (p1[j] - p0[j]) + r[1] * (p2[j] - p0[j]) + r[2] * (p3[j] - p0[j]);
    }
}

void boundary_points(const Space& S, int dim, std::vector<double>& out) {
    const double* X = S.mesh->xyz.data();
    const Quadrature& Q = S.quad;
    out.clear();
    if (dim == 0) {
        out.assign(X, X + 3 * S.n_geo[0]);
    } else if (dim == 1) {
        for (int g = 0; g < S.n_geo[1]; ++g) {
            const double* ps = &X[3 * S.edge_node[2 * g]];
            const double* pe = &X[3 * S.edge_node[2 * g + 1]];
            for (size_t p = 0; p < Q.x1.size(); ++p)
                for (int j = 0; j < 3; ++j) out.push_back(ps[j] * (1 - Q.x1[p]) + pe[j] * Q.x1[p]);
        }
    } else {
        for (int f = 0; f < S.n_geo[2]; ++f)
            for (size_t p = 0; p < Q.w2.size(); ++p)
                for (int j = 0; j < 3; ++j) {
                    double s = 0;
                    for (int k = 0; k < 3; ++k) s += X[3 * S.face_node[3 * f + k] + j] * Q.b2[p][(k + 2) % 3];
                    out.push_back(s);
                }
    }
}

// src/Discretize.cpp:1397-1418, value_f[e][q]
void calc_rhs(const Space& S, const double* f_qp, double* rhs) {
    const int nq = (int)S.quad.w3.size(), nl = S.n_loc;
    std::vector<double> phi((size_t)nq * nl);
    for (int q = 0; q < nq; ++q) S.lb.basis_values(S.quad.x3[q].data(), &phi[(size_t)q * nl]);
    std::fill(rhs, rhs + S.n_dof, 0.0);
    for (int e = 0; e < S.n_ele; ++e) {
        const double* fe = f_qp + (size_t)e * nq;
        for (int i = 0; i < nl; ++i) {
            double c = 0;
            for (int q = 0; q < nq; ++q) c += S.quad.w3[q] * fe[q] * phi[(size_t)q * nl + i];
            c *= S.volume[e];
            size_t b = (size_t)e * nl + i;
            for (int j = 0; j < S.t_n[b]; ++j) rhs[S.t_ind[b * S.max_dep + j]] += c * S.t_val[b * S.max_dep + j];
        }
    }
}

// build_mass_V_matrix (src/Discretize.cpp:668-756): entries |T| sum_q W_q phi_a phi_c V_e(q)
// of every element pair, scattered through T_e; rows diagonal first, then ascending
void assemble_potential(const Space& S, const double* v_qp, Csr& out) {
    const int nq = (int)S.quad.w3.size(), nl = S.n_loc;
    std::vector<double> phi((size_t)nq * nl);
    for (int q = 0; q < nq; ++q) S.lb.basis_values(S.quad.x3[q].data(), &phi[(size_t)q * nl]);
    std::vector<std::map<int, double>> rows(S.n_dof);
    for (int r = 0; r < S.n_dof; ++r) rows[r][r] = 0.0;
    for (int e = 0; e < S.n_ele; ++e) {
        const double* ve = v_qp + (size_t)e * nq;
        for (int a = 0; a < nl; ++a)
            for (int c = 0; c < nl; ++c) {
                double cnt = 0;
                for (int q = 0; q < nq; ++q) cnt += S.quad.w3[q] * phi[(size_t)q * nl + a] * phi[(size_t)q * nl + c] * ve[q];
                cnt *= S.volume[e];
                const size_t ba = (size_t)e * nl + a, bc = (size_t)e * nl + c;
                for (int u = 0; u < S.t_n[ba]; ++u)
                    for (int w = 0; w < S.t_n[bc]; ++w)
                        rows[S.t_ind[ba * S.max_dep + u]][S.t_ind[bc * S.max_dep + w]] +=
                            cnt * S.t_val[ba * S.max_dep + u] * S.t_val[bc * S.max_dep + w];
            }
    }
    out.n = S.n_dof;
    out.rowptr.assign(S.n_dof + 1, 0);
    out.col.clear();
    out.val.clear();
    for (int r = 0; r < S.n_dof; ++r) {
        out.col.push_back(r);
        out.val.push_back(rows[r][r]);
        for (auto& kv : rows[r])
            if (kv.first != r) { out.col.push_back(kv.first); out.val.push_back(kv.second); }
        out.rowptr[r + 1] = (int64_t)out.col.size();
    }
}

static double el(const Csr& A, int r, int c) {
    int64_t p = A.find(r, c);
    return p < 0 ? 0.0 : A.val[p];
}
static void set0(Csr& A, int r, int c) {
    int64_t p = A.find(r, c);
    if (p >= 0) A.val[p] = 0.0;
}

// src/Discretize.cpp:1466-1499 and :1533-1545
void impose_zero_bc(const Space& S, Csr* A, double* rhs, int flag) {
    for (int d = 0; d <= 2; ++d)
        for (int g = 0; g < S.n_geo[d]; ++g) {
            if (S.flag_bm[d][g] != flag) continue;
            int r0 = S.geo_first_dof(d, g);
            for (int i = 0; i < S.n_dof_geo[d]; ++i) {
                int row = r0 + i;
                if (rhs) rhs[row] = 0;
                if (!A) continue;
                for (int64_t p = A->rowptr[row]; p < A->rowptr[row + 1]; ++p) {
                    int c = A->col[p];
                    if (c != row) { A->val[p] = 0.0; set0(*A, c, row); }
                }
            }
        }
}

// src/Discretize.cpp:1683-1776; vb[dim] holds values at vertices / 1-D / 2-D
// boundary quadrature points in the layout of boundary_points().
void impose_dirichlet(const Space& S, const FaceBases& FB, Csr& A, double* rhs, const double* vb0,
                      const double* vb1, const double* vb2, bool modify, int flag) {
    const Quadrature& Q = S.quad;
    const int M = S.M;
    auto diag = [&](int r) { return A.val[A.rowptr[r]]; };
    for (int d = 0; d <= 2; ++d)
        for (int g = 0; g < S.n_geo[d]; ++g) {
            if (flag == -1 && S.flag_bm[d][g] == 0) continue;
            if (flag != -1 && S.flag_bm[d][g] != flag) continue;
            int r0 = S.geo_first_dof(d, g);
            std::vector<double> val(S.n_dof_geo[d], 0.0);
            if (d == 0) val[0] = vb0[g];
            if (d == 1) {
                int ls = S.geo_first_dof(0, S.edge_node[2 * g]), le = S.geo_first_dof(0, S.edge_node[2 * g + 1]);
                double cs = rhs[ls] / diag(ls), ce = rhs[le] / diag(le);
                for (int l = 2; l <= M; ++l) {
                    double c = 0;
                    for (int p = 0; p < FB.nq1; ++p)
                        c += Q.w1[p] * (vb1[(size_t)g * FB.nq1 + p] - cs * (1 - Q.x1[p]) - ce * Q.x1[p]) *
                             FB.interp1[(size_t)p * FB.ndE + l - 2];
                    val[l - 2] = c * -l * (2 * l - 1) / (2 * (l - 1));
                }
            }
            if (d == 2) {
                double vv[3];
                for (int k = 0; k < 3; ++k) {
                    int pv = S.geo_first_dof(0, S.face_node[3 * g + k]);
                    vv[k] = rhs[pv] / diag(pv);
                }
                std::vector<double> ve(3 * FB.ndE);
                for (int k = 0; k < 3; ++k) {
                    int pe = S.geo_first_dof(1, S.face_edge[3 * g + k]);
                    for (int l = 2; l <= M; ++l) {
                        double v = rhs[pe + l - 2] / diag(pe + l - 2);
                        if (!S.face_same[3 * g + k] && l % 2 == 1) v = -v;
                        ve[k * FB.ndE + l - 2] = v;
                    }
                }
                for (int l1 = 2; l1 <= M; ++l1)
                    for (int l2 = 1; l2 <= M - l1; ++l2) {
                        int di = (l1 + l2 - 2) * (l1 + l2 - 3) / 2 + l2 - 1;
                        double c = 0;
                        for (int p = 0; p < FB.nq2; ++p) {
                            const double xp = Q.b2[p][0], yp = Q.b2[p][1], rp = Q.b2[p][2];
                            double cp = vb2[(size_t)g * FB.nq2 + p];
                            for (int k = 0; k < 3; ++k) cp -= vv[k] * Q.b2[p][(k + 2) % 3];
                            for (int l = 2; l <= M; ++l)
                                cp += 2 * (xp * yp * ve[0 * FB.ndE + l - 2] * FB.add1[(size_t)p * FB.ndE + l - 2] +
                                           yp * rp * ve[1 * FB.ndE + l - 2] * FB.add1[(size_t)p * FB.ndE + l - 2] +
                                           xp * rp * ve[2 * FB.ndE + l - 2] * FB.add0[(size_t)p * FB.ndE + l - 2]);
                            c += Q.w2[p] * cp * FB.interp2[(size_t)p * FB.ndF + di];
                        }
                        val[di] = c * -l1 * (2 * l1 - 1) * (2 * l1 + 2 * l2 - 1) / (std::pow(2, l1) * (l1 - 1));
                    }
            }
            for (int i = 0; i < S.n_dof_geo[d]; ++i) {
                int row = r0 + i;
                for (int64_t p = A.rowptr[row]; p < A.rowptr[row + 1]; ++p) {
                    int c = A.col[p];
                    if (c == row) {
                        rhs[row] = diag(row) * val[i];
                    } else {
                        rhs[c] -= el(A, c, row) * val[i];
                        if (modify) { A.val[p] = 0.0; set0(A, c, row); }
                    }
                }
            }
        }
}

// src/Discretize.cpp:2011-2063; g at the 2-D boundary quadrature points
void impose_neumann(const Space& S, const FaceBases& FB, double* rhs, const double* g2, int flag) {
    const double* X = S.mesh->xyz.data();
    const Quadrature& Q = S.quad;
    for (int f = 0; f < S.n_geo[2]; ++f) {
        if (S.flag_bm[2][f] != flag) continue;
        const double* p0 = &X[3 * S.face_node[3 * f]];
        const double* p1 = &X[3 * S.face_node[3 * f + 1]];
        const double* p2 = &X[3 * S.face_node[3 * f + 2]];
        double area = 0.5 * std::sqrt(std::pow((p1[1] - p0[1]) * (p2[2] - p0[2]) - (p1[2] - p0[2]) * (p2[1] - p0[1]), 2) +
                                      std::pow((p1[0] - p0[0]) * (p2[2] - p0[2]) - (p1[2] - p0[2]) * (p2[0] - p0[0]), 2) +
                                      std::pow((p1[0] - p0[0]) * (p2[1] - p0[1]) - (p1[1] - p0[1]) * (p2[0] - p0[0]), 2));
        double cv[3] = {0, 0, 0};
        std::vector<double> ce(3 * FB.ndE, 0.0), cf(FB.ndF, 0.0);
        for (int p = 0; p < FB.nq2; ++p) {
            const auto& qb = Q.b2[p];
            double wgv = Q.w2[p] * g2[(size_t)f * FB.nq2 + p] * area;
            for (int k = 0; k < 3; ++k) cv[k] += wgv * qb[(k + 2) % 3];
            const double xp = qb[0], yp = qb[1], rp = qb[2];
            for (int i = 0; i < FB.ndE; ++i) {
                ce[0 * FB.ndE + i] += wgv * -2 * xp * yp * FB.add1[(size_t)p * FB.ndE + i];
                ce[1 * FB.ndE + i] += wgv * -2 * yp * rp * FB.add1[(size_t)p * FB.ndE + i];
                ce[2 * FB.ndE + i] += wgv * -2 * xp * rp * FB.add0[(size_t)p * FB.ndE + i];
            }
            for (int i = 0; i < FB.ndF; ++i) cf[i] += wgv * FB.face_val[(size_t)p * FB.ndF + i];
        }
        for (int k = 0; k < 3; ++k) rhs[S.geo_first_dof(0, S.face_node[3 * f + k])] += cv[k];
        for (int k = 0; k < 3; ++k) {
            if (!S.face_same[3 * f + k])
                for (int i = 1; i < FB.ndE; i += 2) ce[k * FB.ndE + i] = -ce[k * FB.ndE + i];
            int pe = S.geo_first_dof(1, S.face_edge[3 * f + k]);
            for (int i = 0; i < FB.ndE; ++i) rhs[pe + i] += ce[k * FB.ndE + i];
        }
        int pf = S.geo_first_dof(2, f);
        for (int i = 0; i < FB.ndF; ++i) rhs[pf + i] += cf[i];
    }
}

// src/CalcError.cpp:64-92 (u_qp exact values) and :126-189 (gu_qp exact gradients)
void calc_errors(const Space& S, const double* sol, const double* u_qp, const double* gu_qp, double* l2, double* h1) {
    const int nq = (int)S.quad.w3.size(), nl = S.n_loc;
    std::vector<double> phi((size_t)nq * nl), gphi((size_t)nq * nl * 3);
    for (int q = 0; q < nq; ++q) {
        S.lb.basis_values(S.quad.x3[q].data(), &phi[(size_t)q * nl]);
        S.lb.basis_gradients(S.quad.x3[q].data(), &gphi[(size_t)q * nl * 3]);
    }
    const double* X = S.mesh->xyz.data();
    double el2 = 0, eh1 = 0;
    std::vector<double> c(nl);
    for (int e = 0; e < S.n_ele; ++e) {
        S.gather(e, sol, c.data());
        double d[3][3];
        const double* p0 = &X[3 * S.ele_node[4 * e]];
        for (int k = 0; k < 3; ++k) {
            const double* pk = &X[3 * S.ele_node[4 * e + k + 1]];
            for (int j = 0; j < 3; ++j) d[j][k] = pk[j] - p0[j];
        }
        double V = d[0][0] * d[1][1] * d[2][2] + d[0][1] * d[1][2] * d[2][0] + d[0][2] * d[1][0] * d[2][1] -
                   d[0][0] * d[1][2] * d[2][1] - d[0][1] * d[1][0] * d[2][2] - d[0][2] * d[1][1] * d[2][0];
        double Ji[3][3];  // d xhat_j / d x_k
        Ji[0][0] = (d[1][1] * d[2][2] - d[1][2] * d[2][1]) / V;
        Ji[0][1] = (d[0][2] * d[2][1] - d[0][1] * d[2][2]) / V;
        Ji[0][2] = (d[0][1] * d[1][2] - d[0][2] * d[1][1]) / V;
        Ji[1][0] = (d[1][2] * d[2][0] - d[1][0] * d[2][2]) / V;
        Ji[1][1] = (d[0][0] * d[2][2] - d[0][2] * d[2][0]) / V;
        Ji[1][2] = (d[0][2] * d[1][0] - d[0][0] * d[1][2]) / V;
        Ji[2][0] = (d[1][0] * d[2][1] - d[1][1] * d[2][0]) / V;
        Ji[2][1] = (d[0][1] * d[2][0] - d[0][0] * d[2][1]) / V;
        Ji[2][2] = (d[0][0] * d[1][1] - d[0][1] * d[1][0]) / V;
        double s2 = 0, sg = 0;
        for (int q = 0; q < nq; ++q) {
            double v = 0, g[3] = {0, 0, 0};
            for (int i = 0; i < nl; ++i) {
                v += c[i] * phi[(size_t)q * nl + i];
                for (int k = 0; k < 3; ++k)
                    for (int t = 0; t < 3; ++t) g[k] += Ji[t][k] * c[i] * gphi[((size_t)q * nl + i) * 3 + t];
            }
            double du = v - u_qp[(size_t)e * nq + q];
            s2 += S.quad.w3[q] * du * du;
            double dg = 0;
            for (int k = 0; k < 3; ++k) dg += std::pow(g[k] - gu_qp[((size_t)e * nq + q) * 3 + k], 2);
            sg += S.quad.w3[q] * dg;
        }
        el2 += s2 * S.volume[e];
        eh1 += sg * S.volume[e];
    }
    *l2 = std::sqrt(el2);
    *h1 = std::sqrt(eh1);
}

// calc_val_qp_onElement (src/PointInfo.cpp:2013-2022) through calc_coef_onElement
// (:60-70): values of the FE function with coefficients sol at element e's points
static void values_on_element(const Space& S, const std::vector<double>& phi, int e, const double* sol,
                              std::vector<double>& c, double* out) {
    const int nq = (int)S.quad.w3.size(), nl = S.n_loc;
    S.gather(e, sol, c.data());
    for (int q = 0; q < nq; ++q) {
        double v = 0;
        for (int i = 0; i < nl; ++i) v += c[i] * phi[(size_t)q * nl + i];
        out[q] = v;
    }
}

static std::vector<double> basis_at_qpoints(const Space& S) {
    const int nq = (int)S.quad.w3.size(), nl = S.n_loc;
    std::vector<double> phi((size_t)nq * nl);
    for (int q = 0; q < nq; ++q) S.lb.basis_values(S.quad.x3[q].data(), &phi[(size_t)q * nl]);
    return phi;
}

// src/PointInfo.cpp:72-91: rho(x_q) = sum_j occ_j psi_j(x_q)^2 on every element;
// states j at states + j n_dof, out [E][nq]
void calc_density(const Space& S, const double* states, int k, const double* occ, double* out) {
    const int nq = (int)S.quad.w3.size();
    const std::vector<double> phi = basis_at_qpoints(S);
    std::vector<double> c(S.n_loc), psi(nq);
    for (int e = 0; e < S.n_ele; ++e) {
        double* d = out + (size_t)e * nq;
        for (int q = 0; q < nq; ++q) d[q] = 0;
        for (int j = 0; j < k; ++j) {
            values_on_element(S, phi, e, states + (size_t)j * S.n_dof, c, psi.data());
            for (int q = 0; q < nq; ++q) d[q] += occ[j] * std::pow(psi[q], 2);
        }
    }
}

// src/CalcError.cpp:703-735: || sum_j occ_j (u_j^2 - v_j^2) ||_L2
double calc_density_l2_difference(const Space& S, const double* u, const double* v, int k, const double* occ) {
    const int nq = (int)S.quad.w3.size();
    const std::vector<double> phi = basis_at_qpoints(S);
    std::vector<double> c(S.n_loc), pu(nq), pv(nq), dif(nq);
    double out = 0;
    for (int e = 0; e < S.n_ele; ++e) {
        for (int q = 0; q < nq; ++q) dif[q] = 0;
        for (int j = 0; j < k; ++j) {
            values_on_element(S, phi, e, u + (size_t)j * S.n_dof, c, pu.data());
            values_on_element(S, phi, e, v + (size_t)j * S.n_dof, c, pv.data());
            for (int q = 0; q < nq; ++q) dif[q] += occ[j] * (std::pow(pu[q], 2) - std::pow(pv[q], 2));
        }
        double count = 0;
        for (int q = 0; q < nq; ++q) count += S.quad.w3[q] * std::pow(dif[q], 2);
        out += count * S.volume[e];
    }
    return std::sqrt(out);
}

// calc_interpolation from point values (src/Interpolation.cpp:12-101): vertex values
// u_v [nv]; edge modes by projection of u minus the vertex line on J^{1,1}; face modes
// by projection of u minus the vertex plane and the edge modes' traces; interior
// modes element by element by projection of u minus every non-interior mode on the
// interior interpolation basis (src/BuildSpace.cpp:150-170).  u_e / u_f at the
// points of boundary_points(1 / 2) of EVERY edge and face, u_qp [E][nq3].
void calc_interpolation(const Space& S, const FaceBases& FB, const double* u_v, const double* u_e,
                        const double* u_f, const double* u_qp, double* out) {
    const Quadrature& Q = S.quad;
    const int M = S.M;
    std::fill(out, out + S.n_dof, 0.0);
    for (int v = 0; v < S.n_geo[0]; ++v) out[S.geo_first_dof(0, v)] = u_v[v];
    // edges (:18-30)
    for (int g = 0; g < S.n_geo[1]; ++g) {
        const double cs = out[S.geo_first_dof(0, S.edge_node[2 * g])];
        const double ce = out[S.geo_first_dof(0, S.edge_node[2 * g + 1])];
        const int r0 = S.geo_first_dof(1, g);
        for (int l = 2; l <= M; ++l) {
            double c = 0;
            for (int p = 0; p < FB.nq1; ++p)
                c += Q.w1[p] * (u_e[(size_t)g * FB.nq1 + p] - cs * (1 - Q.x1[p]) - ce * Q.x1[p]) *
                     FB.interp1[(size_t)p * FB.ndE + l - 2];
            out[r0 + l - 2] = c * -l * (2 * l - 1) / (2 * (l - 1));
        }
    }
    // faces (:33-68): the vertex and edge coefficients as set above
    for (int f = 0; f < S.n_geo[2]; ++f) {
        double vv[3];
        for (int k = 0; k < 3; ++k) vv[k] = out[S.geo_first_dof(0, S.face_node[3 * f + k])];
        std::vector<double> ve(3 * FB.ndE);
        for (int k = 0; k < 3; ++k) {
            const int pe = S.geo_first_dof(1, S.face_edge[3 * f + k]);
            for (int l = 2; l <= M; ++l) {
                double v = out[pe + l - 2];
                if (!S.face_same[3 * f + k] && l % 2 == 1) v = -v;
                ve[k * FB.ndE + l - 2] = v;
            }
        }
        const int r0 = S.geo_first_dof(2, f);
        for (int l1 = 2; l1 <= M; ++l1)
            for (int l2 = 1; l2 <= M - l1; ++l2) {
                const int di = (l1 + l2 - 2) * (l1 + l2 - 3) / 2 + l2 - 1;
                double c = 0;
                for (int p = 0; p < FB.nq2; ++p) {
                    const double xp = Q.b2[p][0], yp = Q.b2[p][1], rp = Q.b2[p][2];
                    double cp = u_f[(size_t)f * FB.nq2 + p];
                    for (int k = 0; k < 3; ++k) cp -= vv[k] * Q.b2[p][(k + 2) % 3];
                    for (int l = 2; l <= M; ++l)
                        cp += 2 * (xp * yp * ve[0 * FB.ndE + l - 2] * FB.add1[(size_t)p * FB.ndE + l - 2] +
                                   yp * rp * ve[1 * FB.ndE + l - 2] * FB.add1[(size_t)p * FB.ndE + l - 2] +
                                   xp * rp * ve[2 * FB.ndE + l - 2] * FB.add0[(size_t)p * FB.ndE + l - 2]);
                    c += Q.w2[p] * cp * FB.interp2[(size_t)p * FB.ndF + di];
                }
                out[r0 + di] = c * -l1 * (2 * l1 - 1) * (2 * l1 + 2 * l2 - 1) / (std::pow(2, l1) * (l1 - 1));
            }
    }
    if (S.n_dof_geo[3] == 0) return;
    // interior (:71-100): interpolation basis at the 3-D points, [nq3][n_interior]
    const int nq = (int)Q.w3.size(), nl = S.n_loc, ni = S.n_dof_geo[3];
    std::vector<double> bi((size_t)nq * ni, 0.0), phi((size_t)nq * nl);
    for (int p = 0; p < nq; ++p) {
        const double x = Q.x3[p][0], y = Q.x3[p][1], z = Q.x3[p][2];
        const double xi = 2 * x / (1 - y - z) - 1, eta = 2 * y / (1 - z) - 1, zeta = 2 * z - 1;
        std::vector<double> Jx(M + 1), Je(M + 1), Jz(M + 1);
        jac_run(1, 1, xi, M - 2, Jx.data());
        for (int l1 = 2; l1 <= M; ++l1) {
            jac_run(2 * l1 - 1, 1, eta, M - l1, Je.data());
            for (int l2 = 1; l2 <= M - l1; ++l2) {
                jac_run(2 * l1 + 2 * l2 - 1, 1, zeta, M - l1 - l2, Jz.data());
                for (int l3 = 1; l3 <= M - l1 - l2; ++l3) {
                    const int d = MultiIndexTable::number(l1 - 2, l2 - 1, l3 - 1);
                    bi[(size_t)p * ni + d] = Jx[l1 - 2] * Je[l2 - 1] * std::pow(1 - eta, l1 - 2) * Jz[l3 - 1] *
                                             std::pow(1 - zeta, l1 + l2 - 3);
                }
            }
        }
        S.lb.basis_values(Q.x3[p].data(), &phi[(size_t)p * nl]);
    }
    std::vector<char> interior(nl);
    for (int j = 0; j < nl; ++j) {
        const auto& a = S.lb.mi.num2idx[j];
        interior[j] = a[0] >= 2 && a[1] >= 1 && a[2] >= 1;
    }
    std::vector<double> loc(nl), rem(nq);
    for (int e = 0; e < S.n_ele; ++e) {
        // local coefficients of the vertex, edge and face modes (global -> local)
        for (int j = 0; j < nl; ++j) {
            loc[j] = 0.0;
            if (interior[j]) continue;
            const size_t b = (size_t)e * nl + j;
            for (int t = 0; t < S.t_n[b]; ++t) loc[j] += out[S.t_ind[b * S.max_dep + t]] * S.t_val[b * S.max_dep + t];
        }
        for (int p = 0; p < nq; ++p) {
            double r = u_qp[(size_t)e * nq + p];
            for (int j = 0; j < nl; ++j)
                if (!interior[j]) r -= loc[j] * phi[(size_t)p * nl + j];
            rem[p] = r;
        }
        const int r0 = S.geo_first_dof(3, e);
        for (int l1 = 2; l1 <= M; ++l1)
            for (int l2 = 1; l2 <= M - l1; ++l2)
                for (int l3 = 1; l3 <= M - l1 - l2; ++l3) {
                    const int d = MultiIndexTable::number(l1 - 2, l2 - 1, l3 - 1);
                    double c = 0;
                    for (int p = 0; p < nq; ++p) c += Q.w3[p] * rem[p] * bi[(size_t)p * ni + d];
                    out[r0 + d] = c * -l1 * (2 * l1 - 1) * (2 * l1 + 2 * l2 - 1) * (2 * l1 + 2 * l2 + 2 * l3 - 1) /
                                  (std::pow(2, 2 * l1 + l2 - 5) * (l1 - 1) * 6);
                }
    }
}

}  // namespace tsem_oracle
