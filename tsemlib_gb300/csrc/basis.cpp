// Host-side definition tables of the TSEM discretisation (see basis.hpp).
#include "basis.hpp"
#include "jacobi.cuh"

#include <algorithm>
#include <cmath>
#include <stdexcept>

namespace tsem {

int mi_count(int deg) { return deg < 0 ? 0 : (deg + 1) * (deg + 2) * (deg + 3) / 6; }

std::array<int, 3> mi_index(int number) {
    int deg = 0;
    while (mi_count(deg) <= number) ++deg;
    int r = number - mi_count(deg - 1);      // position inside the degree block
    int s = 0;                               // s = a1 + a2
    while ((s + 1) * (s + 2) / 2 <= r) ++s;
    int a2 = r - s * (s + 1) / 2;
    return {deg - s, s - a2, a2};
}

int face_dof_index(int l1, int l2) { return (l1 + l2 - 2) * (l1 + l2 - 3) / 2 + l2 - 1; }

void LocalTransform::build(int order) {
    M = order;
    n_loc = mi_count(M);
    std::vector<std::vector<std::pair<int, double>>> t(n_loc);
    auto N = [](int a, int b, int c) { return mi_number(a, b, c); };
    // vertex modes: the J of degree <= 1 recombine into the barycentric coordinates
    t[0] = {{0, 0.125}, {1, 0.125}, {2, 0.25}, {3, 0.5}};
    t[1] = {{0, -0.5}, {1, 0.5}};
    t[2] = {{0, -0.25}, {1, -0.25}, {2, 0.5}};
    t[3] = {{0, -0.125}, {1, -0.125}, {2, -0.25}, {3, 0.5}};
    for (int l = 2; l <= M; ++l) {
        const double r = (double)(l - 1) / l;
        t[N(l, 0, 0)] = {{N(l, 0, 0), 2.0}};
        int a = N(0, l, 0), b = N(1, l - 1, 0);
        t[a] = {{a, 1.0}, {b, 1.0}};
        t[b] = {{a, r}, {b, -r}};
        int c = N(0, 0, l), d = N(1, 0, l - 1), e = N(0, 1, l - 1);
        t[c] = {{c, 0.5}, {d, 0.5}, {e, 1.0}};
        t[d] = {{c, r}, {d, -r}};
        t[e] = {{c, 0.5 * r}, {d, 0.5 * r}, {e, -r}};
    }
    for (int l1 = 2; l1 <= M; ++l1)
        for (int l2 = 1; l2 <= M - l1; ++l2) {
            const double r = (double)(l1 - 1) / l1;
            int a = N(0, l1, l2), b = N(1, l1 - 1, l2);
            t[a] = {{a, 1.0}, {b, 1.0}};
            t[b] = {{a, r}, {b, -r}};
            t[N(l1, 0, l2)] = {{N(l1, 0, l2), 2.0}};
            t[N(l1, l2, 0)] = {{N(l1, l2, 0), 2.0}};
        }
    for (int l1 = 2; l1 <= M; ++l1)
        for (int l2 = 1; l2 <= M - l1; ++l2)
            for (int l3 = 1; l3 <= M - l1 - l2; ++l3) t[N(l1, l2, l3)] = {{N(l1, l2, l3), 1.0}};
    start.assign(n_loc + 1, 0);
    target.clear();
    weight.clear();
    for (int i = 0; i < n_loc; ++i) {
        for (auto& p : t[i]) { target.push_back(p.first); weight.push_back(p.second); }
        start[i + 1] = (int)target.size();
    }
}

void StructPatterns::build(const LocalTransform& lt) {
    const int M = lt.M;
    n_loc = lt.n_loc;
    const int n = n_loc;
    auto expand = [&](const std::vector<uint8_t>& jac, int nj, std::vector<uint8_t>& out) {
        out.assign((size_t)n * n, 0);
        for (int r = 0; r < nj; ++r)
            for (int c = 0; c < nj; ++c) {
                if (!jac[(size_t)r * nj + c]) continue;
                for (int a = lt.start[r]; a < lt.start[r + 1]; ++a)
                    for (int b = lt.start[c]; b < lt.start[c + 1]; ++b) out[(size_t)lt.target[a] * n + lt.target[b]] = 1;
            }
        for (int i = 0; i < n; ++i) out[(size_t)i * n + i] = 1;
    };
    // mass in the Jacobi basis
    {
        std::vector<uint8_t> jac((size_t)n * n, 0);
        for (int r = 0; r < n; ++r) {
            auto a = mi_index(r);
            jac[(size_t)r * n + r] = 1;
            for (int d1 = -2; d1 <= 2; ++d1)
                for (int d2 = -3; d2 <= 3; ++d2)
                    for (int d3 = -4; d3 <= 4; ++d3) {
                        int c0 = a[0] + d1, c1 = a[1] + d2 - d1, c2 = a[2] + d3 - d2;
                        if (c0 < 0 || c1 < 0 || c2 < 0 || c0 + c1 + c2 > M) continue;
                        jac[(size_t)r * n + mi_number(c0, c1, c2)] = 1;
                    }
        }
        expand(jac, n, mass);
    }
    // stiffness: six Jacobi-basis patterns of size C(M+2,3), then variations
    const int ns = mi_count(M - 1);
    std::vector<uint8_t> jac[6];
    for (int k = 0; k < 6; ++k) jac[k].assign((size_t)ns * ns, 0);
    for (int r = 0; r < ns; ++r) {
        auto a = mi_index(r);
        for (int k = 0; k < 6; ++k) jac[k][(size_t)r * ns + r] = 1;
        for (int d1 = -2; d1 <= 2; ++d1)
            for (int d2 = -2; d2 <= 2; ++d2)
                for (int d3 = -2; d3 <= 2; ++d3) {
                    int c0 = a[0] + d1, c1 = a[1] + d2 - d1, c2 = a[2] + d3 - d2;
                    if (c0 < 0 || c1 < 0 || c2 < 0 || c0 + c1 + c2 >= M) continue;
                    size_t at = (size_t)r * ns + mi_number(c0, c1, c2);
                    bool n1 = std::abs(d1) <= 1, n2 = std::abs(d2) <= 1;
                    if (d1 == 0 && n2) jac[0][at] = 1;
                    if (n1 && n2) { jac[1][at] = 1; jac[3][at] = 1; }
                    if (n1) { jac[2][at] = 1; jac[5][at] = 1; }
                    jac[4][at] = 1;
                }
    }
    typedef std::array<int, 3> V3;
    const std::vector<std::vector<V3>> var = {
        {{1, 0, 0}},
        {{0, 1, 0}, {1, 0, 0}},
        {{0, 0, 1}, {1, -1, 1}, {0, 1, 0}, {1, 0, 0}},
        {{0, 1, 0}, {1, 0, 0}},
        {{0, 0, 1}, {0, 1, 0}},
        {{0, 0, 1}, {1, -1, 1}, {0, 1, 0}, {1, 0, 0}}};
    stiff_union.assign((size_t)n * n, 0);
    for (int k = 0; k < 6; ++k) {
        std::vector<uint8_t> shifted((size_t)n * n, 0);
        for (int r = 0; r < ns; ++r)
            for (int c = 0; c < ns; ++c) {
                if (!jac[k][(size_t)r * ns + c]) continue;
                auto ar = mi_index(r), ac = mi_index(c);
                for (auto& vr : var[k])
                    for (auto& vc : var[k]) {
                        int r0 = ar[0] + vr[0], r1 = ar[1] + vr[1], r2 = ar[2] + vr[2];
                        int c0 = ac[0] + vc[0], c1 = ac[1] + vc[1], c2 = ac[2] + vc[2];
                        if (r0 < 0 || r1 < 0 || r2 < 0 || c0 < 0 || c1 < 0 || c2 < 0) continue;
                        shifted[(size_t)mi_number(r0, r1, r2) * n + mi_number(c0, c1, c2)] = 1;
                    }
            }
        expand(shifted, n, stiff[k]);
        for (size_t i = 0; i < stiff_union.size(); ++i) stiff_union[i] |= stiff[k][i];
    }
}

static void gauss_legendre01(int q, std::vector<double>& x, std::vector<double>& w) {
    x.assign(q, 0.0);
    w.assign(q, 0.0);
    for (int i = 0; i < q; ++i) {
        double z = std::cos(M_PI * (i + 0.75) / (q + 0.5)), dp = 1;
        for (int it = 0; it < 100; ++it) {
            double p0 = 1, p1 = 0;
            for (int j = 1; j <= q; ++j) { double p2 = p1; p1 = p0; p0 = ((2.0 * j - 1) * z * p1 - (j - 1.0) * p2) / j; }
            dp = q * (z * p0 - p1) / (z * z - 1);
            double dz = p0 / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-16) {
                p0 = 1; p1 = 0;
                for (int j = 1; j <= q; ++j) { double p2 = p1; p1 = p0; p0 = ((2.0 * j - 1) * z * p1 - (j - 1.0) * p2) / j; }
                dp = q * (z * p0 - p1) / (z * z - 1);
                break;
            }
        }
        x[i] = 0.5 * (1 - z);
        w[i] = 1.0 / ((1 - z * z) * dp * dp);
    }
}

void Quadrature::build(int qq) {
    q = qq;
    gauss_legendre01(q, x1, w1);
    b2.clear(); w2.clear(); x3.clear(); w3.clear();
    for (int i = 0; i < q; ++i)
        for (int j = 0; j < q; ++j) {
            double a = x1[i] * (1 - x1[j]), b = x1[j];
            b2.insert(b2.end(), {a, b, 1 - a - b});
            w2.push_back(2 * (1 - x1[j]) * w1[i] * w1[j]);
        }
    for (int i = 0; i < q; ++i)
        for (int j = 0; j < q; ++j)
            for (int k = 0; k < q; ++k) {
                x3.insert(x3.end(), {x1[i] * (1 - x1[j]) * (1 - x1[k]), x1[j] * (1 - x1[k]), x1[k]});
                w3.push_back(6 * (1 - x1[j]) * (1 - x1[k]) * (1 - x1[k]) * w1[i] * w1[j] * w1[k]);
            }
}

// ----------------------------------------------------------- face table
// Trace functions on a triangle with barycentrics (m0, m1, m2) of its vertices,
// written with x = m1, y = m2, r = m0 as in src/Discretize.cpp:1811-1844:
// vertices m_k; edge opposite vertex 0 (v1->v2): -2xy P_{l-2}^{1,1}(2y-1);
// opposite 1 (v0->v2): -2yr P_{l-2}^{1,1}(2y-1); opposite 2 (v0->v1):
// -2xr (1-y)^{l-2} P_{l-2}^{1,1}(2x/(1-y)-1); face modes
// 2 (1-y)^{l1} J_{l1}^{-1,-1}(xi) J_{l2}^{2l1-1,-1}(2y-1).
static void trace_functions(int M, const double m[3], std::vector<double>& out) {
    const double r = m[0], x = m[1], y = m[2];
    const int ndE = M - 1;
    const int nf = (M - 2) * (M - 3) / 2 + M - 2;
    out.assign(3 + 3 * ndE + nf, 0.0);
    out[0] = r; out[1] = x; out[2] = y;
    const double xi = 2 * x / (1 - y) - 1, eta = 2 * y - 1;
    std::vector<double> Pe(M + 1), Px(M + 1), Jx(M + 1), Je(M + 1);
    jacobi_classic<double>(1, 1, eta, M - 2, Pe.data());
    jacobi_classic<double>(1, 1, xi, M - 2, Px.data());
    for (int l = 2; l <= M; ++l) {
        out[3 + 0 * ndE + l - 2] = -2 * x * y * Pe[l - 2];
        out[3 + 1 * ndE + l - 2] = -2 * y * r * Pe[l - 2];
        out[3 + 2 * ndE + l - 2] = -2 * x * r * std::pow(1 - y, l - 2) * Px[l - 2];
    }
    jacobi_general<double, 64>(-1, -1, xi, M, Jx.data());
    for (int l1 = 2; l1 <= M; ++l1) {
        jacobi_general<double, 64>(2 * l1 - 1, -1, eta, M - l1, Je.data());
        for (int l2 = 1; l2 <= M - l1; ++l2)
            out[3 + 3 * ndE + face_dof_index(l1, l2)] = 2 * std::pow(1 - y, l1) * Jx[l1] * Je[l2];
    }
}

// least squares by Householder QR: A [m x n] (row-major), several right-hand sides
static void lstsq(int m, int n, std::vector<double> A, std::vector<double>& B, int nrhs) {
    for (int k = 0; k < n; ++k) {
        double s = 0;
        for (int i = k; i < m; ++i) s += A[(size_t)i * n + k] * A[(size_t)i * n + k];
        double nrm = std::sqrt(s);
        if (nrm == 0) throw std::runtime_error("face table: singular trace system");
        double alpha = A[(size_t)k * n + k] > 0 ? -nrm : nrm;
        std::vector<double> v(m - k);
        for (int i = k; i < m; ++i) v[i - k] = A[(size_t)i * n + k];
        v[0] -= alpha;
        double vn = 0;
        for (double t : v) vn += t * t;
        auto reflect = [&](double* col, int stride) {
            double d = 0;
            for (int i = k; i < m; ++i) d += v[i - k] * col[(size_t)i * stride];
            d = 2 * d / vn;
            for (int i = k; i < m; ++i) col[(size_t)i * stride] -= d * v[i - k];
        };
        for (int j = k; j < n; ++j) reflect(&A[j], n);
        for (int j = 0; j < nrhs; ++j) reflect(&B[j], nrhs);
    }
    for (int j = 0; j < nrhs; ++j)
        for (int k = n - 1; k >= 0; --k) {
            double s = B[(size_t)k * nrhs + j];
            for (int c = k + 1; c < n; ++c) s -= A[(size_t)k * n + c] * B[(size_t)c * nrhs + j];
            B[(size_t)k * nrhs + j] = s / A[(size_t)k * n + k];
        }
}

void FaceTable::derive(int order) {
    M = order;
    const int ndE = M - 1;
    nf = (M - 2) * (M - 3) / 2 + M - 2;
    edge.assign(6, std::vector<std::vector<Edge>>(nf));
    face.assign(6, std::vector<std::vector<Face>>(nf));
    if (nf <= 0) return;
    const int nfun = 3 + 3 * ndE + nf;
    // sample points: a collapsed Gauss rule strictly inside the triangle
    Quadrature Q;
    Q.build(M + 3);
    const int npt = (int)Q.w2.size();
    // var -> pi with local vertex n = global vertex pi[n]; var is the inverse
    // projection type the reference uses for the global -> local transform
    const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {2, 0, 1}, {1, 2, 0}, {2, 1, 0}};
    for (int var = 0; var < 6; ++var) {
        std::vector<double> A((size_t)npt * nfun), B((size_t)npt * (3 * ndE + nf));
        std::vector<double> tf;
        for (int p = 0; p < npt; ++p) {
            double g[3] = {Q.b2[3 * p + 2], Q.b2[3 * p + 0], Q.b2[3 * p + 1]};   // global (m0, m1, m2)
            double l[3] = {g[perm[var][0]], g[perm[var][1]], g[perm[var][2]]};
            trace_functions(M, l, tf);
            for (int j = 0; j < nfun; ++j) A[(size_t)p * nfun + j] = tf[j];
            trace_functions(M, g, tf);
            for (int j = 0; j < 3 * ndE + nf; ++j) B[(size_t)p * (3 * ndE + nf) + j] = tf[3 + j];
        }
        lstsq(npt, nfun, A, B, 3 * ndE + nf);
        const int nr = 3 * ndE + nf;
        for (int d = 0; d < nf; ++d) {
            const int row = 3 + 3 * ndE + d;   // local face-mode coefficient
            for (int k = 0; k < 3; ++k)
                for (int i = 0; i < ndE; ++i) {
                    double v = B[(size_t)row * nr + k * ndE + i];
                    if (std::fabs(v) > 1e-11) edge[var][d].push_back({k, i, v});
                }
            for (int i = 0; i < nf; ++i) {
                double v = B[(size_t)row * nr + 3 * ndE + i];
                if (std::fabs(v) > 1e-11) face[var][d].push_back({i, v});
            }
        }
    }
}

}  // namespace tsem
