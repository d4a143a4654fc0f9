// TEST INFRASTRUCTURE ONLY -- CPU oracle (see oracle.hpp).
// Index algebra, Jacobi coefficient algebra, quadrature and the local basis.
#include "oracle.hpp"
#include <cmath>
#include <cstdio>
#include <algorithm>

namespace tsem_oracle {

// include/Correspondence.h:64-94: n(i, j) = #multi-indices with i+1 components and sum <= j.
static int count_components(int comps, int upto) {
    // number of beta in N^{comps} with |beta| <= upto  = C(upto + comps, comps)
    if (upto < 0) return 0;
    long v = 1;
    for (int i = 1; i <= comps; ++i) v = v * (upto + i) / i;
    return (int)v;
}

void MultiIndexTable::init(int order) {
    M = order;
    n = count_upto(M);
    num2idx.clear();
    // enumerate by degree, then (a1+a2) ascending, then a2 ascending
    for (int deg = 0; deg <= M; ++deg)
        for (int s = 0; s <= deg; ++s)
            for (int a2 = 0; a2 <= s; ++a2)
                num2idx.push_back({deg - s, s - a2, a2});
}

// include/Correspondence.h:97-109
int MultiIndexTable::number(int a0, int a1, int a2) {
    int num = 0;
    int tail[3] = {a0 + a1 + a2, a1 + a2, a2};
    for (int i = 0; i < 3; ++i) {
        if (tail[i] == 0) break;
        num += count_components(3 - i, tail[i] - 1);
    }
    return num;
}

int binom_ref(int n, int m) {
    int val = 1;
    if (n > 0 && n >= m) {
        if (n - m < m) m = n - m;
        for (int i = 0; i < m; ++i) { val *= (n - i); val /= (i + 1); }
    }
    return val;
}

// ---------------------------------------------------- src/Miscellaneous.cpp:175-348
double coef_a(int al, int be, int ind, int k) {
    if (k < 0) return 0.0;
    const bool mm = (al == -1 && be == -1);
    double r = 0.0;
    if (ind == 1) {
        if (mm) {
            if (k == 0) return 1.0;
            if (k == 1) return 4.0;
            if (k == 2) return 0.5;
            return ((double)(2 * (k + 1) * (k + al + be + 1))) / ((2 * k + al + be + 1) * (2 * k + al + be + 2));
        }
        if (k == 0 && al + be != -2) return 2.0 / (al + be + 2);
        return ((double)(2 * (k + 1) * (k + al + be + 1))) / ((2 * k + al + be + 1) * (2 * k + al + be + 2));
    }
    if (ind == 2) {
        if (k <= 2 && mm) return 0.0;
        if (k == 0 && al + be != -2) return ((double)(be - al)) / (al + be + 2);
        return (std::pow(be, 2) - std::pow(al, 2)) / ((2 * k + al + be) * (2 * k + al + be + 2));
    }
    if (ind == 3) {
        if (mm) {
            if (k == 0) return 0.0;
            if (k == 1) return 1.0;
            if (k == 2) return 0.0;
            return ((double)(2 * (k + al) * (k + be))) / ((2 * k + al + be) * (2 * k + al + be + 1));
        }
        if (k == 0 && al + be != -2) return 0.0;
        return ((double)(2 * (k + al) * (k + be))) / ((2 * k + al + be) * (2 * k + al + be + 1));
    }
    return r;
}

double coef_b(int al, int be, int ind, int k) {
    if (k < 0) return 0.0;
    if (ind == 1) {
        if (k == 0 && al >= -1 && be >= -1) return 1.0;
        if (k == 1 && al == -1 && be == -1) return 2.0;
        return ((double)(k + al + be + 1)) / (2 * k + al + be + 1);
    }
    if (k == 0 && al >= -1 && be >= -1) return 0.0;
    if (k == 1 && al == -1 && be == -1) return -1.0;
    return ((double)-(k + be)) / (2 * k + al + be + 1);
}

double coef_c(int al, int be, int ind, int k) {
    switch (ind) {
    case 1: return coef_b(al, be, 1, k) * coef_b(al + 1, be, 1, k);
    case 2: return coef_b(al, be, 1, k) * coef_b(al + 1, be, 2, k) + coef_b(al, be, 2, k) * coef_b(al + 1, be, 1, k - 1);
    default: return coef_b(al, be, 2, k) * coef_b(al + 1, be, 2, k - 1);
    }
}

double coef_d(int al, int be, int k) {
    if (k <= 0) return 0.0;
    if (k == 1 && al == -1 && be == -1) return 1.0;
    return ((double)(k + al + be + 1)) / 2;
}

double coef_e(int al, int be, int ind, int k) {
    if (k < 0) return 0.0;
    const bool mm = (al == -1 && be == -1);
    if (ind == 1) {
        if (mm && k == 0) return 0.5;
        if (mm && k == 1) return 0.0;
        return ((double)(k + al + 1)) / (2 * k + al + be + 2);
    }
    if (mm && k == 0) return -0.5;
    if (mm && k == 1) return -1.0;
    return ((double)-(k + 1)) / (2 * k + al + be + 2);
}

double coef_g(int al, int be, int ind, int k) {
    switch (ind) {
    case 1: return coef_e(al + 1, be, 2, k) * coef_e(al, be, 2, k + 1);
    case 2: return coef_e(al + 1, be, 1, k) * coef_e(al, be, 2, k) + coef_e(al + 1, be, 2, k) * coef_e(al, be, 1, k + 1);
    default: return coef_e(al + 1, be, 1, k) * coef_e(al, be, 1, k);
    }
}

// src/Miscellaneous.cpp:351-378 (rho, kappa, theta depend on l1, l2 only)
static double coef_rho(int l1) {
    return 2 * coef_d(-1, -1, l1) * coef_e(-1, 0, 1, l1 - 1) - l1 * coef_b(-1, -1, 2, l1);
}
static double coef_kappa(int l1) {
    return l1 * coef_b(-1, -1, 2, l1) - 2 * coef_d(-1, -1, l1) * coef_e(-1, 0, 1, l1 - 1);
}
static double coef_theta(int l1, int l2) {
    return 2 * coef_d(2 * l1 - 1, -1, l2) * coef_e(-1, 2 * l1, 1, l2 - 1) - l2 * coef_b(2 * l1 - 1, -1, 2, l2);
}

// src/Miscellaneous.cpp:381-468: derivative coefficients of J_alpha
double coef_D(int ind_derivative, int ind_variation, int l1, int l2, int l3) {
    const int a2 = 2 * l1, a3 = 2 * l1 + 2 * l2;
    // factors shared by several cases
    auto dy_second = [&]() {  // the (x2) derivative, variation 1
        return ((2 * coef_d(-1, -1, l1) * coef_e(-1, 0, 1, l1 - 1) - l1 * coef_b(-1, -1, 2, l1)) * coef_b(a2 - 1, -1, 1, l2)
                + 2 * coef_d(a2 - 1, -1, l2) * coef_b(-1, -1, 2, l1) * coef_e(a2 - 1, 0, 2, l2 - 1)) / coef_b(a2 - 2, 0, 1, l2);
    };
    auto dz_var2 = [&]() {
        return (coef_b(-1, -1, 1, l1) * coef_theta(l1, l2) * coef_b(a3 - 1, -1, 1, l3)
                + 2 * coef_d(a3 - 1, -1, l3) * coef_b(-1, -1, 1, l1) * coef_b(a2 - 1, -1, 2, l2) * coef_e(a3 - 1, 0, 2, l3 - 1))
               / coef_b(a3 - 2, 0, 1, l3);
    };
    auto dz_var3 = [&](double lead) {
        return ((lead + coef_b(-1, -1, 2, l1) * coef_e(a2 - 1, -1, 2, l2 - 1) * coef_theta(l1, l2)) * coef_b(a3 - 1, -1, 1, l3)
                + 2 * coef_b(a2 - 2, -1, 1, l2) * coef_d(a3 - 1, -1, l3) * coef_b(-1, -1, 2, l1) * coef_e(a2 - 2, -1, 1, l2)
                  * coef_e(a3 - 1, 0, 2, l3 - 1))
               / (coef_b(a2 - 2, -1, 1, l2) * coef_b(a3 - 2, 0, 1, l3));
    };
    switch (ind_derivative) {
    case 0: return 2 * coef_d(-1, -1, l1);
    case 1:
        if (ind_variation == 0) return 2 * coef_d(a2 - 1, -1, l2) * coef_b(-1, -1, 1, l1);
        return -dy_second();
    case 2:
        switch (ind_variation) {
        case 0: return -2 * coef_d(a3 - 1, -1, l3) * coef_b(-1, -1, 1, l1) * coef_b(a2 - 1, -1, 1, l2);
        case 1: return 2 * coef_d(a3 - 1, -1, l3) * coef_b(-1, -1, 2, l1) * coef_e(a2 - 2, -1, 2, l2);
        case 2: return -dz_var2();
        default: {
            // (b e theta - kappa) variant, src/Miscellaneous.cpp:424-428
            return ((coef_b(-1, -1, 2, l1) * coef_e(a2 - 1, -1, 2, l2 - 1) * coef_theta(l1, l2) - coef_kappa(l1))
                        * coef_b(a3 - 1, -1, 1, l3)
                    + 2 * coef_b(a2 - 2, -1, 1, l2) * coef_d(a3 - 1, -1, l3) * coef_b(-1, -1, 2, l1) * coef_e(a2 - 2, -1, 1, l2)
                      * coef_e(a3 - 1, 0, 2, l3 - 1))
                   / (coef_b(a2 - 2, -1, 1, l2) * coef_b(a3 - 2, 0, 1, l3));
        }
        }
    case 3:
        if (ind_variation == 0) return 2 * coef_d(a2 - 1, -1, l2) * coef_b(-1, -1, 1, l1);
        return dy_second();
    case 4:
        if (ind_variation == 0) return 2 * coef_d(a3 - 1, -1, l3) * coef_b(a2 - 1, -1, 1, l2);
        return ((l2 * coef_b(-1, a2 - 1, 2, l2) - 2 * coef_d(a2 - 1, -1, l2) * coef_e(a2 - 1, 0, 1, l2 - 1)) * coef_b(a3 - 1, -1, 1, l3)
                - 2 * coef_d(a3 - 1, -1, l3) * coef_b(-1, a2 - 1, 2, l2) * coef_e(a3 - 1, 0, 2, l3 - 1))
               / coef_b(a3 - 2, 0, 1, l3);
    default:
        switch (ind_variation) {
        case 0: return 2 * coef_d(a3 - 1, -1, l3) * coef_b(-1, -1, 1, l1) * coef_b(a2 - 1, -1, 1, l2);
        case 1: return 2 * coef_d(a3 - 1, -1, l3) * coef_b(-1, -1, 2, l1) * coef_e(a2 - 2, -1, 2, l2);
        case 2: return dz_var2();
        default: return dz_var3(coef_rho(l1));
        }
    }
}

// src/Miscellaneous.cpp:510-542
double jacobi_gen(int al, int be, int k, double x) {
    if (k == 0) return 1.0;
    if (al + be == -2) {
        if (k == 1) return x;
        return 0.25 * (x - 1) * (x + 1) * jacobi_gen(1, 1, k - 2, x);
    }
    if (al == -1) return (k + be) * (x - 1) / (k * 2) * jacobi_gen(1, be, k - 1, x);
    if (be == -1) return (k + al) * (x + 1) / (k * 2) * jacobi_gen(al, 1, k - 1, x);
    double powv = 1.0, sum = 0.0;
    for (int j = 0; j <= k; ++j) {
        double f = 1.0;
        for (int i = 0; i < k - j; ++i) f *= ((double)(al + j + 1 + i)) / (i + 1);
        for (int i = 0; i < j; ++i) f *= ((double)(k + al + be + 1 + i)) / (i + 1);
        sum += f * powv;
        powv *= (x - 1) / 2;
    }
    return sum;
}

// three-term recurrence J_{k+1} = ((x - a2) J_k - a3 J_{k-1}) / a1, filling J[0..kmax]
static void jacobi_run(int al, int be, double x, int kmax, double* J) {
    J[0] = 1.0;
    if (kmax < 1) return;
    J[1] = jacobi_gen(al, be, 1, x);
    for (int k = 1; k < kmax; ++k)
        J[k + 1] = ((x - coef_a(al, be, 2, k)) * J[k] - coef_a(al, be, 3, k) * J[k - 1]) / coef_a(al, be, 1, k);
}

// ------------------------------------------------------------------ quadrature
void gauss_legendre01(int q, std::vector<double>& x, std::vector<double>& w) {
    x.assign(q, 0.0);
    w.assign(q, 0.0);
    for (int i = 0; i < q; ++i) {
        double z = std::cos(M_PI * (i + 0.75) / (q + 0.5));
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = 0.0;
            for (int j = 1; j <= q; ++j) { double p2 = p1; p1 = p0; p0 = ((2.0 * j - 1.0) * z * p1 - (j - 1.0) * p2) / j; }
            double dp = q * (z * p0 - p1) / (z * z - 1.0);
            double dz = p0 / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-16) break;
        }
        double p0 = 1.0, p1 = 0.0;
        for (int j = 1; j <= q; ++j) { double p2 = p1; p1 = p0; p0 = ((2.0 * j - 1.0) * z * p1 - (j - 1.0) * p2) / j; }
        double dp = q * (z * p0 - p1) / (z * z - 1.0);
        x[i] = 0.5 * (1.0 - z);              // ascending on [0, 1]
        w[i] = 1.0 / ((1.0 - z * z) * dp * dp);  // 2/((1-z^2)P'^2) scaled by 1/2
    }
}

// src/QuadInfo.cpp:63-119
void Quadrature::build(int qq) {
    q = qq;
    gauss_legendre01(q, x1, w1);
    b2.clear(); w2.clear(); x3.clear(); w3.clear();
    for (int i = 0; i < q; ++i)
        for (int j = 0; j < q; ++j) {
            double a = x1[i] * (1 - x1[j]);
            double b = x1[j];
            b2.push_back({a, b, 1 - a - b});
            w2.push_back(2 * (1 - x1[j]) * w1[i] * w1[j]);
        }
    for (int i = 0; i < q; ++i)
        for (int j = 0; j < q; ++j)
            for (int k = 0; k < q; ++k) {
                x3.push_back({x1[i] * (1 - x1[j]) * (1 - x1[k]), x1[j] * (1 - x1[k]), x1[k]});
                w3.push_back(6 * (1 - x1[j]) * std::pow(1 - x1[k], 2) * w1[i] * w1[j] * w1[k]);
            }
}

// ----------------------------------------------------------- local transform
// src/BuildSpace.cpp:296-413
void LocalBasis::init(int order) {
    M = order;
    mi.init(M);
    n_loc = mi.n;
    tl.assign(n_loc, {});
    wtl.assign(n_loc, {});
    auto N = [](int a, int b, int c) { return MultiIndexTable::number(a, b, c); };
    auto set = [&](int j, std::vector<int> t, std::vector<double> w) { tl[j] = t; wtl[j] = w; };
    // vertex modes
    set(0, {0, 1, 2, 3}, {0.125, 0.125, 0.25, 0.5});
    set(1, {0, 1}, {-0.5, 0.5});
    set(2, {0, 1, 2}, {-0.25, -0.25, 0.5});
    set(3, {0, 1, 2, 3}, {-0.125, -0.125, -0.25, 0.5});
    for (int l = 2; l <= M; ++l) {
        // edges along x1, x2, x3 of the reference tet
        set(N(l, 0, 0), {N(l, 0, 0)}, {2.0});
        int a = N(0, l, 0), b = N(1, l - 1, 0);
        set(a, {a, b}, {1.0, 1.0});
        set(b, {a, b}, {((double)(l - 1)) / l, ((double)-(l - 1)) / l});
        int c = N(0, 0, l), d = N(1, 0, l - 1), e = N(0, 1, l - 1);
        set(c, {c, d, e}, {0.5, 0.5, 1.0});
        set(d, {c, d}, {((double)(l - 1)) / l, ((double)-(l - 1)) / l});
        set(e, {c, d, e}, {((double)(l - 1)) / (2 * l), ((double)(l - 1)) / (2 * l), ((double)-(l - 1)) / l});
    }
    for (int l1 = 2; l1 <= M; ++l1)
        for (int l2 = 1; l2 <= M - l1; ++l2) {
            int a = N(0, l1, l2), b = N(1, l1 - 1, l2);
            set(a, {a, b}, {1.0, 1.0});
            set(b, {a, b}, {((double)(l1 - 1)) / l1, ((double)-(l1 - 1)) / l1});
            set(N(l1, 0, l2), {N(l1, 0, l2)}, {2.0});
            set(N(l1, l2, 0), {N(l1, l2, 0)}, {2.0});
        }
    for (int l1 = 2; l1 <= M; ++l1)
        for (int l2 = 1; l2 <= M - l1; ++l2)
            for (int l3 = 1; l3 <= M - l1 - l2; ++l3) {
                int a = N(l1, l2, l3);
                set(a, {a}, {1.0});
            }
}

// src/BuildSpace.cpp:24-51
void LocalBasis::jacobi_values(const double* pt, double* out) const {
    const double x = pt[0], y = pt[1], z = pt[2];
    const double xi = 2 * x / (1 - y - z) - 1, eta = 2 * y / (1 - z) - 1, zeta = 2 * z - 1;
    std::vector<double> Jx(M + 2), Je(M + 2), Jz(M + 2);
    Jx[0] = 1; Jx[1] = xi;
    for (int k = 1; k < M; ++k)
        Jx[k + 1] = ((xi - coef_a(-1, -1, 2, k)) * Jx[k] - coef_a(-1, -1, 3, k) * Jx[k - 1]) / coef_a(-1, -1, 1, k);
    for (int l1 = 0; l1 <= M; ++l1) {
        jacobi_run(2 * l1 - 1, -1, eta, M - l1, Je.data());
        for (int l2 = 0; l2 <= M - l1; ++l2) {
            jacobi_run(2 * l1 + 2 * l2 - 1, -1, zeta, M - l1 - l2, Jz.data());
            for (int l3 = 0; l3 <= M - l1 - l2; ++l3)
                out[MultiIndexTable::number(l1, l2, l3)] =
                    std::pow(1 - y - z, l1) * Jx[l1] * std::pow(1 - z, l2) * Je[l2] * Jz[l3];
        }
    }
}

void LocalBasis::basis_values(const double* pt, double* out) const {
    std::vector<double> J(n_loc);
    jacobi_values(pt, J.data());
    for (int i = 0; i < n_loc; ++i) out[i] = 0;
    for (int i = 0; i < n_loc; ++i)
        for (size_t j = 0; j < tl[i].size(); ++j) out[tl[i][j]] += wtl[i][j] * J[i];
}

// src/BuildSpace.cpp:172-290
void LocalBasis::jacobi_gradients(const double* pt, double* out) const {
    const double x1 = pt[0], x2 = pt[1], x3 = pt[2];
    const double t1 = 1 - x2 - x3, t2 = 1 - x3;
    const double xi = 2 * x1 / t1 - 1, eta = 2 * x2 / t2 - 1, zeta = 2 * x3 - 1;
    std::vector<double> pt1(M + 1), pt2(M + 1);
    pt1[0] = pt2[0] = 1;
    for (int l = 1; l <= M; ++l) { pt1[l] = pt1[l - 1] * t1; pt2[l] = pt2[l - 1] * t2; }
    std::vector<double> Jx0(M + 2), Jx1(M + 2), Je0(M + 2), Je1(M + 2), Je2(M + 2), Jz0(M + 2), Jz1(M + 2);
    jacobi_run(0, 0, xi, M, Jx0.data());
    jacobi_run(0, -1, xi, M, Jx1.data());
    std::vector<double> cJ0(n_loc), cJ1(n_loc), cJ2(n_loc);
    for (int l1 = 0; l1 <= M; ++l1) {
        jacobi_run(2 * l1 + 1, -1, eta, M - l1, Je0.data());
        jacobi_run(2 * l1, 0, eta, M - l1, Je1.data());
        jacobi_run(2 * l1, -1, eta, M - l1, Je2.data());
        for (int l2 = 0; l2 <= M - l1; ++l2) {
            jacobi_run(2 * l1 + 2 * l2 + 1, -1, zeta, M - l1 - l2, Jz0.data());
            jacobi_run(2 * l1 + 2 * l2, 0, zeta, M - l1 - l2, Jz1.data());
            for (int l3 = 0; l3 <= M - l1 - l2; ++l3) {
                int i = MultiIndexTable::number(l1, l2, l3);
                cJ0[i] = pt1[l1] * Jx0[l1] * pt2[l2] * Je0[l2] * Jz0[l3];
                cJ1[i] = pt1[l1] * Jx1[l1] * pt2[l2] * Je1[l2] * Jz0[l3];
                cJ2[i] = pt1[l1] * Jx1[l1] * pt2[l2] * Je2[l2] * Jz1[l3];
            }
        }
    }
    auto N = [](int a, int b, int c) { return MultiIndexTable::number(a, b, c); };
    for (int i = 0; i < n_loc; ++i) {
        const int a = mi.num2idx[i][0], b = mi.num2idx[i][1], c = mi.num2idx[i][2];
        double g0 = 0, g1 = 0, g2 = 0;
        if (a >= 1) g0 += coef_D(0, 0, a, b, c) * cJ0[N(a - 1, b, c)];
        if (b >= 1) g1 += coef_D(3, 0, a, b, c) * cJ1[N(a, b - 1, c)];
        if (a >= 1) g1 += coef_D(3, 1, a, b, c) * cJ1[N(a - 1, b, c)];
        if (c >= 1) g2 += coef_D(5, 0, a, b, c) * cJ2[N(a, b, c - 1)];
        if (a >= 1 && c >= 1) g2 += coef_D(5, 1, a, b, c) * cJ2[N(a - 1, b + 1, c - 1)];
        if (b >= 1) g2 += coef_D(5, 2, a, b, c) * cJ2[N(a, b - 1, c)];
        if (a >= 1) g2 += coef_D(5, 3, a, b, c) * cJ2[N(a - 1, b, c)];
        out[3 * i + 0] = g0; out[3 * i + 1] = g1; out[3 * i + 2] = g2;
    }
}

void LocalBasis::basis_gradients(const double* pt, double* out) const {
    std::vector<double> G(3 * n_loc);
    jacobi_gradients(pt, G.data());
    for (int i = 0; i < 3 * n_loc; ++i) out[i] = 0;
    for (int i = 0; i < n_loc; ++i)
        for (size_t j = 0; j < tl[i].size(); ++j)
            for (int d = 0; d < 3; ++d) out[3 * tl[i][j] + d] += wtl[i][j] * G[3 * i + d];
}

}  // namespace tsem_oracle
