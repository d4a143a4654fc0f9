// Generalised Jacobi polynomials and the TSEM modal basis, callable on host and device.
//
// The basis is TSEMLib's (src/BuildSpace.cpp:16-51 and :296-413): with collapsed
// coordinates xi = 2x/(1-y-z)-1, eta = 2y/(1-z)-1, zeta = 2z-1,
//   J_{l1,l2,l3} = (1-y-z)^l1 J_l1^{-1,-1}(xi) (1-z)^l2 J_l2^{2l1-1,-1}(eta) J_l3^{2l1+2l2-1,-1}(zeta)
// and the vertex/edge/face/interior basis phi is a fixed sparse recombination of
// the J_alpha.  Polynomials with an index -1 follow the generalised definition of
// src/Miscellaneous.cpp:510-542; the others are the classical P_n^{(a,b)}.  The
// value is evaluated here with a dual-number type, so gradients are exact without
// the reference's derivative-coefficient tables.
#pragma once
#include <cmath>

#ifdef __CUDACC__
#define TSEM_HD __host__ __device__ __forceinline__
#else
#define TSEM_HD inline
#endif

namespace tsem {

// value and gradient with respect to the three reference coordinates
struct Dual {
    double v, d0, d1, d2;
    TSEM_HD Dual() : v(0), d0(0), d1(0), d2(0) {}
    TSEM_HD Dual(double c) : v(c), d0(0), d1(0), d2(0) {}
    TSEM_HD Dual(double a, double b, double c, double d) : v(a), d0(b), d1(c), d2(d) {}
};
TSEM_HD Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d0 + b.d0, a.d1 + b.d1, a.d2 + b.d2); }
TSEM_HD Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d0 - b.d0, a.d1 - b.d1, a.d2 - b.d2); }
TSEM_HD Dual operator*(Dual a, Dual b) {
    return Dual(a.v * b.v, a.d0 * b.v + a.v * b.d0, a.d1 * b.v + a.v * b.d1, a.d2 * b.v + a.v * b.d2);
}
TSEM_HD Dual operator*(double s, Dual a) { return Dual(s * a.v, s * a.d0, s * a.d1, s * a.d2); }
TSEM_HD Dual operator/(Dual a, Dual b) {
    double iv = 1.0 / b.v;
    double q = a.v * iv;
    return Dual(q, (a.d0 - q * b.d0) * iv, (a.d1 - q * b.d1) * iv, (a.d2 - q * b.d2) * iv);
}

// classical Jacobi P_n^{(a,b)}(x), n = 0..nmax, by the standard three-term recurrence
template <class T>
TSEM_HD void jacobi_classic(double a, double b, T x, int nmax, T* P) {
    P[0] = T(1.0);
    if (nmax < 1) return;
    P[1] = T(0.5 * (a - b)) + (0.5 * (a + b + 2)) * x;
    for (int n = 2; n <= nmax; ++n) {
        const double s = 2.0 * n + a + b;
        const double c1 = 2.0 * n * (n + a + b) * (s - 2);
        const double c2 = (s - 1) * (a * a - b * b);
        const double c3 = (s - 1) * s * (s - 2);
        const double c4 = 2.0 * (n + a - 1) * (n + b - 1) * s;
        P[n] = ((T(c2) + c3 * x) * P[n - 1] - c4 * P[n - 2]) / T(c1);
    }
}

// generalised J_k^{(a,b)}(x) for a, b >= -1, k = 0..kmax (kmax <= KMAX)
template <class T, int KMAX>
TSEM_HD void jacobi_general(int a, int b, T x, int kmax, T* J) {
    T tmp[KMAX + 1];
    if (a == -1 && b == -1) {
        J[0] = T(1.0);
        if (kmax >= 1) J[1] = x;
        if (kmax >= 2) {
            jacobi_classic<T>(1, 1, x, kmax - 2, tmp);
            T q = 0.25 * ((x - T(1.0)) * (x + T(1.0)));
            for (int k = 2; k <= kmax; ++k) J[k] = q * tmp[k - 2];
        }
    } else if (a == -1) {
        J[0] = T(1.0);
        if (kmax >= 1) {
            jacobi_classic<T>(1, b, x, kmax - 1, tmp);
            for (int k = 1; k <= kmax; ++k) J[k] = ((double)(k + b) / (2.0 * k)) * ((x - T(1.0)) * tmp[k - 1]);
        }
    } else if (b == -1) {
        J[0] = T(1.0);
        if (kmax >= 1) {
            jacobi_classic<T>(a, 1, x, kmax - 1, tmp);
            for (int k = 1; k <= kmax; ++k) J[k] = ((double)(k + a) / (2.0 * k)) * ((x + T(1.0)) * tmp[k - 1]);
        }
    } else {
        jacobi_classic<T>(a, b, x, kmax, J);
    }
}

// position of alpha in the lexicographic order: degree, then a1+a2, then a2
TSEM_HD int mi_number(int a0, int a1, int a2) {
    const int s0 = a0 + a1 + a2, s1 = a1 + a2;
    int num = 0;
    if (s0 > 0) num += s0 * (s0 + 1) * (s0 + 2) / 6;  // #{|beta| <= s0-1}, 3 components
    if (s1 > 0) num += s1 * (s1 + 1) / 2;             // #{|beta| <= s1-1}, 2 components
    if (a2 > 0) num += a2;                            // #{beta <= a2-1}, 1 component
    return num;
}

// J_alpha for all |alpha| <= M at a reference point; out indexed by mi_number.
template <class T, int MMAX>
TSEM_HD void jacobi_products(int M, const T& x, const T& y, const T& z, T* out) {
    const T one(1.0);
    const T t1 = one - y - z, t2 = one - z;
    const T xi = (2.0 * x) / t1 - one, eta = (2.0 * y) / t2 - one, zeta = 2.0 * z - one;
    T Jx[MMAX + 1], Je[MMAX + 1], Jz[MMAX + 1], p1[MMAX + 1], p2[MMAX + 1];
    jacobi_general<T, MMAX>(-1, -1, xi, M, Jx);
    p1[0] = one; p2[0] = one;
    for (int l = 1; l <= M; ++l) { p1[l] = p1[l - 1] * t1; p2[l] = p2[l - 1] * t2; }
    for (int l1 = 0; l1 <= M; ++l1) {
        jacobi_general<T, MMAX>(2 * l1 - 1, -1, eta, M - l1, Je);
        const T a = p1[l1] * Jx[l1];
        for (int l2 = 0; l2 <= M - l1; ++l2) {
            jacobi_general<T, MMAX>(2 * l1 + 2 * l2 - 1, -1, zeta, M - l1 - l2, Jz);
            const T b = a * (p2[l2] * Je[l2]);
            for (int l3 = 0; l3 <= M - l1 - l2; ++l3) out[mi_number(l1, l2, l3)] = b * Jz[l3];
        }
    }
}

}  // namespace tsem
