// TEST INFRASTRUCTURE ONLY -- CPU oracle (see oracle.hpp).
#pragma once
#include "oracle.hpp"

namespace tsem_oracle {

struct LobpcgStats { int iterations = 0; double residual = 0; int status = 0; };

double solve_inverse_power(const Csr& A, const Csr& B, double* x, double tol, int max_step, int* iters);
void sym_eig(int n, std::vector<double> a, std::vector<double>& w, std::vector<double>& v);
// Rayleigh-Ritz of the pencil (GA, GB), m x m row-major: the r Ritz values of the
// numerically independent span (ascending) and coefficients C (m x r, row-major,
// C^T GB C = I); stands in for LAPACKE_dsygvx at src/TSEMSolver.cpp:2179, 2349
int rayleigh_ritz(int m, const std::vector<double>& GA0, const std::vector<double>& GB0, std::vector<double>& theta,
                  std::vector<double>& C);
LobpcgStats solve_lobpcg(const Csr& A, const Csr& B, int k, double* X, double* lambda, double tol, int max_it,
                         int precond, const PMG* pmg, int smooth);

}  // namespace tsem_oracle
