// TEST INFRASTRUCTURE ONLY -- CPU oracle (see oracle.hpp).
#pragma once
#include "oracle.hpp"

namespace tsem_oracle {

struct LobpcgStats { int iterations = 0; double residual = 0; int status = 0; };

double solve_inverse_power(const Csr& A, const Csr& B, double* x, double tol, int max_step, int* iters);
void sym_eig(int n, std::vector<double> a, std::vector<double>& w, std::vector<double>& v);
LobpcgStats solve_lobpcg(const Csr& A, const Csr& B, int k, double* X, double* lambda, double tol, int max_it,
                         int precond, const PMG* pmg, int smooth);

}  // namespace tsem_oracle
