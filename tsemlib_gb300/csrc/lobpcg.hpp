// Block LOBPCG for the smallest eigenpairs of A x = lambda M x (implementation in lobpcg.cu).
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "device.hpp"

namespace tsem {

struct Solver;
struct MixedSolver;

struct LobpcgResult {
    int iterations = 0;
    int status = 0;          // tsem_status
    double residual = 0.0;   // max relative residual of the wanted pairs
    float device_ms = 0.0f;
    int jacobi_sweeps = 0;   // most Jacobi sweeps of any Rayleigh-Ritz step
};

// X: device, column-major n x k (column j at X + j * n), initial block in and
// eigenvectors out; lambda: host, k values.  The preconditioner is the solver's
// (p-multigrid V-cycle, or Jacobi), FP64 for a plain solver and the FP32
// matrix-free V-cycle for a mixed one.
LobpcgResult lobpcg(const DevCsr& A, const DevCsr& M, Solver* plain, MixedSolver* mixed, int k, int n_want, double* X,
                    double* lambda, double tol, int max_it, cudaStream_t s);

}  // namespace tsem
