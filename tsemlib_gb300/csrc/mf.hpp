// Matrix-free operator and the mixed-precision (FP32 inner / FP64 outer) solver.
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <vector>

#include "device.hpp"
#include "linalg.cuh"

namespace tsem {

// One p-multigrid level of the matrix-free operator: element modes |alpha| <= q.
struct MfLevel {
    int q = 1, nl = 4, nlp = 4, md = 1;  // modes, padded row stride of S, transform terms
    int64_t n = 0;                       // DOFs on this level
    DBuf<int> gi;                        // [E][nl][md] level index of each transform term (-1: none)
    DBuf<float> gv;                      // [E][nl][md] value (0 for Dirichlet DOFs)
    DBuf<float> S;                       // [6][nl][nlp] leading blocks of the reference stiffness
    DBuf<int> bnd;                       // Dirichlet DOFs of this level
    DBuf<float> bnd_diag;                // their diagonal entries
    DBuf<float> dinv;                    // inverse diagonal of the level operator
    DBuf<int> core;                      // this level -> next coarser level (or -1)
    DBuf<float> x, r, v, t, ad;          // work vectors
    float* xv = nullptr;
    double lmax = 1, lmin = 1;
};

struct MfOperator {
    int E = 0, M = 0, n_loc = 0;
    DBuf<float> w6;                      // [E][6] = 2/(3|T|) * G_k (stiffness weights)
    std::vector<MfLevel> levels;         // levels[0] = order M
    void build(tsem_space_s* sp, const DevCsr& A_bc, int dirichlet_flag, int order_step, cudaStream_t s);
    void apply(int level, const float* x, float* y, cudaStream_t s) const;
};

struct MixedSolver {
    const DevCsr* A;                     // FP64 operator with boundary conditions (outer residual)
    MfOperator op;
    tsem_solver_opts opts;
    int smooth = 2;
    double inner_tol = 1e-5;
    int inner_max = 200;
    // outer FP64 residual
    DBuf<double> r64;
    // inner FP32 vectors on the fine level: rhs, solution, residual, preconditioned residual, p, A p
    DBuf<float> rf, dsol, rw, z, p, q;
    DBuf<PcgScalars> sc;
    PcgScalars* hsc = nullptr;
    DBuf<double> red;                    // reduction scratch
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int last_inner = 0, last_outer = 0;

    MixedSolver(tsem_space_s* sp, const DevCsr* A, int dirichlet_flag, const tsem_solver_opts& o, cudaStream_t s);
    ~MixedSolver();
    void solve(const double* b, double* x, tsem_stats* out, cudaStream_t s);

   private:
    void vcycle(const float* r0, float* x0, const PcgScalars* st, cudaStream_t s);
    void chebyshev(MfLevel& lv, const float* rhs, int steps, const PcgScalars* st, cudaStream_t s);
    int inner_pcg(const float* rhs, float* x, cudaStream_t s);
};

}  // namespace tsem
