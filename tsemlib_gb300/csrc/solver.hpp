// PCG and p-multigrid objects (implementation in solve.cu).
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <vector>

#include "device.hpp"
#include "linalg.cuh"

namespace tsem {

struct Pmg {
    struct Level {
        int64_t n = 0;
        const DevCsr* A = nullptr;
        DevCsr own;                       // coarse levels own their operator
        DBuf<int> core;                   // fine index -> coarse index or -1
        DBuf<double> x, r, v, t, ad;      // iterate, level rhs, residual, scratch
        double* xv = nullptr;             // working iterate (the caller's vector on level 0)
        // exact Gauss-Seidel: rows grouped by dependency level
        DBuf<int> fperm, bperm;
        std::vector<int64_t> foff, boff;
        // Chebyshev-Jacobi
        DBuf<double> dinv;
        double lmax = 1, lmin = 1;
    };
    int n_project = 0, smoother = 0, smooth = 2;
    std::vector<Level> levels;

    void build(const DevCsr& fine, const std::vector<int>& sum_dof, int p, int step, int smoother, int smooth,
               cudaStream_t s);
    void vcycle(double* x0, const double* r0, const PcgScalars* st, cudaStream_t s);
    // exact lexicographic (S)OR sweeps of one level, scheduled by dependency levels
    static void build_gs_schedule(Level& lv, cudaStream_t s);
    static void gs_sweep(Level& lv, const double* rhs, bool forward, int steps, const PcgScalars* st, cudaStream_t s,
                         double omega = 1.0);

   private:
    void build_chebyshev(Level& lv, cudaStream_t s);
    void chebyshev(Level& lv, const double* rhs, int steps, const PcgScalars* st, cudaStream_t s);
};

struct Solver {
    const DevCsr* A;
    tsem_solver_opts opts;
    cudaStream_t stream;
    DBuf<double> r, y, pv, q, x, b;
    DBuf<PcgScalars> sc;
    PcgScalars* hsc = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::unique_ptr<Pmg> pmg;
    std::unique_ptr<Pmg::Level> sor;   // SOR / SSOR sweeps on A (precond 2, 3)

    Solver(const DevCsr* A, const tsem_solver_opts& o, const std::vector<int>& sum_dof, int p, cudaStream_t s);
    ~Solver();
    // b, x device pointers (x holds the initial guess)
    void solve(const double* b, double* x, tsem_stats* out, cudaStream_t s);
    // stationary p-multigrid iteration (solve_PMG)
    void solve_pmg(const double* b, double* x, double tol, int max_step, tsem_stats* out, cudaStream_t s);
    void precondition(const PcgScalars* st, cudaStream_t s);
};

}  // namespace tsem

#include "mf.hpp"

struct tsem_solver_s {
    std::unique_ptr<tsem::Solver> impl;
    std::unique_ptr<tsem::MixedSolver> mixed;
    tsem::DBuf<double> hb, hx;   // staging for host-array solves of the mixed solver
    cudaStream_t stream = nullptr;
    int device = 0;
};
