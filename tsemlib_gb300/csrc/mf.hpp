// Matrix-free operator and the mixed-precision (FP32 inner / FP64 outer) solver.
#pragma once
#include <cuda_runtime.h>

#include <deque>
#include <memory>
#include <utility>
#include <vector>

#include "device.hpp"
#include "linalg.cuh"

namespace tsem {

// One p-multigrid level of the matrix-free operator: element modes |alpha| <= q.
struct MfLevel {
    int q = 1, nl = 4, nlp = 4, md = 1;  // modes, padded row stride of S, transform terms
    int nl4 = 4, kpad = 16;              // tensor-core path: row block stride, padded K
    bool tc = false;                     // BF16 tcgen05 apply available on this level
    DBuf<uint16_t> Bt;                   // [512][kpad] BF16 stacked reference matrices (core-matrix layout)
    bool tcw = false;                    // BF16 tcgen05 apply in launches over groups of the six matrices
    int tcw_kc = 0, tcw_nh = 0;          // (levels wider than the accumulator): matrices per launch, MMA N
    bool x3 = false;                     // split-TF32 tcgen05 apply (FP32-accurate) available
    bool x3w = false;                    // the same in launches over the groups of tcw (wide levels)
    int kq = 0;                          // its K steps of 8 modes
    DBuf<float> B3;                      // [kq][hi/lo][512][8] split stacked matrices (core-matrix layout);
                                         // wide levels: [group][kq][hi/lo][2 tcw_nh][8]
    bool csr = false;                    // level applied as an assembled FP32 CSR matrix instead
    int csr_tpr = 8;                     // lanes per row of its SpMV (autotuned on the level)
    DBuf<int64_t> crp;                   // its row starts, columns and values (principal submatrix
    DBuf<int> ccol;                      // of the FP64 operator, rounded to FP32)
    DBuf<float> cval;
    int64_t n = 0;                       // DOFs on this level
    DBuf<int> gi;                        // [E][nl][md] level index of each transform term (-1: none)
    DBuf<float> gv;                      // [E][nl][md] value (0 for Dirichlet DOFs)
    DBuf<float> S;                       // [6][nl][nlp] leading blocks of the reference stiffness
    bool unit = false;                   // one transform term per mode, coefficient 0 or +-1
    DBuf<int> gp;                        // [nl][E] packed signed index of unit levels
    DBuf<int> trp, tpos;                 // transposed transform: per DOF its (mode, element) results
    DBuf<float> tval;                    // their coefficients (empty on unit levels: sign in tpos)
    DBuf<float> bdiag;                   // [n] diagonal of Dirichlet DOFs, 0 elsewhere
    DBuf<int> bnd;                       // Dirichlet DOFs of this level
    DBuf<float> bnd_diag;                // their diagonal entries
    DBuf<float> dinv;                    // inverse diagonal of the level operator
    DBuf<int> core;                      // this level -> next coarser level (or -1)
    DBuf<float> x, r, v, t, ad;          // work vectors
    float* xv = nullptr;
    double lmax = 1, lmin = 1;
};

// One operator of a grouped element GEMM (k_mf_apply_tcg over a ragged table of
// operators of the same order on different meshes): its packed gather indices, input
// vector, element weights and per-element results, its element count and the index
// of its first tile in the launch.
struct TcgOp {
    const int* gp;
    const float* x;
    const float* w6;
    float* V;
    int64_t n;                       // length of x
    int E, tile0;
};

// ---- groups of solves: one launch over the same level of several solves of the same
// order on different meshes.  The operands of every solve on a level sit in a table
// in device memory; the launch runs over the solves' DOFs (or rows) one after the
// other, and solve s owns the indices [g0_s, g0_{s+1}) (entry nops is a sentinel
// whose g0 is the total).
constexpr int kGroupMax = 64;        // solves in one group
constexpr int kChebMax = 64;         // Chebyshev steps a group record holds coefficients for
struct GroupLevel {
    int64_t g0, n;                   // first index of this solve, DOFs of the level
    const int* trp;                  // matrix-free level: transposed transform and results
    const int* tpos;
    const float* V;
    int64_t vlen;                    // floats of V
    const float* bdiag;
    const int64_t* crp;              // assembled level: FP32 CSR
    const int* ccol;
    const float* cval;
    const float* dinv;
    const float* rhs;                // level right-hand side (the PCG residual on level 0)
    float* x;                        // level solution (the preconditioned residual on level 0)
    float *t, *ad, *v;               // work vectors
    const int* core;                 // to the next coarser level (-1: none)
    float* rc;                       // the next coarser level's right-hand side
    const float* xc;                 // the next coarser level's solution
    const PcgScalars* st;            // the solve's inner PCG state (its work is skipped once done)
    float s0;                        // Chebyshev first-step scale and step coefficients
    float a[kChebMax], c[kChebMax];
};
// the level-0 vectors and state of one solve's inner PCG, for the grouped vector updates
struct GroupPcg {
    int64_t n;
    float *x, *r, *p, *q, *z;
    PcgScalars* st;
};

// vector update fused into the scatter of a matrix-free apply (see k_scatter_t)
struct MfPost {
    enum { kStore = 0, kResid = 1, kChebFirst = 2, kChebStep = 3 };
    int mode = kStore;
    float* y = nullptr;
    const float* rhs = nullptr;
    float* v = nullptr;
    float* d = nullptr;
    float* xs = nullptr;
    const float* dinv = nullptr;
    float a = 0.0f, c = 0.0f;
    const PcgScalars* st = nullptr;
};

struct MfOperator {
    int E = 0, M = 0, n_loc = 0;
    DBuf<float> w6;                      // [6][E] = 2/(3|T|) * G_k (stiffness weights)
    std::vector<MfLevel> levels;         // levels[0] = order M
    DBuf<float> U32;                     // gathered element tiles, FP32 path
    DBuf<uint16_t> U16;                  // gathered element tiles, BF16 tensor-core path
    DBuf<float> U3;                      // gathered element tiles, split-TF32 tensor-core path
    DBuf<float> Vbuf;                    // per-element results V[e][i] (row stride nl | 1) before the scatter
    DBuf<int> err;                       // first failing bounded wait (0 = none)
    void build(tsem_space_s* sp, const DevCsr& A_bc, int dirichlet_flag, int order_step, cudaStream_t s);
    // low_precision selects the BF16 tensor-core GEMM where the level has one; otherwise
    // the split-TF32 tensor-core GEMM, or the FP32 CUDA-core GEMM on levels without it
    void apply(int level, const float* x, float* y, cudaStream_t s, bool low_precision = false) const;
    // matrix-free levels only: A x with the update `po` fused into the scatter
    void apply_post(int level, float* x, const MfPost& po, cudaStream_t s, bool low_precision, int ncol = 1) const;
    // ncol columns n_level apart; their results go ncol x vcol floats into Vbuf
    // halt: the solve's state (nothing runs once it is done)
    void elements(int level, const float* x, cudaStream_t s, bool low_precision, cudaEvent_t mid = nullptr,
                  int ncol = 1, const PcgScalars* halt = nullptr) const;
    void elements_col(int level, const float* x, float* V, cudaStream_t s, int path, cudaEvent_t mid) const;
    void scatter(int level, float* x, const MfPost& po, cudaStream_t s, int ncol = 1) const;
    // levels applied as assembled matrices: A x with a Chebyshev row update fused in
    void spmv_cheb(int level, int mode, const float* x, const MfPost& po, float* dn, cudaStream_t s,
                   int ncol = 1) const;
    int64_t vcol = 0;                    // Vbuf floats per column
    int cols = 1;                        // columns Vbuf holds
    void ensure_columns(int ncol);
    void profile(int level, bool low_precision, int reps, const float* x, float* y, cudaStream_t s, double* out) const;
};

// group launches (one per V-cycle step over all members of a group)
void group_elements(const MfLevel& L, const TcgOp* ops, int nops, int units, int* err, cudaStream_t s);
void group_cheb_zero(const GroupLevel* T, int nops, int64_t total, bool deferred, cudaStream_t s);
void group_scatter(int mode, int k, const GroupLevel* T, int nops, int64_t total, cudaStream_t s);
void group_spmv_cheb(int tpr, int mode, int k, const GroupLevel* T, int nops, int64_t total, cudaStream_t s);
void group_f_add(bool use_ad, const GroupLevel* T, int nops, int64_t total, cudaStream_t s);
void group_restrict(const GroupLevel* T, int nops, int64_t total, cudaStream_t s);
void group_prolong(const GroupLevel* T, int nops, int64_t total, cudaStream_t s);
void group_pcg(int phase, const GroupPcg* P, int nops, int64_t nmax, cudaStream_t s);

// allocation-free FP32 apply: scratch in a static device array of this size
constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;
size_t mf_noalloc_need_bytes(const MfOperator& op, int level);
void mf_apply_noalloc(const MfOperator& op, int level, const float* x, float* y, cudaStream_t s);

struct MixedSolver {
    const DevCsr* A;                     // FP64 operator with boundary conditions (outer residual)
    MfOperator op;
    tsem_solver_opts opts;
    int smooth = 2;
    bool lowp = true;                    // BF16 tensor-core operator inside the Chebyshev smoother
    double inner_tol = 1e-6;             // smallest reduction asked of one inner solve
    double inner_rel = 1e-6;             // reduction asked of the current inner solve
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
    // CUDA graphs: one inner PCG iteration, and V-cycles on fixed vectors (LOBPCG)
    cudaStream_t cap = nullptr;
    cudaGraphExec_t it_exec = nullptr;
    long long it_kernels = 0;
    struct VcGraph {
        const float* r;
        float* x;
        int ncol;
        cudaGraphExec_t exec;
        long long kernels;
    };
    std::vector<VcGraph> vc_graphs;
    // z = V-cycle(r) replayed from a graph captured for this (r, z, ncol); a block of
    // ncol columns n apart runs as one V-cycle whose launches cover all columns
    void vcycle_graph(const float* r0, float* x0, cudaStream_t s, int ncol = 1);
    int cols = 1;                        // columns the level vectors hold
    void ensure_columns(int ncol, cudaStream_t s);

    MixedSolver(tsem_space_s* sp, const DevCsr* A, int dirichlet_flag, const tsem_solver_opts& o, cudaStream_t s);
    ~MixedSolver();
    void solve(const double* b, double* x, tsem_stats* out, cudaStream_t s);
    // z = V-cycle(r) of the FP32 matrix-free p-multigrid (z from zero)
    void vcycle(const float* r0, float* x0, const PcgScalars* st, cudaStream_t s, int ncol = 1);
    // the start of an inner solve of A d = rhs: state on the device, r = rhs, d = 0,
    // z = V-cycle(r), p = z (the iterations follow, alone or in a group)
    void inner_begin(const float* rhs, float* x, cudaStream_t s);

   private:
    template <class F>
    cudaGraphExec_t capture(F&& body, long long& kernels);
    void replay(cudaGraphExec_t ex, long long kernels, cudaStream_t s);
    void chebyshev(MfLevel& lv, const float* rhs, int steps, const PcgScalars* st, cudaStream_t s, bool x_zero,
                   int ncol = 1);
    int inner_pcg(const float* rhs, float* x, cudaStream_t s);
};

// A system of a batch solve: the solver, its right-hand side and solution (device).
struct BatchItem {
    MixedSolver* S;
    const double* b;
    double* x;
    tsem_stats stats{};
};
// every matrix-free level of S can run in a group (fused-gather BF16 GEMM), and two
// solvers whose levels have the same shapes can share one
bool groupable(const MixedSolver& S);
bool same_shape(const MixedSolver& a, const MixedSolver& b);
// Solve every system of `items` (FP64 refinement around the FP32 matrix-free PCG of
// each solver, the same result as MixedSolver::solve on each to its tolerance).  The
// inner PCG iterations of all systems in their inner phase run in lockstep rounds:
// solvers of the same order whose levels have the same shape form a group, and each
// step of the group's V-cycle is one launch over a ragged table of their levels (the
// tensor-core element GEMM over all their element tiles, the scatter over all their
// DOFs); a round (one iteration of every member) is one CUDA graph.  Systems whose
// inner solve has converged take their FP64 refinement step between rounds and join
// again; converged systems retire.
void solve_batch(std::vector<BatchItem>& items, cudaStream_t s);

struct MixedGroup;
// Continuous batching: systems join at the next round after submit(); round() runs one
// inner iteration of every system in its inner solve (grouped as solve_batch does),
// the refinement steps that are due, and returns the systems that retired in it
// (converged, failed or cancelled), with their statistics filled in.  Not thread-safe:
// one thread drives an engine.
class BatchEngine {
   public:
    struct Entry;
    explicit BatchEngine(cudaStream_t s);
    ~BatchEngine();
    BatchEngine(const BatchEngine&) = delete;
    BatchEngine& operator=(const BatchEngine&) = delete;
    int64_t submit(BatchItem* it);
    bool cancel(int64_t ticket);
    std::vector<std::pair<int64_t, BatchItem*>> round();
    int in_flight() const;
    cudaStream_t stream() const { return s; }

   private:
    cudaStream_t s;
    int64_t last_ticket = 0;
    std::deque<std::unique_ptr<Entry>> pending;
    std::vector<std::unique_ptr<Entry>> active;
    std::vector<std::unique_ptr<MixedGroup>> slots;   // one per group of a round, reused
    cudaStream_t cap = nullptr;                       // where a steady group's round is captured
};

// test hook: the poll limit of the bounded device waits that may give up
void set_wait_polls(long long polls);
// the bounds checks of the checked build (-DTSEM_CHECK): set the divisor of every
// bound (shrink >= 1), read and clear the first failure; false without the checks
bool bounds_check(int shrink, int* code, long long* index);

}  // namespace tsem
