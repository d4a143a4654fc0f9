// FP64 CSR SpMV, PCG and p-multigrid on the GPU.
//
// PCG restates TSEMSolver::solve_PCG (src/TSEMSolver.cpp:1776-1929): r = A x - b,
// y = M^{-1} r, p = -y, stop on ||r||_1 < tol (or ||r||_2 <= tol_rel ||b||_2).  The
// scalars live on the device and the convergence decision is taken there, so an
// iteration costs no host round trip.  The p-multigrid preconditioner restates
// init_PMG / ite_PMG (:36-135, :1120-1183): levels {sum_dof <= q}, injection,
// principal-submatrix coarse operators, forward Gauss-Seidel down, symmetric GS
// on the coarsest level, backward GS up.  Exact lexicographic GS is run as a
// level-scheduled sweep (rows of one dependency level in parallel, earlier rows
// read from the updated vector, later rows from a copy taken at sweep start);
// a Chebyshev-Jacobi smoother is offered as the parallel alternative.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "device.hpp"
#include "linalg.cuh"
#include "solver.hpp"

namespace tsem {

enum { SPMV_PLAIN = 0, SPMV_PAP = 1, SPMV_RESID = 2, SPMV_AXPBY = 3 };

// y = A x with a fused epilogue.  PAP: y = Ax, st->pap += x.y.  RESID: y = Ax - b,
// st->bb += b.b.  AXPBY: y = b - Ax (used for residuals inside the V-cycle).
// TPR lanes share a row; every lane issues U independent (value, column) loads
// before it uses them, so enough bytes are in flight to cover HBM latency.  With
// VEC the lanes load (value, column) pairs as 16- and 8-byte vectors from the
// first even entry of the row, halving the load instructions per entry.
template <int TPR, int U, int MODE, bool VEC = false>
__global__ void __launch_bounds__(256) k_spmv(int64_t n, const int64_t* __restrict__ rp, const int* __restrict__ ci,
                                              const double* __restrict__ va, const double* __restrict__ x,
                                              double* __restrict__ y, const double* __restrict__ b, PcgScalars* st) {
    if (st && st->done) return;
    if (MODE == SPMV_PAP && blockIdx.x == 0 && threadIdx.x == 0) {
        const int cur = st->iter & 1;
        st->cur = cur;
        st->rty[cur ^ 1] = 0.0;
        st->l1 = 0.0;
        st->rr = 0.0;
    }
    const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / TPR;
    const int lane = threadIdx.x & (TPR - 1);
    double s = 0.0;
    if (VEC && row < n) {
        int64_t k0 = rp[row];
        const int64_t end = rp[row + 1];
        if ((k0 & 1) && k0 < end) {
            if (lane == 0) s += va[k0] * __ldg(x + ci[k0]);
            ++k0;
        }
        const int64_t npair = (end - k0) >> 1;
        const double2* vp = reinterpret_cast<const double2*>(va + k0);
        const int2* cp = reinterpret_cast<const int2*>(ci + k0);
        for (int64_t q = lane; q < npair; q += (int64_t)TPR * U) {
            double2 v[U];
            int2 c[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int64_t qq = q + (int64_t)u * TPR;
                const bool ok = qq < npair;
                v[u] = ok ? __ldcs(vp + qq) : make_double2(0.0, 0.0);
                c[u] = ok ? __ldcs(cp + qq) : make_int2(0, 0);
            }
#pragma unroll
            for (int u = 0; u < U; ++u) s += v[u].x * __ldg(x + c[u].x) + v[u].y * __ldg(x + c[u].y);
        }
        if (((end - k0) & 1) && lane == 0) s += va[end - 1] * __ldg(x + ci[end - 1]);
    } else if (row < n) {
        const int64_t beg = rp[row], end = rp[row + 1];
        for (int64_t k = beg + lane; k < end; k += (int64_t)TPR * U) {
            double v[U];
            int c[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int64_t kk = k + (int64_t)u * TPR;
                const bool ok = kk < end;
                v[u] = ok ? __ldcs(va + kk) : 0.0;
                c[u] = ok ? __ldcs(ci + kk) : 0;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) s += v[u] * __ldg(x + c[u]);
        }
    }
#pragma unroll
    for (int o = TPR / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, TPR);
    double acc[1] = {0.0};
    if (row < n && lane == 0) {
        if (MODE == SPMV_PLAIN) {
            y[row] = s;
        } else if (MODE == SPMV_PAP) {
            y[row] = s;
            acc[0] = s * x[row];
        } else if (MODE == SPMV_RESID) {
            const double bv = b[row];
            y[row] = s - bv;
            acc[0] = bv * bv;
        } else {
            y[row] = b[row] - s;
        }
    }
    if (MODE == SPMV_PAP) {
        double* const dst[1] = {&st->pap};
        block_accumulate<1>(acc, dst);
    } else if (MODE == SPMV_RESID) {
        double* const dst[1] = {&st->bb};
        block_accumulate<1>(acc, dst);
    }
}

// FP64 values split into FP32 pairs hi + lo (split_f64)
__global__ void k_split_f64(int64_t n, const double* __restrict__ v, float2* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = split_f64(v[i]);
}

// y = A x with FP32 arithmetic on (hi, lo) pairs: GB300 runs FP64 FMAs at a small
// fraction of its FP32 rate, and a CSR SpMV in FP64 is limited by that pipe, not by
// HBM.  Each product is formed as p + e with p = fl32(vh xh) and e its exact error
// (FMA) plus the two cross terms; the row sum is kept as an unevaluated pair
// (s_hi, s_lo) with an exact two-sum.  The values carry 48 of FP64's 53 bits, the
// products and the sum about 2^-48 relative error -- the size of the FP64 SpMV's own
// rounding for rows of ~100 entries.  Lanes combine in FP64 and the epilogue is FP64.
__device__ __forceinline__ void split_fma(float2 v, float2 xv, float& sh, float& sl) {
    const float p = __fmul_rn(v.x, xv.x);
    float e = __fmaf_rn(v.x, xv.x, -p);
    e = __fmaf_rn(v.x, xv.y, e);
    e = __fmaf_rn(v.y, xv.x, e);
    const float t = __fadd_rn(sh, p);
    const float bp = __fsub_rn(t, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bp)), __fsub_rn(p, bp));
    sh = t;
    sl = __fadd_rn(sl, __fadd_rn(err, e));
}

// VEC: lanes take pairs of entries from the first even one of the row (16-byte
// value and 8-byte column loads)
template <int TPR, int U, int MODE, bool VEC = false>
__global__ void __launch_bounds__(256) k_spmv_split(int64_t n, const int64_t* __restrict__ rp, const int* __restrict__ ci,
                                                    const float2* __restrict__ va, const float2* __restrict__ xs,
                                                    const double* __restrict__ x, double* __restrict__ y,
                                                    const double* __restrict__ b, PcgScalars* st) {
    if (st && st->done) return;
    if (MODE == SPMV_PAP && blockIdx.x == 0 && threadIdx.x == 0) {
        const int cur = st->iter & 1;
        st->cur = cur;
        st->rty[cur ^ 1] = 0.0;
        st->l1 = 0.0;
        st->rr = 0.0;
    }
    const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / TPR;
    const int lane = threadIdx.x & (TPR - 1);
    float sh = 0.0f, sl = 0.0f;
    if (VEC && row < n) {
        int64_t k0 = rp[row];
        const int64_t end = rp[row + 1];
        if ((k0 & 1) && k0 < end) {
            if (lane == 0) split_fma(va[k0], __ldg(xs + ci[k0]), sh, sl);
            ++k0;
        }
        const int64_t npair = (end - k0) >> 1;
        const float4* vp = reinterpret_cast<const float4*>(va + k0);
        const int2* cp = reinterpret_cast<const int2*>(ci + k0);
        for (int64_t q = lane; q < npair; q += (int64_t)TPR * U) {
            float4 v[U];
            int2 c[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int64_t qq = q + (int64_t)u * TPR;
                const bool ok = qq < npair;
                v[u] = ok ? __ldcs(vp + qq) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                c[u] = ok ? __ldcs(cp + qq) : make_int2(0, 0);
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                split_fma(make_float2(v[u].x, v[u].y), __ldg(xs + c[u].x), sh, sl);
                split_fma(make_float2(v[u].z, v[u].w), __ldg(xs + c[u].y), sh, sl);
            }
        }
        if (((end - k0) & 1) && lane == 0) split_fma(va[end - 1], __ldg(xs + ci[end - 1]), sh, sl);
    } else if (row < n) {
        const int64_t beg = rp[row], end = rp[row + 1];
        for (int64_t k = beg + lane; k < end; k += (int64_t)TPR * U) {
            float2 v[U];
            int c[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int64_t kk = k + (int64_t)u * TPR;
                const bool ok = kk < end;
                v[u] = ok ? __ldcs(va + kk) : make_float2(0.0f, 0.0f);
                c[u] = ok ? __ldcs(ci + kk) : 0;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) split_fma(v[u], __ldg(xs + c[u]), sh, sl);
        }
    }
    double s = (double)sh + (double)sl;
#pragma unroll
    for (int o = TPR / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, TPR);
    double acc[1] = {0.0};
    if (row < n && lane == 0) {
        if (MODE == SPMV_PLAIN) {
            y[row] = s;
        } else if (MODE == SPMV_PAP) {
            y[row] = s;
            acc[0] = s * x[row];
        } else if (MODE == SPMV_RESID) {
            const double bv = b[row];
            y[row] = s - bv;
            acc[0] = bv * bv;
        } else {
            y[row] = b[row] - s;
        }
    }
    if (MODE == SPMV_PAP) {
        double* const dst[1] = {&st->pap};
        block_accumulate<1>(acc, dst);
    } else if (MODE == SPMV_RESID) {
        double* const dst[1] = {&st->bb};
        block_accumulate<1>(acc, dst);
    }
}

void csr_split_values(const DevCsr& A, cudaStream_t s) {
    if (!A.split_ok || A.vsplit.n < (size_t)A.nnz) {
        if (A.vsplit.n < (size_t)A.nnz) A.vsplit.alloc(A.nnz);
        k_split_f64<<<grid_for(A.nnz, 256, 152 * 32), 256, 0, s>>>(A.nnz, A.val.p, A.vsplit.p);
        TSEM_LAUNCHED();
        A.split_ok = true;
    }
}

// the split operands of a launch: values once per change of A, x every launch
static void split_operands(const DevCsr& A, const double* x, cudaStream_t s) {
    csr_split_values(A, s);
    if (A.xsplit.n < (size_t)A.n) A.xsplit.alloc(A.n);
    k_split_f64<<<grid_for(A.n, 256, 152 * 32), 256, 0, s>>>(A.n, x, A.xsplit.p);
    TSEM_LAUNCHED();
}

// launch shapes the autotuner times: 0-11 FP64 arithmetic, 12-28 split (hi, lo)
// arithmetic; the later split shapes keep up to 12 (value, column) loads per lane in
// flight, so that lanes x loads can cover a whole row of a p = 5-7 operator in one pass
constexpr int kSpmvVariants = 29;

template <int MODE>
static void spmv_variant(int v, const DevCsr& A, const double* x, double* y, const double* b, PcgScalars* st,
                         cudaStream_t s) {
    const int64_t n = A.n;
    auto grid = [&](int tpr) { return (unsigned)((n * tpr + 255) / 256); };
#define TSEM_SPMV_CASE(I, T, UU, VV)                                                                              \
    case I:                                                                                                       \
        k_spmv<T, UU, MODE, VV><<<grid(T), 256, 0, s>>>(n, A.rowptr.p, A.col.p, A.val.p, x, y, b, st);         \
        break;
    switch (v) {
        TSEM_SPMV_CASE(0, 4, 4, false)
        TSEM_SPMV_CASE(1, 8, 2, false)
        TSEM_SPMV_CASE(2, 8, 4, false)
        TSEM_SPMV_CASE(3, 16, 2, false)
        TSEM_SPMV_CASE(4, 16, 4, false)
        TSEM_SPMV_CASE(5, 32, 1, false)
        TSEM_SPMV_CASE(6, 32, 2, false)
        TSEM_SPMV_CASE(7, 32, 4, false)
        TSEM_SPMV_CASE(8, 4, 2, true)
        TSEM_SPMV_CASE(9, 8, 1, true)
        TSEM_SPMV_CASE(10, 8, 2, true)
        TSEM_SPMV_CASE(11, 16, 2, true)
        default: {
            // FP32-pipe shapes on (hi, lo) pairs
            split_operands(A, x, s);
            static const int tpr[kSpmvVariants - 12] = {4, 8, 8, 16, 4, 8, 8, 8, 4, 8, 16, 16, 8, 32, 8, 16, 4};
            const unsigned g = grid(tpr[v - 12]);
            const auto* va = A.vsplit.p;
            const auto* xs = A.xsplit.p;
            const auto* rp = A.rowptr.p;
            const auto* ci = A.col.p;
            switch (v) {
                case 12: k_spmv_split<4, 4, MODE><<<g, 256, 0, s>>>(n, rp, ci, va, xs, x, y, b, st); break;
                case 13: k_spmv_split<8, 2, MODE><<<g, 256, 0, s>>>(n, rp, ci, va, xs, x, y, b, st); break;
                case 14: k_spmv_split<8, 4, MODE><<<g, 256, 0, s>>>(n, rp, ci, va, xs, x, y, b, st); break;
                case 15: k_spmv_split<16, 2, MODE><<<g, 256, 0, s>>>(n, rp, ci, va, xs, x, y, b, st); break;
                case 16: k_spmv_split<4, 2, MODE, true><<<g, 256, 0, s>>>(n, rp, ci, va, xs, x, y, b, st); break;
                case 17: k_spmv_split<8, 1, MODE, true><<<g, 256, 0, s>>>(n, rp, ci, va, xs, x, y, b, st); break;
                case 18: k_spmv_split<8, 2, MODE, true><<<g, 256, 0, s>>>(n, rp, ci, va, xs, x, y, b, st); break;
                case 19: k_spmv_split<8, 4, MODE, true><<<g, 256, 0, s>>>(n, rp, ci, va, xs, x, y, b, st); break;
                case 20: k_spmv_split<4, 8, MODE><<<g, 256, 0, s>>>(n, rp, ci, va, xs, x, y, b, st); break;
                case 21: k_spmv_split<8, 8, MODE><<<g, 256, 0, s>>>(n, rp, ci, va, xs, x, y, b, st); break;
                case 22: k_spmv_split<16, 4, MODE><<<g, 256, 0, s>>>(n, rp, ci, va, xs, x, y, b, st); break;
                case 23: k_spmv_split<16, 8, MODE><<<g, 256, 0, s>>>(n, rp, ci, va, xs, x, y, b, st); break;
                case 24: k_spmv_split<8, 6, MODE><<<g, 256, 0, s>>>(n, rp, ci, va, xs, x, y, b, st); break;
                case 25: k_spmv_split<32, 4, MODE><<<g, 256, 0, s>>>(n, rp, ci, va, xs, x, y, b, st); break;
                case 26: k_spmv_split<8, 12, MODE><<<g, 256, 0, s>>>(n, rp, ci, va, xs, x, y, b, st); break;
                case 27: k_spmv_split<16, 6, MODE><<<g, 256, 0, s>>>(n, rp, ci, va, xs, x, y, b, st); break;
                default: k_spmv_split<4, 12, MODE><<<g, 256, 0, s>>>(n, rp, ci, va, xs, x, y, b, st); break;
            }
        }
    }
#undef TSEM_SPMV_CASE
    TSEM_LAUNCHED();
}

// z_i = sum_j |a_ij| |x_j|, one warp per row: the scale of the rounding error of row i
// of any summation order
__global__ void k_abs_spmv(int64_t n, const int64_t* __restrict__ rp, const int* __restrict__ ci,
                           const double* __restrict__ va, const double* __restrict__ x, double* __restrict__ z) {
    const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    double s = 0.0;
    for (int64_t k = rp[row] + lane; k < rp[row + 1]; k += 32) s += fabs(va[k]) * fabs(x[ci[k]]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) z[row] = s;
}

// out[0] = max(out[0], max_i |a_i - b_i| / z_i) (a row with z_i = 0 must agree
// exactly); non-negative doubles order like their bit patterns
__global__ void k_maxdiff_scaled(int64_t n, const double* __restrict__ a, const double* __restrict__ b,
                                 const double* __restrict__ z, unsigned long long* out) {
    double m = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double d = fabs(a[i] - b[i]);
        m = fmax(m, z[i] > 0.0 ? d / z[i] : (d > 0.0 ? 1.0 : 0.0));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// Every launch shape sums the same products in another order, or in (hi, lo) FP32
// pairs that carry 48 bits of each operand.  Against the FP64 shape 0 a row may then
// differ by about nnz_row * 2^-53 (the orders) plus a few 2^-48 (the pairs) times
// (|A| |x|)_row: at most about 4e-14 for rows of up to 160 entries.  A shape whose
// largest scaled difference exceeds this bound is defective and stops the tuning.
constexpr double kSpmvShapeTol = 1e-13;

// time every variant on this matrix once and keep the fastest

// Shapes chosen for matrices of one kind (mean row length, size class): a later matrix
// of the same kind takes the shape without timing all of them again (a service makes
// one matrix per request; the timing of 29 shapes cost it more than its solves).
struct SpmvShapeCache {
    std::mutex mu;
    std::map<std::pair<int, int>, int> best;
};
static SpmvShapeCache& spmv_shape_cache() {
    static SpmvShapeCache c;
    return c;
}
static std::pair<int, int> spmv_kind(const DevCsr& A) {
    const int avg = A.n ? (int)std::lround((double)A.nnz / (double)A.n) : 0;
    int sz = 0;
    while (sz < 62 && ((int64_t)1 << (sz + 1)) <= A.n) ++sz;
    return {avg, sz};
}

void spmv_autotune(DevCsr& A, cudaStream_t s, bool reuse) {
    if (A.spmv_variant >= 0) return;
    if (reuse) {
        SpmvShapeCache& c = spmv_shape_cache();
        std::lock_guard<std::mutex> lock(c.mu);
        const auto it = c.best.find(spmv_kind(A));
        if (it != c.best.end()) {
            A.spmv_variant = it->second;
            A.spmv_ms = 0.0f;
            A.spmv_shape_ms.clear();
            A.spmv_shape_err.clear();
            return;
        }
    }
    DBuf<double> x(A.n), y(A.n), y0(A.n);
    DBuf<unsigned long long> diff(kSpmvVariants + 1);
    diff.zero(s);
    std::vector<double> h(A.n);
    uint64_t r = 0x9E3779B97F4A7C15ull;
    for (int64_t i = 0; i < A.n; ++i) {   // values in [-1, 1): no cancellation against constants
        r ^= r << 13; r ^= r >> 7; r ^= r << 17;
        h[i] = (double)(r >> 11) / (double)(1ull << 52) - 1.0;
    }
    x.upload(h, s);
    DBuf<double> zabs(A.n);
    k_abs_spmv<<<grid_for(A.n * 32, 256, INT32_MAX), 256, 0, s>>>(A.n, A.rowptr.p, A.col.p, A.val.p, x.p, zabs.p);
    TSEM_LAUNCHED();
    cudaEvent_t a, b;
    TSEM_CUDA(cudaEventCreate(&a));
    TSEM_CUDA(cudaEventCreate(&b));
    float best = 1e30f;
    int best_v = 5;
    A.spmv_shape_ms.assign(kSpmvVariants, 0.0f);
    for (int v = 0; v < kSpmvVariants; ++v) {
        // warm-up launch, checked against the first variant's result
        spmv_variant<SPMV_PLAIN>(v, A, x.p, v == 0 ? y0.p : y.p, nullptr, nullptr, s);
        if (v > 0) {
            k_maxdiff_scaled<<<grid_for(A.n, 256, 152 * 16), 256, 0, s>>>(A.n, y.p, y0.p, zabs.p, diff.p + v);
            TSEM_LAUNCHED();
        }
        TSEM_CUDA(cudaEventRecord(a, s));
        for (int r = 0; r < 3; ++r) spmv_variant<SPMV_PLAIN>(v, A, x.p, y.p, nullptr, nullptr, s);
        TSEM_CUDA(cudaEventRecord(b, s));
        TSEM_CUDA(cudaEventSynchronize(b));
        float ms = 0;
        TSEM_CUDA(cudaEventElapsedTime(&ms, a, b));
        A.spmv_shape_ms[v] = ms / 3.0f;
        if (ms < best) { best = ms; best_v = v; }
    }
    unsigned long long hd[kSpmvVariants + 1];
    diff.download(hd, kSpmvVariants + 1, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    double dmax[kSpmvVariants + 1];
    std::memcpy(dmax, hd, sizeof(hd));
    A.spmv_shape_err.assign(dmax, dmax + kSpmvVariants);
    for (int v = 1; v < kSpmvVariants; ++v)
        if (!(dmax[v] <= kSpmvShapeTol))
            throw Error(TSEM_CUDA_ERROR, "SpMV launch shape " + std::to_string(v) + " differs from the FP64 shape by " +
                                             std::to_string(dmax[v]) + " of |A||x| (bound " +
                                             std::to_string(kSpmvShapeTol) + ")");
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    A.spmv_variant = best_v;
    A.spmv_ms = best / 3.0f;
    SpmvShapeCache& c = spmv_shape_cache();
    std::lock_guard<std::mutex> lock(c.mu);
    c.best.emplace(spmv_kind(A), best_v);
}

template <int MODE>
static void spmv_launch(const DevCsr& A, const double* x, double* y, const double* b, PcgScalars* st, cudaStream_t s) {
    int v = A.spmv_variant;
    if (v < 0) {
        // untuned matrix: pick by average row length
        const double avg = A.n ? (double)A.nnz / (double)A.n : 0.0;
        v = avg > 48 ? 6 : (avg > 20 ? 3 : (avg > 8 ? 1 : 0));
    }
    spmv_variant<MODE>(v, A, x, y, b, st, s);
}

void csr_spmv(const DevCsr& A, const double* x, double* y, cudaStream_t s) {
    spmv_launch<SPMV_PLAIN>(A, x, y, nullptr, nullptr, s);
}

void csr_residual(const DevCsr& A, const double* x, double* r, const double* b, cudaStream_t s) {
    spmv_launch<SPMV_AXPBY>(A, x, r, b, nullptr, s);
}

// ------------------------------------------------------------------ PCG kernels
__global__ void k_init_jacobi(int64_t n, const double* __restrict__ r, const double* __restrict__ d, double* y, double* p,
                              PcgScalars* st, int precond) {
    double acc[3] = {0, 0, 0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double ri = r[i];
        const double yi = precond == 1 ? ri / d[i] : ri;
        y[i] = yi;
        p[i] = -yi;
        acc[0] += ri * yi;
        acc[1] += fabs(ri);
        acc[2] += ri * ri;
    }
    double* const dst[3] = {&st->rty[0], &st->l1, &st->rr};
    block_accumulate<3>(acc, dst);
}

// after a preconditioner wrote y: p = -y and the init reductions
__global__ void k_init_dot(int64_t n, const double* __restrict__ r, const double* __restrict__ y, double* p, PcgScalars* st) {
    double acc[3] = {0, 0, 0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double ri = r[i], yi = y[i];
        p[i] = -yi;
        acc[0] += ri * yi;
        acc[1] += fabs(ri);
        acc[2] += ri * ri;
    }
    double* const dst[3] = {&st->rty[0], &st->l1, &st->rr};
    block_accumulate<3>(acc, dst);
}

__device__ __forceinline__ bool pcg_converged(const PcgScalars* st) {
    return st->rel_mode ? (st->rr <= st->tol_rel2 * st->bb) : (st->l1 < st->tol_abs);
}

__global__ void k_check_init(PcgScalars* st) {
    st->init_l1 = st->l1;
    st->iter = 0;
    st->pap = 0.0;
    if (!isfinite(st->l1) || !isfinite(st->rty[0])) { st->done = 1; st->status = TSEM_NONFINITE; }
    else if (pcg_converged(st)) { st->done = 1; st->status = TSEM_OK; }
}

// x += alpha p, r += alpha q; Jacobi y = r / d (precond 1) or y = r (precond 0);
// precond 4 leaves y to the V-cycle and only updates x, r, ||r||.
__global__ void k_update(int64_t n, double* x, double* r, const double* __restrict__ p, const double* __restrict__ q,
                         const double* __restrict__ d, double* y, PcgScalars* st, int precond) {
    if (st->done) return;
    const int cur = st->cur;
    const double pap = st->pap;
    if (!(pap > 0.0) || !isfinite(pap)) return;   // breakdown, flagged by k_update_p
    const double alpha = st->rty[cur] / pap;
    double acc[3] = {0, 0, 0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] += alpha * p[i];
        const double ri = r[i] + alpha * q[i];
        r[i] = ri;
        if (precond == 1) {
            const double yi = ri / d[i];
            y[i] = yi;
            acc[0] += ri * yi;
        } else if (precond == 0) {
            y[i] = ri;
            acc[0] += ri * ri;
        } else {
            y[i] = 0.0;
        }
        acc[1] += fabs(ri);
        acc[2] += ri * ri;
    }
    // sweep preconditioners (2 SOR, 3 SSOR, 4 p-MG) start from y = 0 and add r.y after their sweeps
    double* const dst[3] = {precond >= 2 ? nullptr : &st->rty[cur ^ 1], &st->l1, &st->rr};
    block_accumulate<3>(acc, dst);
}

__global__ void k_dot_ry(int64_t n, const double* __restrict__ r, const double* __restrict__ y, PcgScalars* st) {
    if (st->done) return;
    double acc[1] = {0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        acc[0] += r[i] * y[i];
    double* const dst[1] = {&st->rty[st->cur ^ 1]};
    block_accumulate<1>(acc, dst);
}

__global__ void k_update_p(int64_t n, double* p, const double* __restrict__ y, PcgScalars* st) {
    if (st->done) return;
    const int cur = st->cur;
    const double beta = st->rty[cur ^ 1] / st->rty[cur];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = beta * p[i] - y[i];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const int it = st->iter + 1;
        st->iter = it;
        const double pap = st->pap;
        if (!(pap > 0.0) || !isfinite(pap)) { st->done = 1; st->status = TSEM_BREAKDOWN; }
        else if (!isfinite(st->l1) || !isfinite(st->rty[cur ^ 1])) { st->done = 1; st->status = TSEM_NONFINITE; }
        else if (pcg_converged(st)) { st->done = 1; st->status = TSEM_OK; }
        else if (it > st->max_iter) { st->done = 1; st->status = TSEM_MAXIT; }
        st->pap = 0.0;
    }
}

// ------------------------------------------------------------ p-multigrid
__global__ void k_restrict(int64_t nf, const int* __restrict__ core, const double* __restrict__ v, double* rc,
                           const PcgScalars* st) {
    if (st && st->done) return;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nf; j += (int64_t)gridDim.x * blockDim.x) {
        const int c = core[j];
        if (c >= 0) rc[c] = v[j];
    }
}

__global__ void k_prolong_add(int64_t nf, const int* __restrict__ core, const double* __restrict__ xc, double* x,
                              const PcgScalars* st) {
    if (st && st->done) return;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nf; j += (int64_t)gridDim.x * blockDim.x) {
        const int c = core[j];
        if (c >= 0) x[j] += xc[c];
    }
}

__global__ void k_fill(int64_t n, double* x, double v, const PcgScalars* st) {
    if (st && st->done) return;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) x[j] = v;
}

__global__ void k_copy(int64_t n, const double* __restrict__ a, double* b, const PcgScalars* st) {
    if (st && st->done) return;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) b[j] = a[j];
}

// one dependency level of a lexicographic Gauss-Seidel sweep.  FORWARD: columns
// below the row read the updated x, above it the copy x_old; backward the reverse.
template <int TPR, bool FORWARD>
__global__ void __launch_bounds__(256) k_gs_level(int64_t cnt, const int* __restrict__ rows, const int64_t* __restrict__ rp,
                                                  const int* __restrict__ ci, const double* __restrict__ va,
                                                  const double* __restrict__ rhs, const double* __restrict__ x_old,
                                                  double* x, const PcgScalars* st, double omega) {
    if (st && st->done) return;
    const int64_t t = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / TPR;
    const int lane = threadIdx.x & (TPR - 1);
    int r = -1;
    double s = 0.0;
    if (t < cnt) {
        r = rows[t];
        const int64_t beg = rp[r], end = rp[r + 1];
        for (int64_t k = beg + 1 + lane; k < end; k += TPR) {
            const int c = ci[k];
            const bool fresh = FORWARD ? (c < r) : (c > r);
            s += va[k] * (fresh ? x[c] : x_old[c]);
        }
    }
#pragma unroll
    for (int o = TPR / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, TPR);
    // omega = 1: Gauss-Seidel; else SOR x = (1 - omega) x + omega (rhs - s) / d (ite_SOR, src/TSEMSolver.cpp:1288-1304)
    if (t < cnt && lane == 0) {
        const double g = (rhs[r] - s) / va[rp[r]];
        x[r] = omega == 1.0 ? g : (1.0 - omega) * x_old[r] + omega * g;
    }
}

// Chebyshev-Jacobi helpers: d = D^{-1} r * s ;  x += d ; r -= A d handled by spmv
__global__ void k_cheb_first(int64_t n, const double* __restrict__ dinv, const double* __restrict__ r, double* d, double s,
                             double* x, const PcgScalars* st) {
    if (st && st->done) return;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const double v = dinv[j] * r[j] * s;
        d[j] = v;
        x[j] += v;
    }
}
// r -= Ad (ad precomputed); d = a d + c D^{-1} r; x += d
__global__ void k_cheb_step(int64_t n, const double* __restrict__ dinv, double* r, const double* __restrict__ ad, double* d,
                            double a, double c, double* x, int last, const PcgScalars* st) {
    if (st && st->done) return;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const double rj = r[j] - ad[j];
        r[j] = rj;
        const double dj = a * d[j] + c * dinv[j] * rj;
        d[j] = dj;
        x[j] += dj;
    }
}

__global__ void k_invert(int64_t n, const double* __restrict__ d, double* out) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) out[j] = 1.0 / d[j];
}

// power-iteration helpers for the largest eigenvalue of D^{-1} A
__global__ void k_scale_dot(int64_t n, const double* __restrict__ dinv, const double* __restrict__ ay, double* z,
                            const double* __restrict__ y, double* out) {
    double acc[2] = {0, 0};
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const double zj = dinv[j] * ay[j];
        z[j] = zj;
        acc[0] += zj * zj;
        acc[1] += zj * y[j];
    }
    double* const dst[2] = {out, out + 1};
    block_accumulate<2>(acc, dst);
}
__global__ void k_scale(int64_t n, double* x, const double* __restrict__ s) {
    const double f = 1.0 / sqrt(s[0]);
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) x[j] *= f;
}

// extraction of a principal submatrix: keep rows/columns with map >= 0
__global__ void k_sub_count(int64_t n, const int64_t* __restrict__ rp, const int* __restrict__ ci, const int* __restrict__ map,
                            int64_t* cnt) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const int m = map[r];
        if (m < 0) continue;
        int64_t c = 0;
        for (int64_t k = rp[r]; k < rp[r + 1]; ++k) c += map[ci[k]] >= 0;
        cnt[m] = c;
    }
}
__global__ void k_sub_fill(int64_t n, const int64_t* __restrict__ rp, const int* __restrict__ ci, const double* __restrict__ va,
                           const int* __restrict__ map, const int64_t* __restrict__ rpc, int* cc, double* vc) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        const int m = map[r];
        if (m < 0) continue;
        int64_t o = rpc[m];
        for (int64_t k = rp[r]; k < rp[r + 1]; ++k) {
            const int c = map[ci[k]];
            if (c >= 0) { cc[o] = c; vc[o] = va[k]; ++o; }
        }
    }
}

// ------------------------------------------------------------------ host side
static int nblocks(int64_t n) { return grid_for(n, 256, 152 * 16); }

void principal_submatrix(const DevCsr& fine, const std::vector<int>& map, int64_t nc, DevCsr& C, cudaStream_t s) {
    const int64_t n = fine.n;
    DBuf<int> dmap;
    dmap.upload(map, s);
    DBuf<int64_t> cnt(nc);
    k_sub_count<<<nblocks(n), 256, 0, s>>>(n, fine.rowptr.p, fine.col.p, dmap.p, cnt.p);
    TSEM_LAUNCHED();
    std::vector<int64_t> rp(nc + 1, 0);
    cnt.download(rp.data() + 1, nc, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    for (int64_t i = 0; i < nc; ++i) rp[i + 1] += rp[i];
    C.n = nc;
    C.nnz = rp[nc];
    C.rowptr.upload(rp, s);
    C.col.alloc(C.nnz);
    C.val.alloc(C.nnz);
    k_sub_fill<<<nblocks(n), 256, 0, s>>>(n, fine.rowptr.p, fine.col.p, fine.val.p, dmap.p, C.rowptr.p, C.col.p, C.val.p);
    TSEM_LAUNCHED();
    TSEM_CUDA(cudaStreamSynchronize(s));
}

void Pmg::build(const DevCsr& fine, const std::vector<int>& sum_dof, int p, int step, int smoother_, int smooth_,
                cudaStream_t s) {
    smoother = smoother_;
    smooth = smooth_;
    n_project = (p + step - 1) / step - 1 + ((p - 1) % step == 0 ? 0 : 1);
    if (n_project < 1) throw Error(TSEM_INVALID, "p-multigrid needs order >= 2");
    std::vector<int> order(n_project + 1);
    order[0] = p;
    order[n_project] = 1;
    for (int i = 1; i < n_project; ++i) order[i] = order[i - 1] - step;
    const int64_t n = fine.n;
    if ((int64_t)sum_dof.size() != n) throw Error(TSEM_INVALID, "sum_dof length differs from the matrix size");
    levels.clear();
    levels.resize(n_project + 1);
    levels[0].A = &fine;
    levels[0].n = n;
    // global -> index on each level
    std::vector<std::vector<int>> map(n_project + 1, std::vector<int>(n, -1));
    for (int64_t i = 0; i < n; ++i) map[0][i] = (int)i;
    for (int L = 1; L <= n_project; ++L) {
        int c = 0;
        for (int64_t i = 0; i < n; ++i)
            if (sum_dof[i] <= order[L]) map[L][i] = c++;
        levels[L].n = c;
    }
    for (int L = 0; L < n_project; ++L) {
        std::vector<int> core(levels[L].n, -1);
        for (int64_t i = 0; i < n; ++i)
            if (map[L][i] >= 0) core[map[L][i]] = map[L + 1][i];
        levels[L].core.upload(core, s);
    }
    // coarse operators: principal submatrices of the finest matrix (TSEMSolver.cpp:573-656)
    for (int L = 1; L <= n_project; ++L) {
        auto& C = levels[L].own;
        principal_submatrix(fine, map[L], levels[L].n, C, s);
        C.refresh_diag(s);
        spmv_autotune(C, s);
        levels[L].A = &C;
        TSEM_CUDA(cudaStreamSynchronize(s));
    }
    for (int L = 0; L <= n_project; ++L) {
        auto& lv = levels[L];
        lv.x.alloc(lv.n);
        lv.xv = lv.x.p;
        lv.r.alloc(lv.n);
        lv.v.alloc(lv.n);
        lv.t.alloc(lv.n);
        if (smoother == 0) build_gs_schedule(lv, s);
        else build_chebyshev(lv, s);
    }
}

// dependency levels of the forward and backward sweeps (host, once per matrix)
void Pmg::build_gs_schedule(Level& lv, cudaStream_t s) {
    const DevCsr& A = *lv.A;
    const int64_t n = A.n;
    std::vector<int64_t> rp(n + 1);
    std::vector<int> ci(A.nnz);
    A.rowptr.download(rp.data(), n + 1, s);
    A.col.download(ci.data(), A.nnz, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    auto schedule = [&](bool forward, DBuf<int>& perm, std::vector<int64_t>& off) {
        std::vector<int> lev(n, 0);
        int maxl = 0;
        for (int64_t k = 0; k < n; ++k) {
            const int64_t r = forward ? k : n - 1 - k;
            int l = 0;
            for (int64_t q = rp[r] + 1; q < rp[r + 1]; ++q) {
                const int c = ci[q];
                if (forward ? (c < r) : (c > r)) l = std::max(l, lev[c] + 1);
            }
            lev[r] = l;
            maxl = std::max(maxl, l);
        }
        off.assign(maxl + 2, 0);
        for (int64_t r = 0; r < n; ++r) off[lev[r] + 1]++;
        for (int l = 0; l <= maxl; ++l) off[l + 1] += off[l];
        std::vector<int> pr(n);
        std::vector<int64_t> pos(off.begin(), off.end() - 1);
        for (int64_t r = 0; r < n; ++r) pr[pos[lev[r]]++] = (int)r;
        perm.upload(pr, s);
    };
    schedule(true, lv.fperm, lv.foff);
    schedule(false, lv.bperm, lv.boff);
    TSEM_CUDA(cudaStreamSynchronize(s));
}

void Pmg::build_chebyshev(Level& lv, cudaStream_t s) {
    const DevCsr& A = *lv.A;
    const int64_t n = A.n;
    lv.dinv.alloc(n);
    k_invert<<<nblocks(n), 256, 0, s>>>(n, A.diag.p, lv.dinv.p);
    TSEM_LAUNCHED();
    // power iteration on D^{-1} A from a fixed pseudo-random start
    std::vector<double> y0(n);
    uint64_t st = 0x9E3779B97F4A7C15ull;
    for (int64_t i = 0; i < n; ++i) {
        st ^= st << 13; st ^= st >> 7; st ^= st << 17;
        y0[i] = 0.5 + (double)(st >> 11) / (double)(1ull << 53);
    }
    DBuf<double> y, ay, z, acc(2);
    y.upload(y0, s);
    ay.alloc(n);
    z.alloc(n);
    double lam = 1.0;
    double h[2];
    for (int it = 0; it < 30; ++it) {
        csr_spmv(A, y.p, ay.p, s);
        acc.zero(s);
        k_scale_dot<<<nblocks(n), 256, 0, s>>>(n, lv.dinv.p, ay.p, z.p, y.p, acc.p);
        TSEM_LAUNCHED();
        k_scale<<<nblocks(n), 256, 0, s>>>(n, z.p, acc.p);
        TSEM_LAUNCHED();
        std::swap(y.p, z.p);
    }
    acc.download(h, 2, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    // |D^{-1} A y| for the normalised iterate y
    lam = std::sqrt(std::max(h[0], 0.0));
    lv.lmax = 1.1 * std::max(lam, 1e-30);
    lv.lmin = lv.lmax / kChebRange;
}

void Pmg::gs_sweep(Level& lv, const double* rhs, bool forward, int steps, const PcgScalars* st, cudaStream_t s,
                   double omega) {
    const DevCsr& A = *lv.A;
    const DBuf<int>& perm = forward ? lv.fperm : lv.bperm;
    const std::vector<int64_t>& off = forward ? lv.foff : lv.boff;
    const double avg = A.n ? (double)A.nnz / (double)A.n : 0.0;
    for (int it = 0; it < steps; ++it) {
        k_copy<<<nblocks(lv.n), 256, 0, s>>>(lv.n, lv.xv, lv.t.p, st);
        TSEM_LAUNCHED();
        for (size_t L = 0; L + 1 < off.size(); ++L) {
            const int64_t cnt = off[L + 1] - off[L];
            if (cnt == 0) continue;
            const int* rows = perm.p + off[L];
            if (avg > 24) {
                const unsigned g = (unsigned)((cnt * 16 + 255) / 256);
                if (forward) k_gs_level<16, true><<<g, 256, 0, s>>>(cnt, rows, A.rowptr.p, A.col.p, A.val.p, rhs, lv.t.p, lv.xv, st, omega);
                else k_gs_level<16, false><<<g, 256, 0, s>>>(cnt, rows, A.rowptr.p, A.col.p, A.val.p, rhs, lv.t.p, lv.xv, st, omega);
            } else {
                const unsigned g = (unsigned)((cnt * 4 + 255) / 256);
                if (forward) k_gs_level<4, true><<<g, 256, 0, s>>>(cnt, rows, A.rowptr.p, A.col.p, A.val.p, rhs, lv.t.p, lv.xv, st, omega);
                else k_gs_level<4, false><<<g, 256, 0, s>>>(cnt, rows, A.rowptr.p, A.col.p, A.val.p, rhs, lv.t.p, lv.xv, st, omega);
            }
            TSEM_LAUNCHED();
        }
    }
    TSEM_LAUNCH_CHECK();
}

// Chebyshev polynomial smoother for A x = rhs from the current x
void Pmg::chebyshev(Level& lv, const double* rhs, int steps, const PcgScalars* st, cudaStream_t s) {
    const DevCsr& A = *lv.A;
    const int64_t n = lv.n;
    const double theta = 0.5 * (lv.lmax + lv.lmin), delta = 0.5 * (lv.lmax - lv.lmin);
    // r = rhs - A x  (lv.v holds r, lv.t holds d, lv.r is used as the level rhs, so use a local buffer)
    spmv_launch<SPMV_AXPBY>(A, lv.xv, lv.v.p, rhs, const_cast<PcgScalars*>(st), s);
    double rho_old = delta / theta;
    k_cheb_first<<<nblocks(n), 256, 0, s>>>(n, lv.dinv.p, lv.v.p, lv.t.p, 1.0 / theta, lv.xv, st);
    TSEM_LAUNCHED();
    if (!lv.ad.p || lv.ad.n < (size_t)n) lv.ad.alloc(n);
    for (int k = 1; k < steps; ++k) {
        const double rho = 1.0 / (2.0 * theta / delta - rho_old);
        spmv_launch<SPMV_PLAIN>(A, lv.t.p, lv.ad.p, nullptr, const_cast<PcgScalars*>(st), s);
        k_cheb_step<<<nblocks(n), 256, 0, s>>>(n, lv.dinv.p, lv.v.p, lv.ad.p, lv.t.p, rho * rho_old, 2.0 * rho / delta,
                                               lv.xv, k == steps - 1, st);
        TSEM_LAUNCHED();
        rho_old = rho;
    }
    TSEM_LAUNCH_CHECK();
}

// one V-cycle: x (level-0 vector, in/out) for residual r (level 0)
void Pmg::vcycle(double* x0, const double* r0, const PcgScalars* st, cudaStream_t s) {
    // level 0 works in place on the caller's vectors
    levels[0].xv = x0;
    const double* rhs0 = r0;
    for (int L = 0; L < n_project; ++L) {
        Level& lv = levels[L];
        const double* rhs = L == 0 ? rhs0 : lv.r.p;
        if (smoother == 0) gs_sweep(lv, rhs, true, smooth, st, s);
        else chebyshev(lv, rhs, smooth, st, s);
        spmv_launch<SPMV_AXPBY>(*lv.A, lv.xv, lv.v.p, rhs, const_cast<PcgScalars*>(st), s);
        Level& c = levels[L + 1];
        k_restrict<<<nblocks(lv.n), 256, 0, s>>>(lv.n, lv.core.p, lv.v.p, c.r.p, st);
        TSEM_LAUNCHED();
        k_fill<<<nblocks(c.n), 256, 0, s>>>(c.n, c.xv, 0.0, st);
        TSEM_LAUNCHED();
    }
    Level& cl = levels[n_project];
    if (smoother == 0) {
        for (int k = 0; k < (smooth + 1) / 2; ++k) {
            gs_sweep(cl, cl.r.p, true, 1, st, s);
            gs_sweep(cl, cl.r.p, false, 1, st, s);
        }
    } else {
        chebyshev(cl, cl.r.p, 2 * smooth, st, s);
    }
    for (int L = n_project - 1; L >= 0; --L) {
        Level& lv = levels[L];
        const double* rhs = L == 0 ? rhs0 : lv.r.p;
        k_prolong_add<<<nblocks(lv.n), 256, 0, s>>>(lv.n, lv.core.p, levels[L + 1].xv, lv.xv, st);
        TSEM_LAUNCHED();
        if (smoother == 0) gs_sweep(lv, rhs, false, smooth, st, s);
        else chebyshev(lv, rhs, smooth, st, s);
    }
    TSEM_LAUNCH_CHECK();
    levels[0].xv = levels[0].x.p;
}

// ------------------------------------------------------------------- solver
Solver::Solver(const DevCsr* A_, const tsem_solver_opts& o, const std::vector<int>& sum_dof, int p, cudaStream_t s)
    : A(A_), opts(o), stream(s) {
    spmv_autotune(const_cast<DevCsr&>(*A), s);
    const int64_t n = A->n;
    r.alloc(n); y.alloc(n); pv.alloc(n); q.alloc(n); x.alloc(n); b.alloc(n);
    sc.alloc(1);
    hsc = pinned_slot<PcgScalars>();
    TSEM_CUDA(cudaEventCreate(&ev0));
    TSEM_CUDA(cudaEventCreate(&ev1));
    if (opts.precond == 4) {
        pmg = std::make_unique<Pmg>();
        pmg->build(*A, sum_dof, p, std::max(1, opts.pmg_order_step), opts.smoother, std::max(1, opts.smooth_steps), s);
    } else if (opts.precond == 2 || opts.precond == 3) {
        const double w = opts.omega != 0.0 ? opts.omega : 1.0;
        if (!(w > 0.0 && w < 2.0)) throw Error(TSEM_INVALID, "SOR parameter omega must lie in (0, 2)");
        sor = std::make_unique<Pmg::Level>();
        sor->A = A;
        sor->n = n;
        sor->t.alloc(n);
        Pmg::build_gs_schedule(*sor, s);
    } else if (opts.precond != 0 && opts.precond != 1) {
        throw Error(TSEM_INVALID, "preconditioner must be 0 (none), 1 (Jacobi), 2 (SOR), 3 (SSOR) or 4 (p-multigrid)");
    }
}

// y = preconditioner(r) in place from the current y: one V-cycle (4), or smooth_steps
// SOR sweeps (2) / forward-and-backward SSOR sweeps (3, ite_SSOR, src/TSEMSolver.cpp:1307-1345)
void Solver::precondition(const PcgScalars* st, cudaStream_t s) {
    if (opts.precond == 4) {
        pmg->vcycle(y.p, r.p, st, s);
        return;
    }
    const double w = opts.omega != 0.0 ? opts.omega : 1.0;
    sor->xv = y.p;
    for (int it = 0; it < std::max(1, opts.smooth_steps); ++it) {
        Pmg::gs_sweep(*sor, r.p, true, 1, st, s, w);
        if (opts.precond == 3) Pmg::gs_sweep(*sor, r.p, false, 1, st, s, w);
    }
}

Solver::~Solver() {
    if (hsc) pinned_slot<PcgScalars>(hsc);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
}

__global__ void k_l1_norm(int64_t n, const double* __restrict__ v, double* out) {
    double acc[1] = {0.0};
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        acc[0] += fabs(v[i]);
    double* const dst[1] = {out};
    block_accumulate<1>(acc, dst);
}

// solve_PMG (src/TSEMSolver.cpp:1446-1536): V-cycles on x in place until the l1 norm
// of A x - b drops below tol or max_step cycles ran.  The coarsest level takes the
// (smooth + 1) / 2 symmetric sweeps of ite_PMG (the reference's solve_PMG takes
// smooth / 2 there).
void Solver::solve_pmg(const double* bd, double* xd, double tol, int max_step, tsem_stats* out, cudaStream_t s) {
    if (!pmg) throw Error(TSEM_INVALID, "solver has no p-multigrid preconditioner");
    const int64_t n = A->n;
    DBuf<double> acc(1);
    double l1 = 0.0, l1_0 = 0.0;
    auto residual = [&] {
        csr_residual(*A, xd, r.p, bd, s);
        acc.zero(s);
        k_l1_norm<<<nblocks(n), 256, 0, s>>>(n, r.p, acc.p);
        TSEM_LAUNCHED();
        acc.download(&l1, 1, s);
        TSEM_CUDA(cudaStreamSynchronize(s));
    };
    residual();
    l1_0 = l1;
    int it = 0;
    while (std::isfinite(l1) && l1 >= tol && it <= max_step) {
        pmg->vcycle(xd, bd, nullptr, s);
        ++it;
        residual();
    }
    out->iterations = it;
    out->residual_l1 = l1;
    out->init_l1 = l1_0;
    out->status = !std::isfinite(l1) ? TSEM_NONFINITE : l1 < tol ? TSEM_OK : TSEM_MAXIT;
}

void Solver::solve(const double* bd, double* xd, tsem_stats* out, cudaStream_t s) {
    const int64_t n = A->n;
    const int prec = opts.precond;
    std::memset(hsc, 0, sizeof(PcgScalars));
    hsc->tol_abs = opts.tol_abs_l1;
    hsc->tol_rel2 = opts.tol_rel * opts.tol_rel;
    hsc->rel_mode = opts.tol_rel > 0 ? 1 : 0;
    hsc->max_iter = opts.max_iter > 0 ? opts.max_iter : 100000;
    TSEM_CUDA(cudaEventRecord(ev0, s));
    TSEM_CUDA(cudaMemcpyAsync(sc.p, hsc, sizeof(PcgScalars), cudaMemcpyHostToDevice, s));
    PcgScalars* st = sc.p;
    // r = A x - b
    spmv_launch<SPMV_RESID>(*A, xd, r.p, bd, st, s);
    if (prec >= 2) {
        // the reference's first preconditioner call starts from y = x (TSEMSolver.cpp:1790, 1819)
        TSEM_CUDA(cudaMemcpyAsync(y.p, xd, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        precondition(nullptr, s);
        k_init_dot<<<nblocks(n), 256, 0, s>>>(n, r.p, y.p, pv.p, st);
        TSEM_LAUNCHED();
    } else {
        k_init_jacobi<<<nblocks(n), 256, 0, s>>>(n, r.p, A->diag.p, y.p, pv.p, st, prec);
        TSEM_LAUNCHED();
    }
    TSEM_LAUNCH_CHECK();
    k_check_init<<<1, 1, 0, s>>>(st);
    TSEM_LAUNCHED();
    const int chunk = prec >= 2 ? 1 : 16;
    for (;;) {
        for (int c = 0; c < chunk; ++c) {
            spmv_launch<SPMV_PAP>(*A, pv.p, q.p, nullptr, st, s);
            k_update<<<nblocks(n), 256, 0, s>>>(n, xd, r.p, pv.p, q.p, A->diag.p, y.p, st, prec);
            TSEM_LAUNCHED();
            if (prec >= 2) {
                precondition(st, s);
                k_dot_ry<<<nblocks(n), 256, 0, s>>>(n, r.p, y.p, st);
                TSEM_LAUNCHED();
            }
            k_update_p<<<nblocks(n), 256, 0, s>>>(n, pv.p, y.p, st);
            TSEM_LAUNCHED();
        }
        TSEM_LAUNCH_CHECK();
        TSEM_CUDA(cudaMemcpyAsync(hsc, sc.p, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s));
        TSEM_CUDA(cudaStreamSynchronize(s));
        if (hsc->done) break;
    }
    TSEM_CUDA(cudaEventRecord(ev1, s));
    TSEM_CUDA(cudaEventSynchronize(ev1));
    float ms = 0;
    TSEM_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    if (out) {
        out->iterations = hsc->iter;
        out->status = hsc->status;
        out->residual_l1 = hsc->l1;
        out->init_l1 = hsc->init_l1;
        out->residual_rel = hsc->bb > 0 ? std::sqrt(hsc->rr / hsc->bb) : std::sqrt(hsc->rr);
        out->device_ms = ms;
    }
}

}  // namespace tsem
