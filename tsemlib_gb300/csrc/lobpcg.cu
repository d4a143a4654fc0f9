// Block LOBPCG (TSEMSolver::solve_LOBPCG, src/TSEMSolver.cpp:2071-2222 for one
// vector and :2225-2406 for a block) on the device.
//
// The basis S = [X W P] of every iteration lives row-major in one n x 3k array
// (columns [0,k) X, [k,2k) W, [2k,3k) P), with A S and M S beside it: the block
// products (CSR times a block, Gram matrices S^T A S and S^T M S, and the Ritz
// combinations S C) then read whole rows.  Gram matrices and the Rayleigh-Ritz
// problem are FP64; the small generalized eigenproblem is solved on the device by
// one CTA (K10 below), and so is the convergence test, so that one iteration is a
// fixed sequence of launches: it is captured once as a CUDA graph and replayed in
// chunks, the host reading the state once per chunk.
// The residual block R = A X - M X Lambda is preconditioned with the solver's
// p-multigrid V-cycle: FP64 column by column for a plain solver; FP32 matrix-free
// for a mixed one, where the whole block is one V-cycle whose launches cover all k
// columns (the element GEMMs run over (column, tile) pairs).  The reference
// preconditions with an inner PCG on S/2 - lambda M (src/TSEMSolver.cpp:2136-2151).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "linalg.cuh"
#include "lobpcg.hpp"
#include "solver.hpp"

namespace tsem {

namespace {

constexpr int kMaxBlock = 38;     // columns of one block (X, W or P): the Rayleigh-Ritz kernel holds two 3k x 3k FP64 matrices in shared memory
constexpr int kGramRows = 16;     // rows per shared-memory stage of the Gram kernel (two stages)
constexpr int kGramThreads = 256;

// ---- FP64 on the FP32 pipe.  GB300 runs FP64 instructions, conversions included,
// at a small fraction of its FP32 rate.  The blocks of the iteration (the basis S =
// [X W P], A S and M S, and their successors) therefore live in HBM as (hi, lo) FP32
// pairs, about 2^-48 relative, and every product and sum of the block kernels is
// formed with exact FP32 error terms (compensated sums); FP64 appears only in the
// small Gram and coefficient matrices, the Rayleigh-Ritz factorisation and at the
// entry and exit of the call.
__device__ __forceinline__ float2 split2(double d) { return split_f64(d); }
// (sh, sl) += a * b
__device__ __forceinline__ void acc2(float2 a, float2 b, float& sh, float& sl) {
    const float p = __fmul_rn(a.x, b.x);
    float e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
    const float t = __fadd_rn(sh, p);
    const float bp = __fsub_rn(t, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, bp)), __fsub_rn(p, bp));
    sh = t;
    sl = __fadd_rn(sl, __fadd_rn(err, e));
}
// h + l as a normalised pair (TwoSum): |lo| at most half an ulp of hi
__device__ __forceinline__ float2 pair_norm(float h, float l) {
    const float s = __fadd_rn(h, l);
    const float bb = __fsub_rn(s, h);
    return make_float2(s, __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(l, bb)));
}
__device__ __forceinline__ double pair_val(float2 a) { return (double)a.x + (double)a.y; }

// Ya = A X and, when two patterns coincide, Yb = B X in the same pass (B's values vb
// on A's pattern): the matrices' values as pairs, the block X (row stride ldx) and
// the results (row stride ldy) pairs.  A row is served by 2^lsh lanes, each owning
// CPL consecutive columns of the kc, so that a warp works on several rows at once
// with every lane busy; each (value, column) load of the row then feeds CPL
// products per matrix.
template <int CPL, bool TWO>
__global__ void __launch_bounds__(256, 4)
k_spmm_split(const int* __restrict__ halt, int64_t n, int lsh, const int64_t* __restrict__ rp,
             const int* __restrict__ ci, const float2* __restrict__ va, const float2* __restrict__ vb,
             const float2* __restrict__ X, int ldx, int kc, float2* __restrict__ Ya, float2* __restrict__ Yb, int ldy) {
    if (halt && *halt) return;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t row = t >> lsh;
    const int j0 = (int)(t & ((1 << lsh) - 1)) * CPL;
    if (row >= n || j0 >= kc) return;
    const int nc = min(CPL, kc - j0);
    float ah[CPL], al[CPL], bh[CPL], bl[CPL];
#pragma unroll
    for (int u = 0; u < CPL; ++u) ah[u] = al[u] = bh[u] = bl[u] = 0.0f;
    const int64_t e = rp[row + 1];
    int64_t k = rp[row];
    for (; k + 2 <= e; k += 2) {
        const float2* x0 = X + (size_t)ci[k] * ldx + j0;
        const float2* x1 = X + (size_t)ci[k + 1] * ldx + j0;
        const float2 a0 = va[k], a1 = va[k + 1];
        float2 b0 = a0, b1 = a1;
        if (TWO) { b0 = vb[k]; b1 = vb[k + 1]; }
        float2 y0[CPL], y1[CPL];
#pragma unroll
        for (int u = 0; u < CPL; ++u)
            if (u < nc) { y0[u] = x0[u]; y1[u] = x1[u]; }
#pragma unroll
        for (int u = 0; u < CPL; ++u)
            if (u < nc) {
                acc2(a0, y0[u], ah[u], al[u]);
                acc2(a1, y1[u], ah[u], al[u]);
                if (TWO) {
                    acc2(b0, y0[u], bh[u], bl[u]);
                    acc2(b1, y1[u], bh[u], bl[u]);
                }
            }
    }
    if (k < e) {
        const float2* x0 = X + (size_t)ci[k] * ldx + j0;
        const float2 a0 = va[k];
        const float2 b0 = TWO ? vb[k] : a0;
#pragma unroll
        for (int u = 0; u < CPL; ++u)
            if (u < nc) {
                const float2 y = x0[u];
                acc2(a0, y, ah[u], al[u]);
                if (TWO) acc2(b0, y, bh[u], bl[u]);
            }
    }
#pragma unroll
    for (int u = 0; u < CPL; ++u)
        if (u < nc) {
            Ya[(size_t)row * ldy + j0 + u] = pair_norm(ah[u], al[u]);
            if (TWO) Yb[(size_t)row * ldy + j0 + u] = pair_norm(bh[u], bl[u]);
        }
}

// out[k] for k in the pattern of P (rows rp, columns cp): the (hi, lo) value of Q at
// the same (row, column), zero where Q has no entry; flag = 1 when Q has an entry
// outside P's pattern.  Rows hold the diagonal first and then ascending columns, so
// a row merges in one pass; an entry the merge misses is looked for in the whole row.
__global__ void k_embed_values(int64_t n, const int64_t* __restrict__ rp, const int* __restrict__ cp,
                               const int64_t* __restrict__ rq, const int* __restrict__ cq, const float2* __restrict__ vq,
                               float2* __restrict__ out, int* flag) {
    for (int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; row < n; row += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p0 = rp[row], p1 = rp[row + 1];
        for (int64_t k = p0; k < p1; ++k) out[k] = make_float2(0.f, 0.f);
        int64_t k = p0;
        for (int64_t j = rq[row]; j < rq[row + 1]; ++j) {
            const int c = cq[j];
            while (k < p1 && cp[k] != c && (k == p0 || cp[k] < c)) ++k;
            int64_t hit = (k < p1 && cp[k] == c) ? k : -1;
            if (hit < 0)
                for (int64_t t = p0; t < p1; ++t)
                    if (cp[t] == c) { hit = t; break; }
            if (hit < 0) { *flag = 1; break; }
            out[hit] = vq[j];
            if (hit == p0) k = p0 + 1;
        }
    }
}

// flag = 1 when the two CSR patterns differ (rows or columns)
__global__ void k_pattern_diff(int64_t n, int64_t nnz, const int64_t* __restrict__ ra, const int64_t* __restrict__ rb,
                               const int* __restrict__ ca, const int* __restrict__ cb, int* flag) {
    bool diff = false;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nnz; i += (int64_t)gridDim.x * blockDim.x) {
        diff = diff || ca[i] != cb[i];
        if (i <= n) diff = diff || ra[i] != rb[i];
    }
    if (diff) *flag = 1;
}

// 8-byte asynchronous copy global -> shared; bytes = 0 fills zeros and reads nothing
__device__ __forceinline__ void cp_async8(void* dst, const void* src, int bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// G1[a][b] += sum_i S[i][a] T1[i][b] and, with T2, G2[a][b] += sum_i S[i][a] T2[i][b]
// (a < m1, b < m2; with `upper` only b >= a) on pair blocks, FP64 sums of pair
// products (compensated).  A block streams kGramRows rows of the blocks at a time
// through two shared-memory stages (asynchronous copies, zero-filled to multiples of
// 4 columns): the next stage loads while the current one is summed.  A thread owns
// a 4 x 4 tile of each G in registers and a share of the stage's rows (when the tiles
// are fewer than the threads, several threads take the same tile on different rows),
// so that four 16-byte loads of S and T feed sixteen products per G; the partial
// sums go to G by FP64 atomics.  S^T A S and S^T M S share S's loads.
template <bool TWO>
__global__ void __launch_bounds__(kGramThreads, 2)
k_gram(const int* __restrict__ halt, int64_t n, int m1, int m2, const float2* __restrict__ S, int lds,
       const float2* __restrict__ T1, const float2* __restrict__ T2, int ldt, int upper, double* G1, double* G2) {
    if (halt && *halt) return;
    extern __shared__ float4 shs4[];
    const int m1p = (m1 + 3) & ~3, m2p = (m2 + 3) & ~3;
    const int stage = kGramRows * (m1p + (TWO ? 2 : 1) * m2p);
    float2* const st0 = reinterpret_cast<float2*>(shs4);
    const int ta_n = m1p / 4, tb_n = m2p / 4;
    // the tiles: all of them, or (upper, m1 == m2) those with tb >= ta
    const int n_tiles = upper ? ta_n * (ta_n + 1) / 2 : ta_n * tb_n;
    // row groups: threads beyond the tiles take the same tiles on other rows
    const int groups = n_tiles >= kGramThreads ? 1 : min(kGramRows, kGramThreads / n_tiles);
    const int64_t step = (int64_t)gridDim.x * kGramRows;
    // the copies of the stage of rows r0.. into buffer st
    auto load = [&](int64_t r0, float2* st) {
        if (r0 < n) {
            float2* Ss = st;
            float2* T1s = Ss + kGramRows * m1p;
            float2* T2s = T1s + kGramRows * m2p;
            for (int idx = threadIdx.x; idx < kGramRows * m1p; idx += blockDim.x) {
                const int64_t r = r0 + idx / m1p;
                const int c = idx % m1p;
                const bool in = r < n && c < m1;
                cp_async8(Ss + idx, in ? (const void*)(S + (size_t)r * lds + c) : (const void*)S, in ? 8 : 0);
            }
            for (int idx = threadIdx.x; idx < kGramRows * m2p; idx += blockDim.x) {
                const int64_t r = r0 + idx / m2p;
                const int c = idx % m2p;
                const bool in = r < n && c < m2;
                cp_async8(T1s + idx, in ? (const void*)(T1 + (size_t)r * ldt + c) : (const void*)T1, in ? 8 : 0);
                if (TWO) cp_async8(T2s + idx, in ? (const void*)(T2 + (size_t)r * ldt + c) : (const void*)T2, in ? 8 : 0);
            }
        }
        cp_async_commit();
    };
    for (int tile0 = 0; tile0 < n_tiles; tile0 += kGramThreads) {
        const int slot = threadIdx.x % (groups > 1 ? n_tiles : kGramThreads);
        const int grp = groups > 1 ? threadIdx.x / n_tiles : 0;
        const int tile = tile0 + slot;
        const bool active = tile < n_tiles && grp < groups;
        int ta = 0, tb = 0;
        if (active) {
            if (!upper) {
                ta = tile / tb_n;
                tb = tile % tb_n;
            } else {
                int t = tile;
                while (ta < ta_n && t >= ta_n - ta) {
                    t -= ta_n - ta;
                    ++ta;
                }
                tb = ta + t;
            }
        }
        float ah[4][4], al[4][4], bh[4][4], bl[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) ah[i][j] = al[i][j] = bh[i][j] = bl[i][j] = 0.0f;
        __syncthreads();   // the stages are free (a previous tile pass may still read them)
        int64_t r0 = (int64_t)blockIdx.x * kGramRows;
        load(r0, st0);
        for (int it = 0; r0 < n; ++it, r0 += step) {
            float2* cur = st0 + (it & 1) * stage;
            load(r0 + step, st0 + ((it + 1) & 1) * stage);   // the next stage (an empty group past the end)
            cp_async_wait1();
            __syncthreads();
            if (active) {
                const float2* Ss = cur;
                const float2* T1s = Ss + kGramRows * m1p;
                const float2* T2s = T1s + kGramRows * m2p;
                const int rows = (int)min((int64_t)kGramRows, n - r0);
                for (int r = grp; r < rows; r += groups) {
                    const float4* sp = reinterpret_cast<const float4*>(Ss + r * m1p + 4 * ta);
                    const float4 s01 = sp[0], s23 = sp[1];
                    const float2 sv[4] = {make_float2(s01.x, s01.y), make_float2(s01.z, s01.w),
                                          make_float2(s23.x, s23.y), make_float2(s23.z, s23.w)};
                    {
                        const float4* tp = reinterpret_cast<const float4*>(T1s + r * m2p + 4 * tb);
                        const float4 t01 = tp[0], t23 = tp[1];
                        const float2 tv[4] = {make_float2(t01.x, t01.y), make_float2(t01.z, t01.w),
                                              make_float2(t23.x, t23.y), make_float2(t23.z, t23.w)};
#pragma unroll
                        for (int i = 0; i < 4; ++i)
#pragma unroll
                            for (int j = 0; j < 4; ++j) acc2(sv[i], tv[j], ah[i][j], al[i][j]);
                    }
                    if (TWO) {
                        const float4* tp = reinterpret_cast<const float4*>(T2s + r * m2p + 4 * tb);
                        const float4 t01 = tp[0], t23 = tp[1];
                        const float2 tv[4] = {make_float2(t01.x, t01.y), make_float2(t01.z, t01.w),
                                              make_float2(t23.x, t23.y), make_float2(t23.z, t23.w)};
#pragma unroll
                        for (int i = 0; i < 4; ++i)
#pragma unroll
                            for (int j = 0; j < 4; ++j) acc2(sv[i], tv[j], bh[i][j], bl[i][j]);
                    }
                }
            }
            __syncthreads();   // the stage is read before the copies two steps on refill it
        }
        if (active) {
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int a = 4 * ta + i, b = 4 * tb + j;
                    if (a < m1 && b < m2 && (!upper || b >= a)) {
                        atomicAdd(G1 + (size_t)a * m2 + b, (double)ah[i][j] + (double)al[i][j]);
                        if (TWO) atomicAdd(G2 + (size_t)a * m2 + b, (double)bh[i][j] + (double)bl[i][j]);
                    }
                }
        }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
}

// Ritz combinations of up to three pair blocks with one coefficient matrix: for z =
// blockIdx.y, Y_z[i][j] = sum_{a<m} S_z[i][a0 + a] C[a][j] (j < kc, C row-major
// m x kc, FP64, split once per block into shared memory); with P set (z = 0 only)
// also P[i][j] = sum_{a>=c0} S_0[i][a0 + a] C[a][j], the partial sum on the way down
// from a = m - 1.  A row is served by 2^lsh lanes of one warp, each owning CPL
// consecutive columns; the warp has read all its rows before any lane writes, so Y_z
// may overwrite S_z's columns in place.
struct ComboBlocks {
    const float2* S[3];
    float2* Y[3];
};
template <int CPL>
__global__ void __launch_bounds__(256)
k_combo(const int* __restrict__ halt, int64_t n, int lsh, int m, int kc, int lds, int a0,
        const double* __restrict__ C, ComboBlocks blk, int ldy, float2* __restrict__ P, int c0) {
    if (halt && *halt) return;
    extern __shared__ float2 Cs[];
    for (int idx = threadIdx.x; idx < m * kc; idx += blockDim.x) Cs[idx] = split2(C[idx]);
    __syncthreads();
    const int z = blockIdx.y;
    const float2* __restrict__ S = z == 0 ? blk.S[0] : z == 1 ? blk.S[1] : blk.S[2];
    float2* Y = z == 0 ? blk.Y[0] : z == 1 ? blk.Y[1] : blk.Y[2];
    float2* Pz = z == 0 ? P : nullptr;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t row = t >> lsh;
    const int j0 = (int)(t & ((1 << lsh) - 1)) * CPL;
    const bool live = row < n && j0 < kc;
    const int nc = live ? min(CPL, kc - j0) : 0;
    float h[CPL], l[CPL];
#pragma unroll
    for (int u = 0; u < CPL; ++u) h[u] = l[u] = 0.0f;
    if (live) {
        const float2* sr = S + (size_t)row * lds + a0;
        for (int a = m - 1; a >= 0; --a) {
            if (Pz && a == c0 - 1) {
#pragma unroll
                for (int u = 0; u < CPL; ++u)
                    if (u < nc) Pz[(size_t)row * ldy + j0 + u] = pair_norm(h[u], l[u]);
            }
            const float2 sv = sr[a];
            const float2* cr = Cs + a * kc + j0;
#pragma unroll
            for (int u = 0; u < CPL; ++u)
                if (u < nc) acc2(sv, cr[u], h[u], l[u]);
        }
    }
    __syncwarp();
#pragma unroll
    for (int u = 0; u < CPL; ++u)
        if (u < nc) Y[(size_t)row * ldy + j0 + u] = pair_norm(h[u], l[u]);
}

// R[i][j] = AX[i][j] - lambda_j MX[i][j] (pairs); nrm[j] += R^2, nrm[k + j] += MX^2
// (FP32 squares of the leading parts, FP64 totals: the norms only scale and test)
__global__ void k_block_resid(const int* __restrict__ halt, int64_t n, int kc, const float2* __restrict__ AX,
                              const float2* __restrict__ MX, int ld, const double* __restrict__ lam,
                              float2* __restrict__ R, int ldr, double* nrm) {
    if (halt && *halt) return;
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int j = lane; j < kc; j += 32) {
        float rr = 0.0f, mm = 0.0f;
        const float2 l2 = split2(-lam[j]);
        for (int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; row < n; row += warps) {
            const float2 mx = MX[(size_t)row * ld + j];
            const float2 ax = AX[(size_t)row * ld + j];
            float h = ax.x, l = ax.y;
            acc2(l2, mx, h, l);
            const float2 r = pair_norm(h, l);
            R[(size_t)row * ldr + j] = r;
            rr = __fmaf_rn(r.x, r.x, rr);
            mm = __fmaf_rn(mx.x, mx.x, mm);
        }
        atomicAdd(nrm + j, (double)rr);
        atomicAdd(nrm + kc + j, (double)mm);
    }
}

// column j of a row-major pair block <-> a contiguous FP64 vector
__global__ void k_col_get(const int* __restrict__ halt, int64_t n, const float2* __restrict__ B, int ld,
                          double* __restrict__ v) {
    if (halt && *halt) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v[i] = pair_val(B[(size_t)i * ld]);
}
__global__ void k_col_put(const int* __restrict__ halt, int64_t n, const double* __restrict__ v, float2* __restrict__ B,
                          int ld) {
    if (halt && *halt) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        B[(size_t)i * ld] = split2(v[i]);
}
// the k columns of B (row stride ld) as FP32 columns n apart, column j scaled by sc[j]
__global__ void k_block_get_f32(const int* __restrict__ halt, int64_t n, int k, const float2* __restrict__ B, int ld,
                                const double* __restrict__ sc, float* __restrict__ v) {
    if (halt && *halt) return;
    const int j = blockIdx.y;
    const float f = (float)sc[j];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float2 b = B[(size_t)i * ld + j];
        v[(size_t)j * n + i] = __fmul_rn(__fadd_rn(b.x, b.y), f);
    }
}
// back: B[i][j] = v[j][i] * sc[j], the product exact as a pair
__global__ void k_block_put_f32(const int* __restrict__ halt, int64_t n, int k, const float* __restrict__ v,
                                const double* __restrict__ sc, float2* __restrict__ B, int ld) {
    if (halt && *halt) return;
    const int j = blockIdx.y;
    const float2 f = split2(sc[j]);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float z = v[(size_t)j * n + i];
        const float p = __fmul_rn(z, f.x);
        const float e = __fmaf_rn(z, f.y, __fmaf_rn(z, f.x, -p));
        B[(size_t)i * ld + j] = pair_norm(p, e);
    }
}
__global__ void k_jacobi_col(const int* __restrict__ halt, int64_t n, const double* __restrict__ d, double* v) {
    if (halt && *halt) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v[i] /= d[i];
}
// column-major FP64 n x k block <-> columns [0, k) of a row-major pair block
__global__ void k_cm_to_rm(int64_t n, int kc, const double* __restrict__ X, float2* __restrict__ B, int ld) {
    const int64_t total = n * kc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / kc;
        const int j = (int)(t % kc);
        B[(size_t)i * ld + j] = split2(X[(size_t)j * n + i]);
    }
}
__global__ void k_rm_to_cm(int64_t n, int kc, const float2* __restrict__ B, int ld, double* __restrict__ X) {
    const int64_t total = n * kc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int j = (int)(t / n);
        const int64_t i = t % n;
        X[(size_t)j * n + i] = pair_val(B[(size_t)i * ld + j]);
    }
}

__global__ void k_zero(const int* __restrict__ halt, int64_t n, double* __restrict__ p) {
    if (halt && *halt) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = 0.0;
}
// columns [c0, c0 + kc) of three row-major pair blocks (blockIdx.y picks the pair): dst = src
__global__ void k_copy_cols(const int* __restrict__ halt, int64_t n, int kc, int ld, int c0, const float2* s0, float2* d0,
                            const float2* s1, float2* d1, const float2* s2, float2* d2) {
    if (halt && *halt) return;
    const float2* src = blockIdx.y == 0 ? s0 : blockIdx.y == 1 ? s1 : s2;
    float2* dst = blockIdx.y == 0 ? d0 : blockIdx.y == 1 ? d1 : d2;
    const int64_t total = n * kc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const size_t o = (size_t)(t / kc) * ld + c0 + t % kc;
        dst[o] = src[o];
    }
}

// ---- the iteration's state on the device
struct LobState {
    PcgScalars ps;           // ps.done: every kernel of an iteration returns at once; ps.status
    int k, n_want, max_it;
    int iter;                // iterations done
    int rank;                // numerical rank of the last Rayleigh-Ritz basis
    int sweeps;              // most Jacobi sweeps of any Rayleigh-Ritz step
    double tol, residual;
};

// per-column scales of the block V-cycle: 1/|r_j| in, |r_j| out
__global__ void k_lob_scales(const int* __restrict__ halt, int k, const double* __restrict__ nrm, double* __restrict__ sc) {
    if (halt && *halt) return;
    const int j = threadIdx.x;
    if (j >= k) return;
    const double rn = sqrt(nrm[j]);
    sc[j] = rn > 0 ? 1.0 / rn : 1.0;
    sc[k + j] = rn > 0 ? rn : 1.0;
}

// K = [-G; I] (2k x k) for W <- X (-G) + W, G = (M X)^T W
__global__ void k_lob_projcoef(const int* __restrict__ halt, int k, const double* __restrict__ G, double* __restrict__ K) {
    if (halt && *halt) return;
    for (int t = threadIdx.x; t < 2 * k * k; t += blockDim.x) {
        const int a = t / k, b = t % k;
        K[t] = a < k ? -G[(size_t)a * k + b] : (a - k == b ? 1.0 : 0.0);
    }
}

// relative residuals |A x_j - lambda_j M x_j| / (|lambda_j| |M x_j|) of the wanted
// pairs against tol; `count` adds one iteration first (0 for the start block)
__global__ void k_lob_check(const double* __restrict__ nrm, const double* __restrict__ lam, LobState* st, int count) {
    if (threadIdx.x != 0 || st->ps.done) return;
    const int k = st->k;
    double worst = 0.0;
    bool finite = true;
    for (int j = 0; j < st->n_want; ++j) {
        const double rel = sqrt(nrm[j]) / (fabs(lam[j]) * sqrt(nrm[k + j]));
        if (!isfinite(rel)) finite = false;
        else worst = fmax(worst, rel);
    }
    st->iter += count;
    st->residual = finite ? worst : NAN;
    if (!finite) { st->ps.status = TSEM_NONFINITE; st->ps.done = 1; }
    else if (worst < st->tol) { st->ps.status = TSEM_OK; st->ps.done = 1; }
    else if (st->iter >= st->max_it) { st->ps.status = TSEM_MAXIT; st->ps.done = 1; }
}

// ------------------------------------------- K10: Rayleigh-Ritz on the device
// The small generalised eigenproblem of every iteration, (S^T A S) c = theta
// (S^T M S) c on the m basis columns, solved in FP64 by one CTA (LAPACKE_dsygvx in
// the reference, src/TSEMSolver.cpp:2179, 2349):
//   1. D = diag(GB)^(-1/2): GA' = D GA D, GB' = D GB D (residual directions shrink as
//      the iteration converges; unscaled they would fall under the rank threshold);
//   2. GB' = P L L^T P^T by Cholesky with diagonal pivoting, stopped at the numerical
//      rank r (remaining pivots <= 1e-13 of the largest diagonal entry): Q = P L^-T
//      is a GB'-orthonormal basis of r of the columns;
//   3. H = Q^T GA' Q = L^-1 GA'_pp L^-T by triangular solves, symmetrised;
//      H = Y diag(theta) Y^T by cyclic Jacobi, theta ascending;
//   4. C = D Q Y: the Ritz coefficients; the first k columns give X and P.
// The Jacobi sweeps use the round-robin (Brent-Luk) order: the rotations of a round
// touch disjoint index pairs and run in parallel; a sweep is (even) m - 1 rounds.
// FP64 runs at a small fraction of the FP32 rate on this GPU, so the one dense
// eigensolve is the Jacobi of H; the factorisation of GB' costs about m^3 / 3.
// The gram kernels fill the upper triangles of GA and GB (row stride m); C is m x k
// row-major, lam k values.
constexpr int kRRThreads = 512;
constexpr int kRRSweeps = 60;

// row stride of the shared m x m matrices: odd, so that a column's 8-byte entries
// fall in distinct banks
__host__ __device__ inline int rr_ld(int m) { return m | 1; }
size_t rr_smem_bytes(int m) {
    const int ld = rr_ld(m);
    return ((size_t)2 * ld * ld + 3 * (size_t)ld + 1) * sizeof(double) + 2 * (size_t)ld * sizeof(int);
}

// pair i of round t of the circle schedule on rr (even) players
__device__ __forceinline__ void rr_pair(int i, int t, int rr, int& p, int& q) {
    if (i == 0) { p = t; q = rr - 1; }
    else { p = (t + i) % (rr - 1); q = (t - i + rr - 1) % (rr - 1); }
}

// (hi, lo) pair arithmetic of the Jacobi rotations: c x - s y (minus) or s x + c y
// with every product's rounding error kept by FMA and the sum by TwoSum, then
// renormalised (Fast2Sum); about 2^-47 relative to the larger term
__device__ __forceinline__ float2 df_rot(float2 c, float2 x, float2 s, float2 y, bool minus) {
    const float p = __fmul_rn(c.x, x.x);
    float pe = __fmaf_rn(c.x, x.x, -p);
    pe = __fmaf_rn(c.x, x.y, pe);
    pe = __fmaf_rn(c.y, x.x, pe);
    float q = __fmul_rn(s.x, y.x);
    float qe = __fmaf_rn(s.x, y.x, -q);
    qe = __fmaf_rn(s.x, y.y, qe);
    qe = __fmaf_rn(s.y, y.x, qe);
    if (minus) { q = -q; qe = -qe; }
    const float sh = __fadd_rn(p, q);
    const float bb = __fsub_rn(sh, p);
    float se = __fadd_rn(__fsub_rn(p, __fsub_rn(sh, bb)), __fsub_rn(q, bb));
    se = __fadd_rn(se, __fadd_rn(pe, qe));
    const float hi = __fadd_rn(sh, se);
    return make_float2(hi, __fsub_rn(se, __fsub_rn(hi, sh)));
}
__device__ __forceinline__ double df_val(float2 a) { return (double)a.x + (double)a.y; }

// Jacobi rotations: a pair is rotated while |a_pq| > kJacobiRel sqrt|a_pp a_qq| (the
// relative test of Jacobi methods, which keeps the eigenvectors accurate however far
// apart the diagonal entries are).  The pair arithmetic carries about 2^-47 per
// operation, so the largest relative off-diagonal entry of a sweep falls
// quadratically to a rounding floor near 1e-13 and stays there; the sweeps end when
// a sweep rotates nothing, or when that largest entry is below kJacobiFloor and fell
// by less than a factor 4 in the last sweep (the floor is reached).
constexpr float kJacobiRel = 1e-14f;
constexpr float kJacobiFloor = 1e-10f;

// a (r x r in an ld-strided buffer of (hi, lo) pairs) -> diag(eigenvalues) in place;
// V eigenvectors (V[i ld + j] is component i of vector j), also pairs.  All threads
// of the block call it.  FP64 runs at a small fraction of the FP32 rate on this GPU
// and a sweep applies about 9 m^3 operations to a and V, so the rotations run on
// the FP32 pipe in pair arithmetic; a rotation's angle is found in FP32 (its
// accuracy only sets how far a_pq falls, the next sweep takes the rest) and its
// cosine and sine in FP64 from that angle, so that every rotation is orthogonal to
// the pairs' precision.  The sweeps stop after one that rotates nothing; rotations
// that are the identity cost nothing in the update phases.
__device__ int rr_jacobi(int r, int ld, float2* a, float2* V, float2* cs, int2* pq, int* nrot, unsigned* offmax) {
    const int tid = threadIdx.x, nt = blockDim.x;
    // update phases: 64 lanes over the columns (rows) of a pair, kRRThreads / 64 pairs at a time
    constexpr int kSlots = kRRThreads / 64;
    const int cl = tid & 63, slot = tid >> 6;
    float prev = 0.0f;
    const int rr = r + (r & 1), npair = rr / 2, nblk = npair * (npair + 1) / 2;
    for (int t = tid; t < r * r; t += nt)
        V[(t / r) * ld + t % r] = make_float2((t / r == t % r) ? 1.0f : 0.0f, 0.0f);
    __syncthreads();
    int sweeps = 0;
    for (int sweep = 0; sweep < kRRSweeps && r > 1; ++sweep) {
        if (tid == 0) { *nrot = 0; *offmax = 0u; }
        __syncthreads();
        ++sweeps;
        for (int round = 0; round < rr - 1; ++round) {
            // the rotations of the round: whole warps (npair <= 64), one shared atomic
            // per warp for the counts
            for (int i0 = 0; i0 < npair && tid < 64; i0 += 64) {
                const int i = i0 + tid;
                int p = 0, q = 0;
                unsigned offv = 0u;
                int rot = 0;
                float2 c2 = make_float2(1.0f, 0.0f), s2 = make_float2(0.0f, 0.0f);
                if (i < npair) rr_pair(i, round, rr, p, q);
                if (i < npair && p < r && q < r) {
                    const float2 apq = a[p * ld + q], app = a[p * ld + p], aqq = a[q * ld + q];
                    const float b = fabsf(apq.x), g = sqrtf(fabsf(app.x)) * sqrtf(fabsf(aqq.x));
                    if (b != 0.0f) offv = __float_as_uint(g > 0.0f ? fminf(b / g, 1.0f) : 1.0f);
                    if (b != 0.0f && b > kJacobiRel * g) {
                        const float dd = __fadd_rn(__fsub_rn(aqq.x, app.x), __fsub_rn(aqq.y, app.y));
                        const float tau = dd / (2.0f * apq.x);
                        const float at = fabsf(tau);
                        const float tt = at > 1e18f ? 0.5f / tau
                                                    : copysignf(1.0f, tau) / (at + sqrtf(__fmaf_rn(tau, tau, 1.0f)));
                        const double c = rsqrt(fma((double)tt, (double)tt, 1.0));
                        const double sn = (double)tt * c;
                        c2 = split2(c);
                        s2 = split2(sn);
                        rot = 1;
                    }
                }
                offv = __reduce_max_sync(0xffffffffu, offv);
                rot = __reduce_add_sync(0xffffffffu, rot);
                if ((tid & 31) == 0) {
                    if (offv) atomicMax(offmax, offv);
                    if (rot) atomicAdd(nrot, rot);
                }
                if (i < npair) {
                    cs[2 * i] = c2;
                    cs[2 * i + 1] = s2;
                    pq[i] = make_int2(p, q);
                }
            }
            __syncthreads();
            // The round's rotation is the direct sum of the pairs' 2 x 2 rotations, so
            // block (I, J) of the pairs' rows and columns becomes R_I^T A_IJ R_J: each
            // block I <= J is read, rotated on both sides and written with its transpose
            // by one thread (no block is read by another), and V's columns of every pair
            // are rotated beside it; one phase, one barrier.  Rows and columns at the
            // padding index r (odd r) do not exist; their pair never rotates.
            for (int t = tid; t < nblk; t += nt) {
                int J = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
                while (J * (J + 1) / 2 > t) --J;
                while ((J + 1) * (J + 2) / 2 <= t) ++J;
                const int I = t - J * (J + 1) / 2;
                const float2 sI = cs[2 * I + 1], sJ = cs[2 * J + 1];
                const bool rI = sI.x != 0.0f, rJ = sJ.x != 0.0f;
                if (!rI && !rJ) continue;
                const float2 cI = cs[2 * I], cJ = cs[2 * J];
                const int2 PI = pq[I], PJ = pq[J];
                const bool x0 = PI.x < r, x1 = PI.y < r, y0 = PJ.x < r, y1 = PJ.y < r;
                const float2 z = make_float2(0.0f, 0.0f);
                float2 e00 = x0 && y0 ? a[PI.x * ld + PJ.x] : z, e01 = x0 && y1 ? a[PI.x * ld + PJ.y] : z;
                float2 e10 = x1 && y0 ? a[PI.y * ld + PJ.x] : z, e11 = x1 && y1 ? a[PI.y * ld + PJ.y] : z;
                if (rI) {   // rows: R_I^T
                    const float2 t00 = df_rot(cI, e00, sI, e10, true), t10 = df_rot(sI, e00, cI, e10, false);
                    const float2 t01 = df_rot(cI, e01, sI, e11, true), t11 = df_rot(sI, e01, cI, e11, false);
                    e00 = t00; e10 = t10; e01 = t01; e11 = t11;
                }
                if (rJ) {   // columns: R_J
                    const float2 t00 = df_rot(cJ, e00, sJ, e01, true), t01 = df_rot(sJ, e00, cJ, e01, false);
                    const float2 t10 = df_rot(cJ, e10, sJ, e11, true), t11 = df_rot(sJ, e10, cJ, e11, false);
                    e00 = t00; e01 = t01; e10 = t10; e11 = t11;
                }
                if (I == J) {
                    if (x0) a[PI.x * ld + PI.x] = e00;
                    if (x1) a[PI.y * ld + PI.y] = e11;
                    if (x0 && x1) { a[PI.x * ld + PI.y] = e01; a[PI.y * ld + PI.x] = e01; }
                } else {
                    if (x0 && y0) { a[PI.x * ld + PJ.x] = e00; a[PJ.x * ld + PI.x] = e00; }
                    if (x0 && y1) { a[PI.x * ld + PJ.y] = e01; a[PJ.y * ld + PI.x] = e01; }
                    if (x1 && y0) { a[PI.y * ld + PJ.x] = e10; a[PJ.x * ld + PI.y] = e10; }
                    if (x1 && y1) { a[PI.y * ld + PJ.y] = e11; a[PJ.y * ld + PI.y] = e11; }
                }
            }
            for (int i = slot; i < npair; i += kSlots) {
                const float2 sn = cs[2 * i + 1];
                if (sn.x == 0.0f) continue;
                const float2 c = cs[2 * i];
                const int p = pq[i].x, q = pq[i].y;
                for (int row = cl; row < r; row += 64) {
                    const float2 vp = V[row * ld + p], vq = V[row * ld + q];
                    V[row * ld + p] = df_rot(c, vp, sn, vq, true);
                    V[row * ld + q] = df_rot(sn, vp, c, vq, false);
                }
            }
            __syncthreads();
        }
        // read after the round's last barrier: the same for every thread
        const float off = __uint_as_float(*offmax);
        if (*nrot == 0 || (off < kJacobiFloor && prev > 0.0f && off > 0.25f * prev)) break;
        prev = off;
        __syncthreads();         // before thread 0 resets the counts
    }
    __syncthreads();
    return sweeps;
}

// ascending order of the r values d: perm[rank] = index (ties by index)
__device__ void rr_sort(int r, const double* d, int* perm) {
    for (int i = threadIdx.x; i < r; i += blockDim.x) {
        int rank = 0;
        for (int j = 0; j < r; ++j) rank += (d[j] < d[i] || (d[j] == d[i] && j < i)) ? 1 : 0;
        perm[rank] = i;
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kRRThreads)
k_rayleigh_ritz(int m, int k, const double* __restrict__ GA, const double* __restrict__ GB, double* __restrict__ scr,
                double* __restrict__ C, double* __restrict__ lam, LobState* st) {
    if (st->ps.done) return;
    extern __shared__ double rs[];
    const int ld = rr_ld(m), tid = threadIdx.x, nt = blockDim.x;
    double* a = rs;
    double* V = a + (size_t)ld * ld;
    double* dsc = V + (size_t)ld * ld;
    double* d = dsc + ld;
    double* cs = d + ld;              // ld + 1 values: (c, s) of (ld + 1) / 2 rotations, as (hi, lo) pairs
    int* perm = reinterpret_cast<int*>(cs + ld + 1);
    int* keep = perm + ld;
    __shared__ int s_nrot, s_best, s_stop;
    __shared__ unsigned s_off;
    __shared__ int2 s_pq[(3 * kMaxBlock + 1) / 2 + 1];   // the round's index pairs
    __shared__ double s_rd[3 * kMaxBlock + 1];            // 1 / L_ii
    double* ga = scr;                           // D GA D, m x m
    double* Lg = scr + (size_t)m * m;           // the Cholesky factor, r x r (row stride m)
    double* T = scr + 2 * (size_t)m * m;        // L^-1 GA'_pp, r x r (row stride m)
    int* piv = keep;                            // basis column of pivot j
    // 1. scaled pencil; GB' into a
    for (int i = tid; i < m; i += nt) {
        const double g = GB[(size_t)i * m + i];
        dsc[i] = g > 0 ? 1.0 / sqrt(g) : 0.0;
        piv[i] = i;
    }
    __syncthreads();
    for (int t = tid; t < m * m; t += nt) {
        const int i = t / m, j = t % m;
        const size_t u = i <= j ? (size_t)i * m + j : (size_t)j * m + i;
        const double f = dsc[i] * dsc[j];
        a[i * ld + j] = GB[u] * f;
        ga[t] = GA[u] * f;
    }
    __syncthreads();
    // 2. pivoted Cholesky of GB' = P L L^T P^T, the largest remaining diagonal entry
    // first; it stops when that entry is at most 1e-13 of GB''s largest diagonal
    // entry: the columns left out lie in the span of the kept ones to that accuracy,
    // and the kept ones give Q = P L^-T, a GB'-orthonormal basis of r columns
    double dmax = 0.0;
    for (int i = 0; i < m; ++i) dmax = fmax(dmax, a[i * ld + i]);
    int r = m;
    for (int j = 0; j < m; ++j) {
        if (tid < 32) {
            // the largest remaining diagonal entry (ties: the first), one warp
            int best = -1;
            double bv = 0.0;
            for (int i = j + tid; i < m; i += 32) {
                const double v = a[i * ld + i];
                if (best < 0 || v > bv) { bv = v; best = i; }
            }
            for (int o = 16; o > 0; o >>= 1) {
                const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
                const int ob = __shfl_xor_sync(0xffffffffu, best, o);
                if (ob >= 0 && (best < 0 || ov > bv || (ov == bv && ob < best))) { bv = ov; best = ob; }
            }
            if (tid == 0) {
                s_best = best;
                s_stop = !(bv > 1e-13 * dmax) ? 1 : 0;
            }
        }
        __syncthreads();
        if (s_stop) { r = j; break; }
        const int best = s_best;
        if (best != j) {
            for (int t = tid; t < m; t += nt) {
                const double x = a[j * ld + t];
                a[j * ld + t] = a[best * ld + t];
                a[best * ld + t] = x;
            }
            __syncthreads();
            for (int t = tid; t < m; t += nt) {
                const double x = a[t * ld + j];
                a[t * ld + j] = a[t * ld + best];
                a[t * ld + best] = x;
            }
            if (tid == 0) {
                const int x = piv[j];
                piv[j] = piv[best];
                piv[best] = x;
            }
            __syncthreads();
        }
        const double ljj = sqrt(a[j * ld + j]);
        const double rj = 1.0 / ljj;
        for (int i = j + 1 + tid; i < m; i += nt) a[i * ld + j] *= rj;
        __syncthreads();
        if (tid == 0) a[j * ld + j] = ljj;
        const int rest = m - j - 1;
        for (int t = tid; t < rest * rest; t += nt) {
            const int i = j + 1 + t / rest, c = j + 1 + t % rest;
            a[i * ld + c] -= a[i * ld + j] * a[c * ld + j];
        }
        __syncthreads();
    }
    // L to global scratch (a is reused for H), 1 / L_ii to shared memory
    for (int t = tid; t < r * r; t += nt) {
        const int i = t / r, j = t % r;
        Lg[(size_t)i * m + j] = j <= i ? a[i * ld + j] : 0.0;
    }
    for (int i = tid; i < r; i += nt) s_rd[i] = 1.0 / a[i * ld + i];
    __syncthreads();
    // 3. H = L^-1 GA'_pp L^-T: T = L^-1 GA'_pp (a forward substitution per column),
    // then H^T = L^-1 T^T the same way; symmetrised.  A column is served by 8 lanes of
    // one warp, each summing every eighth term of a row's dot product (shuffle sum);
    // the row's result is visible to the column's lanes after __syncwarp.
    const int tg = tid >> 3, tl = tid & 7;
    for (int b0 = 0; b0 < r; b0 += nt / 8) {
        const int b = b0 + tg;
        const bool on = b < r;
        for (int i = 0; i < r; ++i) {
            double x = 0.0;
            if (on)
                for (int jj = tl; jj < i; jj += 8) x = fma(-Lg[(size_t)i * m + jj], T[(size_t)jj * m + b], x);
            x += __shfl_xor_sync(0xffffffffu, x, 1);
            x += __shfl_xor_sync(0xffffffffu, x, 2);
            x += __shfl_xor_sync(0xffffffffu, x, 4);
            if (on && tl == 0) T[(size_t)i * m + b] = (ga[(size_t)piv[i] * m + piv[b]] + x) * s_rd[i];
            __syncwarp();
        }
    }
    __syncthreads();
    for (int b0 = 0; b0 < r; b0 += nt / 8) {
        const int b = b0 + tg;
        const bool on = b < r;
        for (int i = 0; i < r; ++i) {
            double x = 0.0;
            if (on)
                for (int jj = tl; jj < i; jj += 8) x = fma(-Lg[(size_t)i * m + jj], a[jj * ld + b], x);
            x += __shfl_xor_sync(0xffffffffu, x, 1);
            x += __shfl_xor_sync(0xffffffffu, x, 2);
            x += __shfl_xor_sync(0xffffffffu, x, 4);
            if (on && tl == 0) a[i * ld + b] = (T[(size_t)b * m + i] + x) * s_rd[i];
            __syncwarp();
        }
    }
    __syncthreads();
    // symmetrised, then held as (hi, lo) pairs in place (one thread per entry: the
    // pair takes the double's 8 bytes)
    float2* a2 = reinterpret_cast<float2*>(a);
    float2* V2 = reinterpret_cast<float2*>(V);
    for (int t = tid; t < r * r; t += nt) {
        const int x = t / r, y = t % r;
        if (y < x) continue;
        const double h = y == x ? a[x * ld + x] : 0.5 * (a[x * ld + y] + a[y * ld + x]);
        a2[x * ld + y] = split2(h);
        a2[y * ld + x] = split2(h);
    }
    __syncthreads();
    // 4. H = Y diag(theta) Y^T; C = D P L^-T Y[:, first k] (a back substitution per
    // column), zero on the basis columns left out
    const int sweeps = rr_jacobi(r, ld, a2, V2, reinterpret_cast<float2*>(cs), s_pq, &s_nrot, &s_off);
    for (int i = tid; i < r; i += nt) d[i] = df_val(a2[i * ld + i]);
    __syncthreads();
    rr_sort(r, d, perm);
    const int kc = min(k, r);
    for (int t = tid; t < m * k; t += nt) C[t] = 0.0;
    __syncthreads();
    // back substitution, 8 lanes per column as above
    for (int j0 = 0; j0 < kc; j0 += nt / 8) {
        const int j = j0 + tg;
        const bool on = j < kc;
        for (int i = r - 1; i >= 0; --i) {
            double x = 0.0;
            if (on)
                for (int l = i + 1 + tl; l < r; l += 8) x = fma(-Lg[(size_t)l * m + i], T[(size_t)l * m + j], x);
            x += __shfl_xor_sync(0xffffffffu, x, 1);
            x += __shfl_xor_sync(0xffffffffu, x, 2);
            x += __shfl_xor_sync(0xffffffffu, x, 4);
            if (on && tl == 0) {
                const double z = (df_val(V2[i * ld + perm[j]]) + x) * s_rd[i];
                T[(size_t)i * m + j] = z;            // T's rows are free again: the back substitution's z
                C[(size_t)piv[i] * k + j] = z * dsc[piv[i]];
            }
            __syncwarp();
        }
    }
    for (int j = tid; j < kc; j += nt) lam[j] = d[perm[j]];
    __syncthreads();
    if (tid == 0) {
        st->rank = r;
        st->sweeps = max(st->sweeps, sweeps);
        bool finite = true;
        for (int j = 0; j < kc; ++j) finite = finite && isfinite(d[perm[j]]);
        if (!finite) { st->ps.status = TSEM_NONFINITE; st->ps.done = 1; }
        else if (r < k) { st->ps.status = TSEM_BREAKDOWN; st->ps.done = 1; }
    }
}

int nblk(int64_t n) { return grid_for(n, 256, 152 * 16); }

// the running LOBPCG's "done" flag on the device: every block kernel of an iteration
// returns at once when it is set (nullptr outside a LOBPCG call)
thread_local const int* t_halt = nullptr;

// dynamic shared memory beyond the 48 KB default: the Gram kernel (blocks of up to
// 3 x kMaxBlock columns) and the Rayleigh-Ritz kernel, once per device
void smem_limits() {
    static std::mutex mu;
    static std::vector<char> done;
    int dev = 0;
    TSEM_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    if ((int)done.size() <= dev) done.resize(dev + 1, 0);
    if (done[dev]) return;
    TSEM_CUDA(cudaFuncSetAttribute(k_gram<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)(2 * kGramRows * 2 * ((3 * kMaxBlock + 3) & ~3) * sizeof(float2))));
    TSEM_CUDA(cudaFuncSetAttribute(k_gram<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)(2 * kGramRows * 3 * ((3 * kMaxBlock + 3) & ~3) * sizeof(float2))));
    TSEM_CUDA(cudaFuncSetAttribute(k_rayleigh_ritz, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)rr_smem_bytes(3 * kMaxBlock)));
    done[dev] = 1;
}

// the lanes per row (log2) and the columns per lane of a block product with kc
// columns: about five columns a lane, every lane of a row busy
void spmm_shape(int kc, int& lsh, int& cpl) {
    const int want = (kc + 4) / 5;
    lsh = 0;
    while ((1 << lsh) < want) ++lsh;
    cpl = (kc + (1 << lsh) - 1) >> lsh;
}

template <int CPL>
void spmm_launch(int64_t n, int lsh, const DevCsr& A, const float2* vb, const float2* X, int ldx, int kc, float2* Ya,
                 float2* Yb, int ldy, cudaStream_t s) {
    const unsigned g = (unsigned)(((n << lsh) + 255) / 256);
    if (vb)
        k_spmm_split<CPL, true><<<g, 256, 0, s>>>(t_halt, n, lsh, A.rowptr.p, A.col.p, A.vsplit.p, vb, X, ldx, kc, Ya, Yb,
                                                  ldy);
    else
        k_spmm_split<CPL, false><<<g, 256, 0, s>>>(t_halt, n, lsh, A.rowptr.p, A.col.p, A.vsplit.p, nullptr, X, ldx, kc,
                                                   Ya, nullptr, ldy);
    TSEM_LAUNCHED();
}

// true when A and M have the same sparsity pattern (one comparison on the device)
bool same_pattern(const DevCsr& A, const DevCsr& M, cudaStream_t s) {
    if (A.n != M.n || A.nnz != M.nnz) return false;
    if (A.rowptr.p == M.rowptr.p && A.col.p == M.col.p) return true;
    DBuf<int> flag(1);
    flag.zero(s);
    k_pattern_diff<<<grid_for(A.nnz, 256, 152 * 8), 256, 0, s>>>(A.n, A.nnz, A.rowptr.p, M.rowptr.p, A.col.p, M.col.p,
                                                                flag.p);
    TSEM_LAUNCHED();
    int h = 1;
    flag.download(&h, 1, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    return h == 0;
}

// How A X and M X are formed together: one pass over a common pattern gathers each
// row of X once for both products.  kSame: A and M share a pattern; kAinM / kMinA:
// one pattern holds the other (the mass pattern holds the stiffness pattern in
// TSEM), and the smaller matrix's values are laid out on the larger pattern once
// per call; kApart: two passes.
struct PairPlan {
    enum Mode { kApart, kSame, kAinM, kMinA } mode = kApart;
    DBuf<float2> emb;   // the embedded values (kAinM, kMinA)
};

// the values of Q on P's pattern; false when Q has an entry outside it
bool embed_values(const DevCsr& P, const DevCsr& Q, DBuf<float2>& out, cudaStream_t s) {
    out.alloc(P.nnz);
    DBuf<int> flag(1);
    flag.zero(s);
    k_embed_values<<<grid_for(P.n, 256, 152 * 8), 256, 0, s>>>(P.n, P.rowptr.p, P.col.p, Q.rowptr.p, Q.col.p, Q.vsplit.p,
                                                            out.p, flag.p);
    TSEM_LAUNCHED();
    int h = 1;
    flag.download(&h, 1, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    if (h) out.release();
    return h == 0;
}

void plan_pair(const DevCsr& A, const DevCsr& M, PairPlan& plan, cudaStream_t s) {
    csr_split_values(A, s);
    csr_split_values(M, s);
    plan.mode = PairPlan::kApart;
    if (A.n != M.n) return;
    if (same_pattern(A, M, s)) plan.mode = PairPlan::kSame;
    else if (A.nnz <= M.nnz && embed_values(M, A, plan.emb, s)) plan.mode = PairPlan::kAinM;
    else if (M.nnz < A.nnz && embed_values(A, M, plan.emb, s)) plan.mode = PairPlan::kMinA;
}

// YA = A X and YM = M X on pair blocks (row strides ldx, ldy) with the matrices'
// (hi, lo) values (kept with each matrix), one pass over a common pattern where the
// plan has one
void spmm_pair(const DevCsr& A, const DevCsr& M, const PairPlan& plan, const float2* X, int ldx, int kc, float2* YA,
               float2* YM, int ldy, cudaStream_t s) {
    int lsh = 0, cpl = 1;
    spmm_shape(kc, lsh, cpl);
    auto run = [&](const DevCsr& P, const float2* vb, float2* Ya, float2* Yb) {
        switch (cpl) {
            case 1: spmm_launch<1>(A.n, lsh, P, vb, X, ldx, kc, Ya, Yb, ldy, s); break;
            case 2: spmm_launch<2>(A.n, lsh, P, vb, X, ldx, kc, Ya, Yb, ldy, s); break;
            case 3: spmm_launch<3>(A.n, lsh, P, vb, X, ldx, kc, Ya, Yb, ldy, s); break;
            case 4: spmm_launch<4>(A.n, lsh, P, vb, X, ldx, kc, Ya, Yb, ldy, s); break;
            default: spmm_launch<5>(A.n, lsh, P, vb, X, ldx, kc, Ya, Yb, ldy, s); break;
        }
    };
    switch (plan.mode) {
        case PairPlan::kSame: run(A, M.vsplit.p, YA, YM); break;
        case PairPlan::kAinM: run(M, plan.emb.p, YM, YA); break;
        case PairPlan::kMinA: run(A, plan.emb.p, YA, YM); break;
        default:
            run(A, nullptr, YA, nullptr);
            run(M, nullptr, YM, nullptr);
    }
}

// G1 = S^T T1 and (T2 set) G2 = S^T T2 of the first m columns (m x m, row stride m;
// with `upper` only the upper triangle), on the device
void gram(int64_t n, int m, const float2* S, const float2* T1, const float2* T2, int ld, double* G1, double* G2,
          bool upper, cudaStream_t s) {
    k_zero<<<1, 256, 0, s>>>(t_halt, (int64_t)m * m, G1);
    TSEM_LAUNCHED();
    if (T2) {
        k_zero<<<1, 256, 0, s>>>(t_halt, (int64_t)m * m, G2);
        TSEM_LAUNCHED();
    }
    const size_t shm = (size_t)2 * kGramRows * (T2 ? 3 : 2) * ((m + 3) & ~3) * sizeof(float2);
    const int blocks = (int)std::min<int64_t>(152 * 4, (n + kGramRows - 1) / kGramRows);
    if (T2)
        k_gram<true><<<std::max(blocks, 1), kGramThreads, shm, s>>>(t_halt, n, m, m, S, ld, T1, T2, ld, upper ? 1 : 0, G1, G2);
    else
        k_gram<false><<<std::max(blocks, 1), kGramThreads, shm, s>>>(t_halt, n, m, m, S, ld, T1, nullptr, ld, upper ? 1 : 0,
                                                                     G1, nullptr);
    TSEM_LAUNCHED();
}

// Y_z = S_z[:, a0 : a0 + m] C for the nb blocks (C m x kc row-major, on the device);
// with P, also P = S_0[:, a0 + c0 : a0 + m] C[c0 :, :]
void combo(int64_t n, int m, int kc, int nb, const float2* const* S, int lds, int a0, const double* C,
           float2* const* Y, int ldy, float2* P, int c0, cudaStream_t s) {
    int lsh = 0, cpl = 1;
    spmm_shape(kc, lsh, cpl);
    ComboBlocks b{};
    for (int z = 0; z < nb; ++z) { b.S[z] = S[z]; b.Y[z] = Y[z]; }
    const dim3 g((unsigned)(((n << lsh) + 255) / 256), (unsigned)nb);
    const size_t shm = (size_t)m * kc * sizeof(float2);
    switch (cpl) {
        case 1: k_combo<1><<<g, 256, shm, s>>>(t_halt, n, lsh, m, kc, lds, a0, C, b, ldy, P, c0); break;
        case 2: k_combo<2><<<g, 256, shm, s>>>(t_halt, n, lsh, m, kc, lds, a0, C, b, ldy, P, c0); break;
        case 3: k_combo<3><<<g, 256, shm, s>>>(t_halt, n, lsh, m, kc, lds, a0, C, b, ldy, P, c0); break;
        case 4: k_combo<4><<<g, 256, shm, s>>>(t_halt, n, lsh, m, kc, lds, a0, C, b, ldy, P, c0); break;
        default: k_combo<5><<<g, 256, shm, s>>>(t_halt, n, lsh, m, kc, lds, a0, C, b, ldy, P, c0); break;
    }
    TSEM_LAUNCHED();
}

// t_halt for the duration of one LOBPCG call
struct HaltScope {
    explicit HaltScope(const int* h) { t_halt = h; }
    ~HaltScope() { t_halt = nullptr; }
};

}  // namespace

LobpcgResult lobpcg(const DevCsr& A, const DevCsr& M, Solver* plain, MixedSolver* mixed, int k, int n_want, double* X,
                    double* lambda, double tol, int max_it, cudaStream_t s) {
    const int64_t n = A.n;
    if (M.n != n) throw Error(TSEM_INVALID, "A and M differ in size");
    if (k < 1 || k > kMaxBlock) throw Error(TSEM_INVALID, "block size must be 1.." + std::to_string(kMaxBlock));
    if (n_want < 1 || n_want > k) throw Error(TSEM_INVALID, "n_want must be 1..k");
    if (n < 3 * (int64_t)k) throw Error(TSEM_INVALID, "block too large for the problem");
    smem_limits();
    LobpcgResult res;
    cudaEvent_t e0, e1;
    TSEM_CUDA(cudaEventCreate(&e0));
    TSEM_CUDA(cudaEventCreate(&e1));
    TSEM_CUDA(cudaEventRecord(e0, s));
    const int ld = 3 * k, m = 3 * k;
    // the basis [X W P], A times it and M times it, and their successors: pair blocks
    DBuf<float2> S((size_t)n * ld), AS((size_t)n * ld), MS((size_t)n * ld);
    DBuf<float2> S2((size_t)n * ld), AS2((size_t)n * ld), MS2((size_t)n * ld);
    DBuf<double> GA((size_t)m * m), GB((size_t)m * m), G((size_t)k * k), dC((size_t)m * k), dlam(k), nrm(2 * k);
    DBuf<double> rr_scr((size_t)3 * m * m), dK((size_t)2 * k * k), bsc(2 * k), col(n);
    DBuf<float> cf, zf;
    DBuf<LobState> st(1);
    if (mixed) { cf.alloc((size_t)n * k); zf.alloc((size_t)n * k); }
    LobState h0{};
    h0.k = k;
    h0.n_want = n_want;
    h0.max_it = max_it;
    h0.tol = tol;
    st.upload(&h0, 1, s);
    const int* halt = &st.p->ps.done;
    const PcgScalars* halt_ps = &st.p->ps;
    const size_t rr_shm = rr_smem_bytes(m);

    // ---- the start block: P = 0, Rayleigh-Ritz on X alone, residual, test
    TSEM_CUDA(cudaMemsetAsync(S.p, 0, S.n * sizeof(float2), s));
    TSEM_CUDA(cudaMemsetAsync(AS.p, 0, AS.n * sizeof(float2), s));
    TSEM_CUDA(cudaMemsetAsync(MS.p, 0, MS.n * sizeof(float2), s));
    k_cm_to_rm<<<nblk(n * k), 256, 0, s>>>(n, k, X, S.p, ld);
    TSEM_LAUNCHED();
    PairPlan plan;
    plan_pair(A, M, plan, s);
    spmm_pair(A, M, plan, S.p, ld, k, AS.p, MS.p, ld, s);
    gram(n, k, S.p, AS.p, MS.p, ld, GA.p, GB.p, true, s);
    k_rayleigh_ritz<<<1, kRRThreads, rr_smem_bytes(k), s>>>(k, k, GA.p, GB.p, rr_scr.p, dC.p, dlam.p, st.p);
    TSEM_LAUNCHED();
    const float2* const blocks[3] = {S.p, AS.p, MS.p};
    float2* const blocks2[3] = {S2.p, AS2.p, MS2.p};
    combo(n, k, k, 3, blocks, ld, 0, dC.p, blocks2, ld, nullptr, 0, s);
    k_copy_cols<<<dim3((unsigned)nblk(n * k), 3), 256, 0, s>>>(nullptr, n, k, ld, 0, S2.p, S.p, AS2.p, AS.p, MS2.p, MS.p);
    TSEM_LAUNCHED();
    struct Blocks {
        float2 *S, *AS, *MS;
    };
    auto residual = [&](const Blocks& b, cudaStream_t c) {
        k_zero<<<1, 64, 0, c>>>(t_halt, 2 * k, nrm.p);
        TSEM_LAUNCHED();
        k_block_resid<<<nblk(n * 32), 256, 0, c>>>(t_halt, n, k, b.AS, b.MS, ld, dlam.p, b.S + k, ld, nrm.p);
        TSEM_LAUNCHED();
    };
    residual(Blocks{S.p, AS.p, MS.p}, s);
    k_lob_check<<<1, 32, 0, s>>>(nrm.p, dlam.p, st.p, 0);
    TSEM_LAUNCHED();
    LobState hs{};
    st.download(&hs, 1, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    if (hs.ps.done && hs.ps.status == TSEM_BREAKDOWN) throw Error(TSEM_INVALID, "initial block is rank deficient");

    if (!hs.ps.done) {
        HaltScope scope(halt);
        // one uncaptured V-cycle first: it allocates the work vectors the preconditioner
        // keeps (no allocation may happen while the iteration is captured)
        if (mixed) {
            TSEM_CUDA(cudaMemsetAsync(cf.p, 0, cf.n * sizeof(float), s));
            mixed->vcycle_graph(cf.p, zf.p, s, k);
        } else if (plain && plain->pmg) {
            TSEM_CUDA(cudaMemsetAsync(col.p, 0, col.n * sizeof(double), s));
            TSEM_CUDA(cudaMemsetAsync(plain->y.p, 0, (size_t)n * sizeof(double), s));
            plain->pmg->vcycle(plain->y.p, col.p, nullptr, s);
        }
        TSEM_CUDA(cudaStreamSynchronize(s));

        // ---- two iterations, captured as a graph
        cudaStream_t c = nullptr;
        cudaGraphExec_t exec = nullptr;
        TSEM_CUDA(cudaStreamCreateWithFlags(&c, cudaStreamNonBlocking));
        try {
            const long long k0 = g_kernel_launches.load();
            TSEM_CUDA(cudaStreamBeginCapture(c, cudaStreamCaptureModeThreadLocal));
            cudaGraph_t graph = nullptr;
            // one iteration from the basis in `cur` to the next one in `nxt` (the two sets of
            // blocks trade roles every iteration, so that X and P need no copy back)
            auto iteration = [&](const Blocks& cur, const Blocks& nxt) {
                // 1. W = preconditioned residual (the residual sits in the W columns)
                if (mixed) {
                    // the whole block in one V-cycle, each column scaled to unit norm in FP32
                    k_lob_scales<<<1, 64, 0, c>>>(t_halt, k, nrm.p, bsc.p);
                    TSEM_LAUNCHED();
                    const dim3 g((unsigned)nblk(n), (unsigned)k);
                    k_block_get_f32<<<g, 256, 0, c>>>(t_halt, n, k, cur.S + k, ld, bsc.p, cf.p);
                    TSEM_LAUNCHED();
                    mixed->vcycle(cf.p, zf.p, halt_ps, c, k);
                    k_block_put_f32<<<g, 256, 0, c>>>(t_halt, n, k, zf.p, bsc.p + k, cur.S + k, ld);
                    TSEM_LAUNCHED();
                } else {
                    for (int j = 0; j < k; ++j) {
                        float2* wj = cur.S + k + j;
                        k_col_get<<<nblk(n), 256, 0, c>>>(t_halt, n, wj, ld, col.p);
                        TSEM_LAUNCHED();
                        if (plain && plain->pmg) {
                            DBuf<double>& z = plain->y;   // scratch of the PCG, unused between solves
                            // the V-cycle (ite_PMG) works on z in place: from z = 0 it is one
                            // fixed linear preconditioner for every column
                            k_zero<<<nblk(n), 256, 0, c>>>(t_halt, n, z.p);
                            TSEM_LAUNCHED();
                            plain->pmg->vcycle(z.p, col.p, halt_ps, c);
                            k_col_put<<<nblk(n), 256, 0, c>>>(t_halt, n, z.p, wj, ld);
                        } else {
                            k_jacobi_col<<<nblk(n), 256, 0, c>>>(t_halt, n, A.diag.p, col.p);
                            TSEM_LAUNCHED();
                            k_col_put<<<nblk(n), 256, 0, c>>>(t_halt, n, col.p, wj, ld);
                        }
                        TSEM_LAUNCHED();
                    }
                }
                // 2. W <- W - X ((M X)^T W): the preconditioned residuals M-orthogonal to X
                // (M-orthonormal after the last Rayleigh-Ritz step), formed on the vectors
                // so that the Gram matrices need not resolve W's small part outside
                // span(X) next to its large part inside it; A W and M W from the new W
                gram(n, k, cur.MS, cur.S + k, nullptr, ld, G.p, nullptr, false, c);
                k_lob_projcoef<<<1, 256, 0, c>>>(t_halt, k, G.p, dK.p);
                TSEM_LAUNCHED();
                {
                    const float2* const src[1] = {cur.S};
                    float2* const dst[1] = {cur.S + k};   // in place: W is one of the combined columns
                    combo(n, 2 * k, k, 1, src, ld, 0, dK.p, dst, ld, nullptr, 0, c);
                }
                spmm_pair(A, M, plan, cur.S + k, ld, k, cur.AS + k, cur.MS + k, ld, c);
                // 3. Gram matrices of the 3k columns [X W P] (P = 0 in the first
                // iteration: its directions fall out at the rank test), Rayleigh-Ritz
                gram(n, m, cur.S, cur.AS, cur.MS, ld, GA.p, GB.p, true, c);
                k_rayleigh_ritz<<<1, kRRThreads, rr_shm, c>>>(m, k, GA.p, GB.p, rr_scr.p, dC.p, dlam.p, st.p);
                TSEM_LAUNCHED();
                // 4. Ritz update: X = S C, P = S[:, k:] C[k:, :].  A P and M P come from P
                // itself: combined like P they would lose their relative accuracy when P
                // is small, and the next Gram matrices would no longer describe the same
                // vectors
                {
                    const float2* const from[3] = {cur.S, cur.AS, cur.MS};
                    float2* const to[3] = {nxt.S, nxt.AS, nxt.MS};
                    combo(n, m, k, 3, from, ld, 0, dC.p, to, ld, nxt.S + 2 * k, k, c);
                }
                spmm_pair(A, M, plan, nxt.S + 2 * k, ld, k, nxt.AS + 2 * k, nxt.MS + 2 * k, ld, c);
                // 5. residual (into the next basis's W columns) and test
                residual(nxt, c);
                k_lob_check<<<1, 32, 0, c>>>(nrm.p, dlam.p, st.p, 1);
                TSEM_LAUNCHED();
            };
            try {
                iteration(Blocks{S.p, AS.p, MS.p}, Blocks{S2.p, AS2.p, MS2.p});
                iteration(Blocks{S2.p, AS2.p, MS2.p}, Blocks{S.p, AS.p, MS.p});
            } catch (...) {
                cudaStreamEndCapture(c, &graph);
                if (graph) cudaGraphDestroy(graph);
                throw;
            }
            TSEM_CUDA(cudaStreamEndCapture(c, &graph));
            const long long body_kernels = g_kernel_launches.load() - k0;
            g_kernel_launches.fetch_sub(body_kernels);   // counted when replayed
            const cudaError_t irc = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            TSEM_CUDA(irc);
            // replays in chunks: the host reads the state once per chunk, never per
            // iteration; replays after the test has passed return at once.  The device
            // stops at max_it; the host bound only guards against a state that never
            // reports
            constexpr int kChunk = 4;
            long long replays = 0;
            for (;;) {
                st.download(&hs, 1, s);
                TSEM_CUDA(cudaStreamSynchronize(s));
                if (hs.ps.done || replays > (long long)max_it + kChunk) break;
                for (int r = 0; r < kChunk; ++r) {
                    TSEM_CUDA(cudaGraphLaunch(exec, s));
                    g_kernel_launches.fetch_add(body_kernels);
                    ++replays;
                }
            }
        } catch (...) {
            if (exec) cudaGraphExecDestroy(exec);
            cudaStreamSynchronize(s);
            cudaStreamDestroy(c);
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            throw;
        }
        cudaGraphExecDestroy(exec);
        cudaStreamDestroy(c);
    }
    res.iterations = hs.iter;
    res.jacobi_sweeps = hs.sweeps;
    res.status = hs.ps.done ? hs.ps.status : TSEM_MAXIT;
    res.residual = hs.residual;
    // iteration j reads the blocks it wrote in iteration j - 1: after an odd number of
    // completed iterations the current basis is the second set (an iteration stopped
    // inside, by the Rayleigh-Ritz step, writes nothing and counts nothing)
    k_rm_to_cm<<<nblk(n * k), 256, 0, s>>>(n, k, (hs.iter & 1) ? S2.p : S.p, ld, X);
    TSEM_LAUNCHED();
    TSEM_CUDA(cudaEventRecord(e1, s));
    TSEM_CUDA(cudaEventSynchronize(e1));
    dlam.download(lambda, k, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    TSEM_CUDA(cudaEventElapsedTime(&res.device_ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (mixed) {
        int herr = 0;
        mixed->op.err.download(&herr, 1, s);
        TSEM_CUDA(cudaStreamSynchronize(s));
        if (herr) {
            mixed->op.err.zero(s);
            throw Error(TSEM_TIMEOUT, "a bounded wait of the matrix-free apply gave up (code " + std::to_string(herr) + ")");
        }
    }
    return res;
}

}  // namespace tsem
