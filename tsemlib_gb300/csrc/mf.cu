// Matrix-free TSEM operator and the mixed-precision solver.
//
// The stiffness operator with Dirichlet rows eliminated is applied per element,
//     y = sum_e T_e^T [ sum_k w_{e,k} S_k ] T_e x ,   w_{e,k} = 2/(3|T_e|) G_{e,k},
// which is TSEMLib's element stiffness (src/Discretize.cpp:1352-1393) without
// forming the global matrix.  Level q of the p-multigrid hierarchy uses the
// leading block of the reference matrices (modes |alpha| <= q, which the
// hierarchical basis orders first), and equals the principal submatrix
// {sum_dof <= q} of init_PMG (src/TSEMSolver.cpp:573-656).
//
// Solver: FP64 iterative refinement around an FP32 PCG whose operator and
// p-multigrid (Chebyshev-Jacobi smoothing) are matrix-free; the outer residual
// r = b - A x uses the FP64 CSR operator.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_bf16.h>

#include "check.cuh"
#include "mf.hpp"
#include "ptx.cuh"

namespace tsem {

constexpr int kTileE = 64;      // elements per tile of the FP32 apply kernel
constexpr int kTileT = 128;     // elements per tile of the tensor-core apply kernel (MMA M)
constexpr int kApplyThreads = 512;

// n rounded up to an odd multiple of q: strides of the [mode][element] arrays that
// are not multiples of large powers of two, so that rows of one element column do
// not all fall into the same memory partition
static int odd_multiple(int n, int q) {
    int m = (n + q - 1) / q;
    if (m % 2 == 0) ++m;
    return m * q;
}
// element count of the per-element results V[e][i]: whole tiles of the larger tile size
static int v_stride(int E) { return odd_multiple(E, kTileT); }

// ------------------------------------------------------------------ gathers
// U32[tile][j][kTileE]: local coefficients of every element, FP32, the layout the
// CUDA-core GEMM reads.  Elements past E are zero.
__global__ void k_gather_f32(int E, int E_pad, int nl, int md, const int* __restrict__ gi, const float* __restrict__ gv,
                             const float* __restrict__ x, int64_t nx, float* __restrict__ U) {
    const int64_t total = (int64_t)E_pad * nl;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int e = (int)(t % E_pad), j = (int)(t / E_pad);
        float u = 0.0f;
        if (e < E)
            for (int q = 0; q < md; ++q) {
                const size_t o = ((size_t)j * md + q) * E + e;
                const int g = gi[o];
                if (g >= 0 && in_bounds(g, nx, 31)) u += gv[o] * __ldg(x + g);
            }
        U[((size_t)(e / kTileE) * nl + j) * kTileE + (e % kTileE)] = u;
    }
}

// Levels whose transform has one term per local mode with coefficient 0 or +-1 keep
// a packed index instead of (gi, gv): p >= 0 reads +x[p], p == -1 gives 0 and
// p <= -2 reads -x[-p - 2].
__device__ __forceinline__ float unit_load(int p, const float* __restrict__ x, int64_t nx) {
#ifdef TSEM_CHECK
    if (p == -1) return 0.0f;
    const int g = p >= 0 ? p : -p - 2;
    if (!in_bounds(g, nx, 32)) return 0.0f;
    const float v = __ldg(x + g);
    return p >= 0 ? v : -v;
#else
    // selects, no branches: the gathers keep all their loads in flight
    (void)nx;
    return p >= 0 ? __ldg(x + p) : (p == -1 ? 0.0f : -__ldg(x + (-p - 2)));
#endif
}

__global__ void k_gather_f32_unit(int E, int E_pad, int nl, const int* __restrict__ gp, const float* __restrict__ x,
                                  int64_t nx, float* __restrict__ U) {
    const int64_t total = (int64_t)E_pad * nl;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int e = (int)(t % E_pad), j = (int)(t / E_pad);
        const float u = e < E ? unit_load(gp[(size_t)j * E + e], x, nx) : 0.0f;
        U[((size_t)(e / kTileE) * nl + j) * kTileE + (e % kTileE)] = u;
    }
}

// U16: BF16 tiles of kTileT elements in the no-swizzle K-major core-matrix layout
// (8 rows x 8 BF16 per 128-byte core matrix; K-adjacent core matrices 128 B apart,
// M-adjacent ones kpad/8 * 128 B apart).  One thread writes one 16-byte core row.
__global__ void k_gather_bf16(int E, int E_pad, int nl, int kpad, int md, const int* __restrict__ gi,
                              const float* __restrict__ gv, const float* __restrict__ x, int64_t nx,
                              uint4* __restrict__ U) {
    const int kb = kpad / 8;
    const int64_t total = (int64_t)E_pad * kb;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int e = (int)(t % E_pad), jb = (int)(t / E_pad);
        float v[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            const int j = jb * 8 + c;
            float u = 0.0f;
            if (e < E && j < nl)
                for (int q = 0; q < md; ++q) {
                    const size_t o = ((size_t)j * md + q) * E + e;
                    const int g = gi[o];
                    if (g >= 0 && in_bounds(g, nx, 33)) u += gv[o] * __ldg(x + g);
                }
            v[c] = u;
        }
        uint4 w;
        w.x = (uint32_t)__bfloat16_as_ushort(__float2bfloat16(v[0])) | ((uint32_t)__bfloat16_as_ushort(__float2bfloat16(v[1])) << 16);
        w.y = (uint32_t)__bfloat16_as_ushort(__float2bfloat16(v[2])) | ((uint32_t)__bfloat16_as_ushort(__float2bfloat16(v[3])) << 16);
        w.z = (uint32_t)__bfloat16_as_ushort(__float2bfloat16(v[4])) | ((uint32_t)__bfloat16_as_ushort(__float2bfloat16(v[5])) << 16);
        w.w = (uint32_t)__bfloat16_as_ushort(__float2bfloat16(v[6])) | ((uint32_t)__bfloat16_as_ushort(__float2bfloat16(v[7])) << 16);
        const int tile = e / kTileT, m = e % kTileT;
        // 16-byte units: core matrix (m/8, jb) holds 8 rows of 16 bytes
        const size_t unit = (size_t)tile * (kTileT / 8) * kb * 8 + ((size_t)(m / 8) * kb + jb) * 8 + (m % 8);
        U[unit] = w;
    }
}

// ------------------------------------------------- FP32 CUDA-core apply kernel
// Persistent register-tiled GEMM per element tile:  Z[e][(i,k)] = sum_j U[e][j] S_k[i][j],
// y_e[i] = sum_k w_{e,k} Z[e][(i,k)], scattered through the transform.  The stacked
// reference matrices of a block of rows stay in shared memory (layout [j][i][k]:
// the 6 matrices of two rows are 12 consecutive floats); element tiles arrive by
// double-buffered bulk copies from U32.  Each thread owns a 4-element x 2-row x
// 6-matrix micro-tile (48 accumulators).
// Global layouts: gi/gv [nl][md][E], w6 [6][E], S [6][nl][nlp].
__global__ void __launch_bounds__(kApplyThreads, 1)
k_mf_apply(int E, int nl, int nlp, int md, int row_beg, int row_cnt, const int* __restrict__ gi,
           const float* __restrict__ gv, const float* __restrict__ w6, const float* __restrict__ S,
           const float* __restrict__ U32, float* __restrict__ V, int se, int si, int* err) {
    extern __shared__ float4 smem4[];
    float* sm = reinterpret_cast<float*>(smem4);
    const int rows2 = (row_cnt + 1) & ~1;
    const size_t tile_floats = (size_t)nl * kTileE;
    float* Ub[2] = {sm, sm + tile_floats};                  // double-buffered tiles [j][kTileE]
    float* Ss = sm + 2 * tile_floats;                       // [nl][rows2][6]
    __shared__ __align__(8) uint64_t full[2];
    const int n_tiles = (E + kTileE - 1) / kTileE;
    const uint32_t bytes = (uint32_t)(tile_floats * sizeof(float));
    if (threadIdx.x == 0) {
        mbar_init(&full[0], 1);
        mbar_init(&full[1], 1);
        fence_mbar_init();
        if ((int)blockIdx.x < n_tiles) {
            mbar_expect_tx(&full[0], bytes);
            bulk_g2s(Ub[0], U32 + (size_t)blockIdx.x * tile_floats, bytes, &full[0]);
        }
    }
    for (int idx = threadIdx.x; idx < nl * rows2 * 6; idx += blockDim.x) {
        const int k = idx % 6, r = (idx / 6) % rows2, j = idx / (6 * rows2);
        const int i = row_beg + r;
        Ss[idx] = (r < row_cnt) ? S[((size_t)k * nl + i) * nlp + j] : 0.0f;
    }
    const int n_micro = (kTileE / 4) * (rows2 / 2);
    int it = 0;
    for (int tile = blockIdx.x; tile < n_tiles; tile += gridDim.x, ++it) {
        const int b = it & 1;
        __syncthreads();                                    // all threads are done with tile it-1
        if (threadIdx.x == 0 && tile + (int)gridDim.x < n_tiles) {
            mbar_expect_tx(&full[b ^ 1], bytes);
            bulk_g2s(Ub[b ^ 1], U32 + (size_t)(tile + gridDim.x) * tile_floats, bytes, &full[b ^ 1]);
        }
        // block-uniform decision: every thread takes the same path out of the loop
        const int ok = __syncthreads_and(mbar_wait_bounded(&full[b], (uint32_t)((it >> 1) & 1), err, 1));
        if (!ok) {
            // the copies this block issued (this tile's and the prefetch) land before it exits
            if (threadIdx.x == 0) {
                mbar_wait_bounded(&full[b], (uint32_t)((it >> 1) & 1), err, 1, 1ll << 26, true);
                if (tile + (int)gridDim.x < n_tiles)
                    mbar_wait_bounded(&full[b ^ 1], (uint32_t)(((it + 1) >> 1) & 1), err, 1, 1ll << 26, true);
            }
            break;
        }
        const float* Us = Ub[b];
        const int e0 = tile * kTileE;
        for (int mt = threadIdx.x; mt < n_micro; mt += blockDim.x) {
            const int eg = mt % (kTileE / 4), rp = mt / (kTileE / 4);
            float acc[4][12];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int c = 0; c < 12; ++c) acc[a][c] = 0.0f;
            const float* up = Us + eg * 4;
            const float* sp = Ss + rp * 12;
            for (int j = 0; j < nl; ++j) {
                const float4 u = *reinterpret_cast<const float4*>(up + (size_t)j * kTileE);
                const float4 s0 = *reinterpret_cast<const float4*>(sp + (size_t)j * rows2 * 6);
                const float4 s1 = *reinterpret_cast<const float4*>(sp + (size_t)j * rows2 * 6 + 4);
                const float4 s2 = *reinterpret_cast<const float4*>(sp + (size_t)j * rows2 * 6 + 8);
                const float sv[12] = {s0.x, s0.y, s0.z, s0.w, s1.x, s1.y, s1.z, s1.w, s2.x, s2.y, s2.z, s2.w};
                const float uv[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int c = 0; c < 12; ++c) acc[a][c] += uv[a] * sv[c];
            }
            // combine the six matrices with the element weights: V[e * se + i * si] (scattered later)
            float w[4][6];
#pragma unroll
            for (int a = 0; a < 4; ++a) {
                const int e = e0 + eg * 4 + a;
#pragma unroll
                for (int k = 0; k < 6; ++k) w[a][k] = e < E ? __ldg(w6 + (size_t)k * E + e) : 0.0f;
            }
#pragma unroll
            for (int rr = 0; rr < 2; ++rr) {
                const int r = rp * 2 + rr;
                if (r >= row_cnt) continue;
                float v[4];
#pragma unroll
                for (int a = 0; a < 4; ++a) {
                    float t = 0.0f;
#pragma unroll
                    for (int k = 0; k < 6; ++k) t += w[a][k] * acc[a][rr * 6 + k];
                    v[a] = t;
                }
                if (se == 1) {
                    *reinterpret_cast<float4*>(V + (size_t)(row_beg + r) * si + e0 + eg * 4) = make_float4(v[0], v[1], v[2], v[3]);
                } else {
#pragma unroll
                    for (int a = 0; a < 4; ++a) V[(size_t)(e0 + eg * 4 + a) * se + (size_t)(row_beg + r) * si] = v[a];
                }
            }
        }
    }
}

// y[g] += t * V[i][e] over the transform terms of every (element, mode)
__global__ void k_scatter(int E, int E_pad, int nl, int md, const int* __restrict__ gi, const float* __restrict__ gv,
                          const float* __restrict__ V, float* __restrict__ y, int64_t ny) {
    const int64_t total = (int64_t)E * nl;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int e = (int)(t % E), i = (int)(t / E);
        const float v = V[(size_t)i * E_pad + e];
        for (int q = 0; q < md; ++q) {
            const size_t o = ((size_t)i * md + q) * E + e;
            const int g = gi[o];
            const float c = gv[o];
            if (g >= 0 && c != 0.0f && in_bounds(g, ny, 34)) atomicAdd(y + g, c * v);
        }
    }
}

// y[g] = sum over the (element, mode) results that DOF g receives, read through the
// transposed transform (row g lists positions e * epi_stride(nl) + i of the
// element-major results, a negative entry ~pos
// for coefficient -1 on unit levels, else with coefficient tval); a DOF that
// receives nothing is a Dirichlet DOF: y[g] = d_g x[g].  No atomics: each DOF is
// written once, and the result does not depend on the launch.
//
// The Chebyshev smoother's vector updates are fused into this pass (MODE):
//   MfPost::kStore      y = A x
//   MfPost::kChebFirst  v = rhs - A x,  d = s dinv v,  x += d         (x updated in place)
//   MfPost::kChebStep   v -= A d,  d = a d + c dinv v,  xs += d       (d is the applied vector)
//   MfPost::kResid      v = rhs - A x
// Each DOF's entries are read and written by one thread only, so the in-place
// updates of the applied vector are safe.
template <bool UNIT>
__device__ __forceinline__ float scatter_row(int b, int e, const int* __restrict__ pos, const float* __restrict__ tval,
                                             const float* __restrict__ V, int64_t nv) {
    // the first four entries (most DOFs have at most four): positions first, then values
    int p[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) p[u] = b + u < e ? pos[b + u] : INT_MIN;
    float t[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        float r = 0.0f;
        if (p[u] != INT_MIN) {
#ifdef TSEM_CHECK
            const int q = UNIT && p[u] < 0 ? ~p[u] : p[u];
            if (in_bounds(q, nv, 35)) {
                if (UNIT) r = p[u] >= 0 ? V[q] : -V[q];
                else r = tval[b + u] * V[q];
            }
#else
            if (UNIT) r = p[u] >= 0 ? V[p[u]] : -V[~p[u]];
            else r = tval[b + u] * V[p[u]];
#endif
        }
        t[u] = r;
    }
    float acc = ((t[0] + t[1]) + t[2]) + t[3];
    for (int k = b + 4; k < e; ++k) {
        const int q = pos[k];
#ifdef TSEM_CHECK
        const int qq = UNIT && q < 0 ? ~q : q;
        if (!in_bounds(qq, nv, 35)) continue;
        if (UNIT) acc += q >= 0 ? V[qq] : -V[qq];
        else acc += tval[k] * V[qq];
#else
        (void)nv;
        if (UNIT) acc += q >= 0 ? V[q] : -V[~q];
        else acc += tval[k] * V[q];
#endif
    }
    return acc;
}

// Block V-cycles run one column per blockIdx.y: the column's vectors are `off`
// further on (the inverse diagonal is shared)
__device__ __forceinline__ MfPost col_post(const MfPost& po, int64_t off) {
    MfPost q = po;
    if (off) {
        if (q.y) q.y += off;
        if (q.rhs) q.rhs += off;
        if (q.v) q.v += off;
        if (q.d) q.d += off;
        if (q.xs) q.xs += off;
    }
    return q;
}

template <int MODE>
__device__ __forceinline__ void scatter_post(int64_t g, float acc, float* x, const MfPost& po) {
    if (MODE == MfPost::kStore) {
        po.y[g] = acc;
    } else if (MODE == MfPost::kResid) {
        po.v[g] = po.rhs[g] - acc;
    } else if (MODE == MfPost::kChebFirst) {
        const float v = po.rhs[g] - acc;
        po.v[g] = v;
        const float d = po.dinv[g] * v * po.a;
        po.d[g] = d;
        x[g] += d;
    } else {
        const float v = po.v[g] - acc;
        po.v[g] = v;
        const float d = po.a * x[g] + po.c * po.dinv[g] * v;
        x[g] = d;
        po.xs[g] += d;
    }
}

template <bool UNIT, int MODE>
__global__ void k_scatter_t(int64_t n, const int* __restrict__ rp, const int* __restrict__ pos,
                            const float* __restrict__ tval, const float* __restrict__ V,
                            const float* __restrict__ bdiag, float* x, MfPost po0, int64_t vcol) {
    if (MODE != MfPost::kStore && po0.st && po0.st->done) return;
    // column blockIdx.y of a block apply
    const MfPost po = col_post(po0, (int64_t)blockIdx.y * n);
    x += (int64_t)blockIdx.y * n;
    V += (int64_t)blockIdx.y * vcol;
    // two DOFs per thread and step (g and g + stride) so that their load chains overlap
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < n; g += 2 * stride) {
        const int64_t g2 = g + stride;
        const bool two = g2 < n;
        const int b1 = rp[g], e1 = rp[g + 1];
        const int b2 = two ? rp[g2] : 0, e2 = two ? rp[g2 + 1] : 0;
        float a1 = b1 == e1 ? bdiag[g] * x[g] : scatter_row<UNIT>(b1, e1, pos, tval, V, vcol);
        float a2 = 0.0f;
        if (two) a2 = b2 == e2 ? bdiag[g2] * x[g2] : scatter_row<UNIT>(b2, e2, pos, tval, V, vcol);
        scatter_post<MODE>(g, a1, x, po);
        if (two) scatter_post<MODE>(g2, a2, x, po);
    }
}

// ------------------------------------- epilogue of the tensor-core apply kernels
// Per-element results are element-major, V[e][i] with the odd row stride
// epi_stride(nl): the DOFs a scatter thread and its neighbours sum are mostly
// neighbouring modes of the same elements, so their entries share sectors.  A thread
// owns one element (its TMEM lane) and writes its rows into a staging tile with the
// tile's global layout (the odd stride puts the lanes of a warp on distinct banks);
// one thread then stores the whole tile with a bulk copy.
__host__ __device__ constexpr int epi_stride(int nl) { return nl | 1; }
static size_t epi_bytes(int nl) { return (size_t)kTileT * epi_stride(nl) * sizeof(float); }

// rows i = i_first, i_first + i_step, ... (blocks of 4) of y_e = sum_k w_k D[k nl4 + i]
__device__ __forceinline__ void epi_combine(uint32_t tl, int nl, int nl4, int i_first, int i_step, const float (&w)[6],
                                            float* srow) {
    for (int i0 = i_first; i0 < nl; i0 += i_step) {
        float v[6][4];
#pragma unroll
        for (int k = 0; k < 6; ++k) tmem_ld4(tl + (uint32_t)(k * nl4 + i0), v[k][0], v[k][1], v[k][2], v[k][3]);
        tmem_ld_wait();
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int i = i0 + r;
            if (i >= nl) break;
            float acc = 0.0f;
#pragma unroll
            for (int k = 0; k < 6; ++k) acc += w[k] * v[k][r];
            srow[i] = acc;
        }
    }
}

// ------------------------------------------------- tcgen05 BF16 apply kernel
// D[e][n] = sum_j U[e][j] B[n][j] with B the stacked reference matrices, row
// n = k*nl4 + i.  M = 128 elements per tile, N = 2 x 256 accumulator columns (the
// whole 512-column tensor memory), K = kpad.  One CTA per SM: thread 0 issues the
// bulk copies and the MMAs, all four warps read their 32 lanes of tensor memory,
// combine the six matrices with the element weights and scatter.
constexpr int kTcThreads = 512;   // four warps per tensor-memory lane quarter
constexpr int kTcGroups = kTcThreads / 128;

__global__ void __launch_bounds__(kTcThreads, 1)
k_mf_apply_tc(int E, int nl, int nl4, int kpad, int md, const int* __restrict__ gi, const float* __restrict__ gv,
              const float* __restrict__ w6, const uint16_t* __restrict__ Bg, const uint16_t* __restrict__ U16,
              float* __restrict__ V, int* err) {
    extern __shared__ float4 smem4[];
    uint8_t* sm = reinterpret_cast<uint8_t*>(smem4);
    const uint32_t b_bytes = 512u * (uint32_t)kpad * 2u;
    const uint32_t a_bytes = (uint32_t)kTileT * (uint32_t)kpad * 2u;
    uint8_t* Bs = sm;
    uint8_t* Ab[2] = {sm + b_bytes, sm + b_bytes + a_bytes};
    float* St = reinterpret_cast<float*>(sm + b_bytes + 2 * a_bytes);
    __shared__ __align__(8) uint64_t full[2];
    __shared__ __align__(8) uint64_t bfull, mma_done, drain;
    __shared__ uint32_t tmem_slot;
    const int n_tiles = (E + kTileT - 1) / kTileT;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // thread 0's count of the tile copies issued into / landed in each buffer: on a
    // give-up it waits for the ones still in flight before the block exits
    int issued[2] = {0, 0}, landed[2] = {0, 0};
    if (threadIdx.x == 0) {
        mbar_init(&full[0], 1);
        mbar_init(&full[1], 1);
        mbar_init(&bfull, 1);
        mbar_init(&mma_done, 1);
        mbar_init(&drain, 1);
        fence_mbar_init();
        mbar_expect_tx(&bfull, b_bytes);
        bulk_g2s(Bs, Bg, b_bytes, &bfull);
        if ((int)blockIdx.x < n_tiles) {
            mbar_expect_tx(&full[0], a_bytes);
            bulk_g2s(Ab[0], U16 + (size_t)blockIdx.x * (a_bytes / 2), a_bytes, &full[0]);
            issued[0] = 1;
        }
    }
    if (warp == 0) {
        tmem_alloc(&tmem_slot, 512);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const bool b_landed = mbar_wait_bounded(&bfull, 0, err, 2);
    int ok = __syncthreads_and(b_landed);
    const uint32_t lbo = 128, sbo = (uint32_t)(kpad / 8) * 128u;
    const uint32_t idesc = idesc_bf16(128, 256);
    int it = 0;
    for (int tile = blockIdx.x; ok && tile < n_tiles; tile += gridDim.x, ++it) {
        const int b = it & 1;
        if (threadIdx.x == 0) {
            if (tile + (int)gridDim.x < n_tiles) {
                mbar_expect_tx(&full[b ^ 1], a_bytes);
                bulk_g2s(Ab[b ^ 1], U16 + (size_t)(tile + gridDim.x) * (a_bytes / 2), a_bytes, &full[b ^ 1]);
                ++issued[b ^ 1];
            }
            if (mbar_wait_bounded(&full[b], (uint32_t)((it >> 1) & 1), err, 3)) {
                ++landed[b];
                tc_fence_after();
                const uint32_t a0 = smem_u32(Ab[b]), b0 = smem_u32(Bs);
                for (int c = 0; c < 2; ++c)
                    for (int s = 0; s < kpad / 16; ++s) {
                        const uint64_t ad = smem_desc(a0 + (uint32_t)s * 2u * lbo, lbo, sbo);
                        const uint64_t bd = smem_desc(b0 + (uint32_t)c * 32u * sbo + (uint32_t)s * 2u * lbo, lbo, sbo);
                        mma_bf16(tmem + (uint32_t)c * 256u, ad, bd, idesc, s > 0 ? 1u : 0u);
                    }
                mma_commit(&mma_done);
            }
        }
        ok = __syncthreads_and(mbar_wait_bounded(&mma_done, (uint32_t)(it & 1), err, 4));
        tc_fence_after();
        if (ok) {
            // warp -> lane quarter (warp % 4) and every kTcGroups-th block of 4 rows (warp / 4)
            const int quarter = warp & 3, group = warp >> 2;
            const int el = quarter * 32 + lane, e = tile * kTileT + el;
            float w[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) w[k] = e < E ? __ldg(w6 + (size_t)k * E + e) : 0.0f;
            const uint32_t tl = tmem + ((uint32_t)(quarter * 32) << 16);
            epi_combine(tl, nl, nl4, 4 * group, 4 * kTcGroups, w, St + el * epi_stride(nl));
        }
        fence_proxy_async();     // the staging tile is read by the bulk copy
        tc_fence_before();
        __syncthreads();
        if (ok && threadIdx.x == 0) {
            const uint32_t tb = (uint32_t)kTileT * epi_stride(nl) * 4u;
            bulk_s2g(V + (size_t)tile * kTileT * epi_stride(nl), St, tb);
            bulk_wait_read();    // the next tile rewrites the staging tile after the barrier that opens it
        }
    }
    if (threadIdx.x == 0) {
        // after a give-up: the weight copy, the tile copies still in flight (at most one
        // per buffer) and every MMA issued finish before the tensor memory is freed
        if (!b_landed) mbar_wait_bounded(&bfull, 0, err, 2, 1ll << 26, true);
        for (int b = 0; b < 2; ++b)
            if (issued[b] > landed[b]) mbar_wait_bounded(&full[b], (uint32_t)(landed[b] & 1), err, 3, 1ll << 26, true);
        mma_commit(&drain);
        mbar_wait_bounded(&drain, 0, err, 4, 1ll << 26, true);
        bulk_wait_all();
    }
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 512);
}

// Epilogue passes of the wide kernels: every 4 groups x 4 rows of an element, up to
// kWideRows rows (p = 8: 165 modes); a group of at most kWideKc matrices per launch
constexpr int kWideKc = 3;
constexpr int kWideRows = 176;
constexpr int kWidePasses = kWideRows / 16;

// V rows of one element for a later group's launch: read into registers before the
// accumulators are ready, so that their latency hides behind the MMAs (a load, add and
// store per value in turn waited for memory once per value)
__device__ __forceinline__ void wide_prefetch(const float* __restrict__ vr, int nl, int group, bool on,
                                              float (&old)[kWidePasses][4]) {
#pragma unroll
    for (int t = 0; t < kWidePasses; ++t)
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int i = 4 * group + 16 * t + r;
            old[t][r] = (on && i < nl) ? vr[i] : 0.0f;
        }
}
// sum_k w_k D_k of the element (TMEM lane tl) over the group's matrices, plus old
__device__ __forceinline__ void wide_store(uint32_t tl, int nl, int nl4, int kc, int group, const float (&w)[kWideKc],
                                           bool on, const float (&old)[kWidePasses][4], float* __restrict__ vr) {
#pragma unroll
    for (int t = 0; t < kWidePasses; ++t) {
        const int i0 = 4 * group + 16 * t;
        if (i0 >= nl) break;
        float v[kWideKc][4];
#pragma unroll
        for (int k = 0; k < kWideKc; ++k) {
            if (k < kc) tmem_ld4(tl + (uint32_t)(k * nl4 + i0), v[k][0], v[k][1], v[k][2], v[k][3]);
            else v[k][0] = v[k][1] = v[k][2] = v[k][3] = 0.0f;
        }
        tmem_ld_wait();
        if (!on) continue;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int i = i0 + r;
            if (i >= nl) break;
            float acc = old[t][r];
#pragma unroll
            for (int k = 0; k < kWideKc; ++k) acc += w[k] * v[k][r];
            vr[i] = acc;
        }
    }
}

// ------------------------------ tcgen05 BF16 apply kernel for wide levels
// Levels whose six stacked matrices need more than the 512 accumulator columns
// (orders 7 and 8: 6 nl4 = 720 / 1008 rows).  One launch applies the matrices
// k0 .. k0 + kc - 1: their rows of B (kc nl4, padded to 2 nh) sit in shared memory
// and two MMAs of N = nh fill the accumulator; the epilogue stores sum_k w_k D_k into
// V on the first launch and adds it on the others.  Element tiles come from the BF16
// gather (U16), double-buffered as in k_mf_apply_tc; the results go straight to V
// (no staging tile: B and two A buffers use the shared memory).
__global__ void __launch_bounds__(kTcThreads, 1)
k_mf_apply_tcw(int E, int nl, int nl4, int kpad, int k0, int kc, int nh, int accumulate, const float* __restrict__ w6,
               const uint16_t* __restrict__ Bg, const uint16_t* __restrict__ U16, float* __restrict__ V, int* err) {
    static_assert(kTcGroups == 4, "the wide epilogue passes assume four row groups");
    extern __shared__ float4 smem4[];
    uint8_t* sm = reinterpret_cast<uint8_t*>(smem4);
    const uint32_t b_bytes = 2u * (uint32_t)nh * (uint32_t)kpad * 2u;
    const uint32_t a_bytes = (uint32_t)kTileT * (uint32_t)kpad * 2u;
    uint8_t* Bs = sm;
    uint8_t* Ab[2] = {sm + b_bytes, sm + b_bytes + a_bytes};
    __shared__ __align__(8) uint64_t full[2];
    __shared__ __align__(8) uint64_t bfull, mma_done, drain;
    __shared__ uint32_t tmem_slot;
    const int n_tiles = (E + kTileT - 1) / kTileT;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int kb = kpad / 8;
    // rows k0 nl4 ... of B: whole groups of 8 rows (nl4 is a multiple of 8 on these
    // levels), kb core matrices of 64 values each per group
    const uint16_t* Bsrc = Bg + (size_t)(k0 * nl4 / 8) * kb * 64;
    int issued[2] = {0, 0}, landed[2] = {0, 0};
    if (threadIdx.x == 0) {
        mbar_init(&full[0], 1);
        mbar_init(&full[1], 1);
        mbar_init(&bfull, 1);
        mbar_init(&mma_done, 1);
        mbar_init(&drain, 1);
        fence_mbar_init();
        mbar_expect_tx(&bfull, b_bytes);
        bulk_g2s(Bs, Bsrc, b_bytes, &bfull);
        if ((int)blockIdx.x < n_tiles) {
            mbar_expect_tx(&full[0], a_bytes);
            bulk_g2s(Ab[0], U16 + (size_t)blockIdx.x * (a_bytes / 2), a_bytes, &full[0]);
            issued[0] = 1;
        }
    }
    if (warp == 0) {
        tmem_alloc(&tmem_slot, 512);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const bool b_landed = mbar_wait_bounded(&bfull, 0, err, 21);
    int ok = __syncthreads_and(b_landed);
    const uint32_t lbo = 128, sbo = (uint32_t)kb * 128u;
    const uint32_t idesc = idesc_bf16(128, nh);
    const int stride = epi_stride(nl);
    int it = 0;
    for (int tile = blockIdx.x; ok && tile < n_tiles; tile += gridDim.x, ++it) {
        const int b = it & 1;
        if (threadIdx.x == 0) {
            if (tile + (int)gridDim.x < n_tiles) {
                mbar_expect_tx(&full[b ^ 1], a_bytes);
                bulk_g2s(Ab[b ^ 1], U16 + (size_t)(tile + gridDim.x) * (a_bytes / 2), a_bytes, &full[b ^ 1]);
                ++issued[b ^ 1];
            }
            if (mbar_wait_bounded(&full[b], (uint32_t)((it >> 1) & 1), err, 22)) {
                ++landed[b];
                tc_fence_after();
                const uint32_t a0 = smem_u32(Ab[b]), b0 = smem_u32(Bs);
                for (int c = 0; c < 2; ++c)
                    for (int q = 0; q < kpad / 16; ++q) {
                        const uint64_t ad = smem_desc(a0 + (uint32_t)q * 2u * lbo, lbo, sbo);
                        const uint64_t bd =
                            smem_desc(b0 + (uint32_t)c * (uint32_t)(nh / 8) * sbo + (uint32_t)q * 2u * lbo, lbo, sbo);
                        mma_bf16(tmem + (uint32_t)(c * nh), ad, bd, idesc, q > 0 ? 1u : 0u);
                    }
                mma_commit(&mma_done);
            }
        }
        // warp -> lane quarter (warp % 4) and every kTcGroups-th block of 4 rows (warp / 4)
        const int quarter = warp & 3, group = warp >> 2;
        const int el = quarter * 32 + lane, e = tile * kTileT + el;
        float* vr = V + (size_t)e * stride;
        float old[kWidePasses][4];
        wide_prefetch(vr, nl, group, accumulate && e < E, old);
        ok = __syncthreads_and(mbar_wait_bounded(&mma_done, (uint32_t)(it & 1), err, 23));
        tc_fence_after();
        if (ok) {
            float w[kWideKc];
#pragma unroll
            for (int k = 0; k < kWideKc; ++k) w[k] = (e < E && k < kc) ? __ldg(w6 + (size_t)(k0 + k) * E + e) : 0.0f;
            const uint32_t tl = tmem + ((uint32_t)(quarter * 32) << 16);
            wide_store(tl, nl, nl4, kc, group, w, e < E, old, vr);
        }
        tc_fence_before();
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        // after a give-up: the weight copy, the tile copies still in flight (at most one
        // per buffer) and every MMA issued finish before the tensor memory is freed
        if (!b_landed) mbar_wait_bounded(&bfull, 0, err, 21, 1ll << 26, true);
        for (int b = 0; b < 2; ++b)
            if (issued[b] > landed[b]) mbar_wait_bounded(&full[b], (uint32_t)(landed[b] & 1), err, 22, 1ll << 26, true);
        mma_commit(&drain);
        mbar_wait_bounded(&drain, 0, err, 24, 1ll << 26, true);
    }
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 512);
}

// ---------------------------------- tcgen05 BF16 apply kernel with a fused gather
// The BF16 GEMM of k_mf_apply_tc for unit levels, with the gather inside: twelve
// warps read the local coefficients of the next tile (packed indices gp [j][E]) into
// the other of two shared-memory A buffers, in the no-swizzle core-matrix layout,
// while sixteen warps read the accumulators of the current one.  The tiles never go
// through HBM and the gather overlaps the epilogue.
// Roles: warps 0-15 epilogue (as k_mf_apply_tc), warps 16-27 gather, warp 28 lane 0
// issues the MMAs.  Barriers: a_full[b] (gather -> MMA), a_empty[b] (MMA done reading
// buffer b), acc_full (MMAs of a tile done), acc_empty (epilogue done with TMEM).
// one work unit of the kernel below: a tile of one operator (a column of a block
// apply, or a member of a group: the largest i with ops[i].tile0 <= unit)
struct TcgUnit {
    int tile, E;
    int64_t n;            // length of x (the bounds check of the checked build)
    const int* gp;
    const float* x;
    const float* w6;
    float* V;
};
__device__ __forceinline__ TcgUnit tcg_unit(int unit, int E, int n_tiles, const int* gp, const float* x, const float* w6,
                                            float* V, int64_t xcol, int64_t vcol, const TcgOp* ops, int nops,
                                            int64_t nx) {
    TcgUnit u;
    if (ops) {
        int lo = 0, hi = nops - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (ops[mid].tile0 <= unit) lo = mid; else hi = mid - 1;
        }
        const TcgOp& o = ops[lo];
        u.tile = unit - o.tile0; u.E = o.E; u.n = o.n; u.gp = o.gp; u.x = o.x; u.w6 = o.w6; u.V = o.V;
    } else {
        const int col = unit / n_tiles;
        u.tile = unit % n_tiles; u.E = E; u.n = nx; u.gp = gp; u.x = x + (int64_t)col * xcol; u.w6 = w6;
        u.V = V + (int64_t)col * vcol;
    }
    return u;
}

constexpr int kTgEpi = 512;
constexpr int kTgGather = 384;
constexpr int kTgThreads = kTgEpi + kTgGather + 32;

__global__ void __launch_bounds__(kTgThreads, 1)
k_mf_apply_tcg(int E, int nl, int nl4, int kpad, const int* __restrict__ gp, const float* __restrict__ x,
               const float* __restrict__ w6, const uint16_t* __restrict__ Bg, float* __restrict__ V, int* err, int ncol,
               int64_t xcol, int64_t vcol, const TcgOp* __restrict__ ops, int nops, int units,
               const PcgScalars* __restrict__ halt, int64_t nx) {
    // a solve whose iteration has ended: nothing to do (every thread reads the same flag)
    if (halt && halt->done) return;
    extern __shared__ float4 smem4[];
    uint8_t* sm = reinterpret_cast<uint8_t*>(smem4);
    const uint32_t b_bytes = 512u * (uint32_t)kpad * 2u;
    const uint32_t a_bytes = (uint32_t)kTileT * (uint32_t)kpad * 2u;
    uint8_t* Bs = sm;
    uint8_t* Ab[2] = {sm + b_bytes, sm + b_bytes + a_bytes};
    float* St = reinterpret_cast<float*>(sm + b_bytes + 2 * a_bytes);
    __shared__ __align__(8) uint64_t bfull, a_full[2], a_empty[2], acc_full, acc_empty, drain;
    __shared__ uint32_t tmem_slot;
    // work units: (column, tile) pairs of a block apply, column-major; or the tiles of
    // the operators of a group one after another
    const int n_tiles = (E + kTileT - 1) / kTileT;
    const int n_units = ops ? units : n_tiles * ncol;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int kb = kpad / 8;
    if (threadIdx.x == 0) {
        mbar_init(&bfull, 1);
        for (int i = 0; i < 2; ++i) {
            mbar_init(&a_full[i], kTgGather);
            mbar_init(&a_empty[i], 1);
        }
        mbar_init(&acc_full, 1);
        mbar_init(&acc_empty, kTgEpi);
        mbar_init(&drain, 1);
        fence_mbar_init();
        mbar_expect_tx(&bfull, b_bytes);
        bulk_g2s(Bs, Bg, b_bytes, &bfull);
    }
    if (warp == 0) {
        tmem_alloc(&tmem_slot, 512);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const int my_tiles = (int)blockIdx.x < n_units ? (n_units - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    if (warp >= kTgEpi / 32 && warp < (kTgEpi + kTgGather) / 32) {
        // gather: 16-byte core rows (element m, modes 8 jb .. 8 jb + 7) of tile it into buffer it & 1
        const int gt = threadIdx.x - kTgEpi;
        for (int it = 0; it < my_tiles; ++it) {
            const int b = it & 1;
            if (it >= 2 && !mbar_wait_bounded(&a_empty[b], (uint32_t)(((it >> 1) - 1) & 1), err, 11)) break;
            const TcgUnit un = tcg_unit(blockIdx.x + it * gridDim.x, E, n_tiles, gp, x, w6, V, xcol, vcol, ops, nops, nx);
            const int tile = un.tile, Eu = un.E;
            const int* gpu = un.gp;
            const float* xc = un.x;
            // two core rows per thread and step: sixteen independent loads in flight
            for (int u0 = gt; u0 < kTileT * kb; u0 += 2 * kTgGather) {
                int pk[2][8];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int u = u0 + h * kTgGather;
                    const int m = u % kTileT, jb = u / kTileT, e = tile * kTileT + m;
#pragma unroll
                    for (int c = 0; c < 8; ++c) {
                        const int j = jb * 8 + c;
                        pk[h][c] = (u < kTileT * kb && e < Eu && j < nl) ? gpu[(size_t)j * Eu + e] : -1;
                    }
                }
                float v[2][8];
#pragma unroll
                for (int h = 0; h < 2; ++h)
#pragma unroll
                    for (int c = 0; c < 8; ++c) v[h][c] = unit_load(pk[h][c], xc, un.n);
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int u = u0 + h * kTgGather;
                    if (u >= kTileT * kb) break;
                    const int m = u % kTileT, jb = u / kTileT;
                    uint4 w;
                    w.x = (uint32_t)__bfloat16_as_ushort(__float2bfloat16(v[h][0])) | ((uint32_t)__bfloat16_as_ushort(__float2bfloat16(v[h][1])) << 16);
                    w.y = (uint32_t)__bfloat16_as_ushort(__float2bfloat16(v[h][2])) | ((uint32_t)__bfloat16_as_ushort(__float2bfloat16(v[h][3])) << 16);
                    w.z = (uint32_t)__bfloat16_as_ushort(__float2bfloat16(v[h][4])) | ((uint32_t)__bfloat16_as_ushort(__float2bfloat16(v[h][5])) << 16);
                    w.w = (uint32_t)__bfloat16_as_ushort(__float2bfloat16(v[h][6])) | ((uint32_t)__bfloat16_as_ushort(__float2bfloat16(v[h][7])) << 16);
                    *reinterpret_cast<uint4*>(Ab[b] + ((size_t)(m / 8) * kb + jb) * 128 + (m % 8) * 16) = w;
                }
            }
            // the MMAs read shared memory through the async proxy
            fence_proxy_async();
            mbar_arrive(&a_full[b]);
        }
    } else if (warp == (kTgEpi + kTgGather) / 32) {
        if (lane == 0) {
            const uint32_t lbo = 128, sbo = (uint32_t)kb * 128u;
            const uint32_t idesc = idesc_bf16(128, 256);
            bool ok = mbar_wait_bounded(&bfull, 0, err, 12);
            for (int it = 0; ok && it < my_tiles; ++it) {
                const int b = it & 1;
                if (!mbar_wait_bounded(&a_full[b], (uint32_t)((it >> 1) & 1), err, 13)) break;
                if (it > 0 && !mbar_wait_bounded(&acc_empty, (uint32_t)((it - 1) & 1), err, 14)) break;
                tc_fence_after();
                const uint32_t a0 = smem_u32(Ab[b]), b0 = smem_u32(Bs);
                for (int c = 0; c < 2; ++c)
                    for (int q = 0; q < kpad / 16; ++q) {
                        const uint64_t ad = smem_desc(a0 + (uint32_t)q * 2u * lbo, lbo, sbo);
                        const uint64_t bd = smem_desc(b0 + (uint32_t)c * 32u * sbo + (uint32_t)q * 2u * lbo, lbo, sbo);
                        mma_bf16(tmem + (uint32_t)c * 256u, ad, bd, idesc, q > 0 ? 1u : 0u);
                    }
                mma_commit(&a_empty[b]);
                mma_commit(&acc_full);
            }
            mma_commit(&drain);
            mbar_wait_bounded(&drain, 0, err, 15, 1ll << 26, true);
        }
    } else if (warp < kTgEpi / 32) {
        const int quarter = warp & 3, group = warp >> 2;
        const uint32_t tl = tmem + ((uint32_t)(quarter * 32) << 16);
        for (int it = 0; it < my_tiles; ++it) {
            // one decision for all epilogue warps: they meet at named barriers below
            // each lane quarter (its 4 warps, 32 elements) stages and stores its own rows
            if (group == 0 && lane == 0) bulk_wait_read();   // its previous store has read the staging rows
            if (!named_bar_and(1 + quarter, 128, mbar_wait_bounded(&acc_full, (uint32_t)(it & 1), err, 16))) break;
            tc_fence_after();
            const TcgUnit un = tcg_unit(blockIdx.x + it * gridDim.x, E, n_tiles, gp, x, w6, V, xcol, vcol, ops, nops, nx);
            const int tile = un.tile, Eu = un.E;
            float* Vc = un.V;
            const int el = quarter * 32 + lane, e = tile * kTileT + el;
            float w[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) w[k] = e < Eu ? __ldg(un.w6 + (size_t)k * Eu + e) : 0.0f;
            epi_combine(tl, nl, nl4, 4 * group, 4 * (kTgEpi / 128), w, St + el * epi_stride(nl));
            fence_proxy_async();               // the staging tile is read by the bulk copy
            tc_fence_before();
            mbar_arrive(&acc_empty);           // accumulators read: the next tile's MMAs may start
            named_bar(1 + quarter, 128);       // the quarter's staging rows are complete
            if (group == 0 && lane == 0) {
                const size_t r0 = (size_t)quarter * 32 * epi_stride(nl);
                bulk_s2g(Vc + (size_t)tile * kTileT * epi_stride(nl) + r0, St + r0, 32u * epi_stride(nl) * 4u);
            }
        }
        if (group == 0 && lane == 0) bulk_wait_all();
    }
    // the B copy has landed even if no tile ran (the block may not exit with it in flight)
    if (threadIdx.x == 0) mbar_wait_bounded(&bfull, 0, err, 17, 1ll << 26, true);
    __syncwarp();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, 512);
}

// ------------------------------------------- tcgen05 split-TF32 apply kernel
// The FP32-accurate element GEMM (the Krylov operator) on the tensor cores.  Both
// operands are split into TF32 pairs, U = Uh + Ul and S = Sh + Sl (every part exactly
// representable in TF32), and
//     D = Uh Sh^T + Uh Sl^T + Ul Sh^T
// omits only Ul Sl^T, of relative size 2^-22: the rounding level of an FP32 dot
// product.  The split stack (2 x 512 x kpad x 4 B) does not fit in shared memory next
// to the tiles, so both operands stream through a ring of stages of one K step (8
// modes): [Uh 4 KB | Ul 4 KB | Sh 16 KB | Sl 16 KB], each part in the no-swizzle
// K-major core-matrix layout (K-adjacent core matrices 128 B apart, M/N-adjacent ones
// 256 B apart).  The global layouts U3 [tile][q][2][128][8] and B3 [q][2][512][8]
// match a stage, which is then two bulk copies.
// Roles: warps 0-15 read the accumulators and combine the six matrices (as in the
// BF16 kernel), warp 16 lane 0 issues the bulk copies, warp 17 lane 0 the MMAs.  The
// accumulators fill the tensor memory, so the MMAs of a tile wait for the epilogue
// of the previous one while the copies run ahead.
constexpr int kX3Stages = 4;
constexpr int kX3EpiThreads = 512;
constexpr int kX3Threads = kX3EpiThreads + 64;
constexpr uint32_t kX3ABytes = 2u * kTileT * 8u * 4u;     // Uh + Ul of one K step
constexpr uint32_t kX3BBytes = 2u * 512u * 8u * 4u;       // Sh + Sl of one K step
constexpr uint32_t kX3StageBytes = kX3ABytes + kX3BBytes;

__global__ void __launch_bounds__(kX3Threads, 1)
k_mf_apply_x3(int E, int nl, int nl4, int kq, int nhalf, const float* __restrict__ w6, const float* __restrict__ B3,
              const float* __restrict__ U3, float* __restrict__ V, int* err) {
    extern __shared__ float4 smem4[];
    uint8_t* sm = reinterpret_cast<uint8_t*>(smem4);
    float* St = reinterpret_cast<float*>(sm + (size_t)kX3Stages * kX3StageBytes);
    __shared__ __align__(8) uint64_t full[kX3Stages], empty[kX3Stages];
    __shared__ __align__(8) uint64_t acc_full, acc_empty, drain;
    __shared__ uint32_t tmem_slot;
    const int n_tiles = (E + kTileT - 1) / kTileT;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int i = 0; i < kX3Stages; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        mbar_init(&acc_full, 1);
        mbar_init(&acc_empty, kX3EpiThreads);
        mbar_init(&drain, 1);
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem_alloc(&tmem_slot, 512);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const int my_tiles = (int)blockIdx.x < n_tiles ? (n_tiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    if (warp == kX3EpiThreads / 32) {
        if (lane == 0) {
            // producer: stage g = it * kq + q over this block's tiles
            const long long total = (long long)my_tiles * kq;
            long long g = 0;
            for (; g < total; ++g) {
                const int st = (int)(g % kX3Stages);
                const long long use = g / kX3Stages;
                if (use > 0 && !mbar_wait_bounded(&empty[st], (uint32_t)((use - 1) & 1), err, 5)) break;
                const int it = (int)(g / kq), q = (int)(g % kq);
                const size_t tile = (size_t)blockIdx.x + (size_t)it * gridDim.x;
                uint8_t* dst = sm + (size_t)st * kX3StageBytes;
                mbar_expect_tx(&full[st], kX3StageBytes);
                bulk_g2s(dst, U3 + (tile * kq + q) * (kX3ABytes / 4), kX3ABytes, &full[st]);
                bulk_g2s(dst + kX3ABytes, B3 + (size_t)q * (kX3BBytes / 4), kX3BBytes, &full[st]);
            }
            // every copy issued has landed before the block may exit: wait for the last
            // use of each stage
            for (long long h = g - 1; h >= 0 && h >= g - kX3Stages; --h)
                mbar_wait_bounded(&full[h % kX3Stages], (uint32_t)((h / kX3Stages) & 1), err, 10, 1ll << 26, true);
        }
    } else if (warp == kX3EpiThreads / 32 + 1) {
        if (lane == 0) {
            const uint32_t idesc = idesc_tf32(128, 256);
            long long g = 0;
            bool ok = true;
            for (int it = 0; ok && it < my_tiles; ++it) {
                // the epilogue has read the previous tile's accumulators
                if (it > 0 && !mbar_wait_bounded(&acc_empty, (uint32_t)((it - 1) & 1), err, 6)) break;
                tc_fence_after();
                for (int q = 0; q < kq; ++q, ++g) {
                    const int st = (int)(g % kX3Stages);
                    if (!mbar_wait_bounded(&full[st], (uint32_t)((g / kX3Stages) & 1), err, 7)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t base = smem_u32(sm + (size_t)st * kX3StageBytes);
                    const uint64_t ah = smem_desc(base, 128, 256), al = smem_desc(base + kX3ABytes / 2, 128, 256);
                    for (int c = 0; c < nhalf; ++c) {
                        const uint32_t b0 = base + kX3ABytes + (uint32_t)c * 8192u;
                        const uint64_t bh = smem_desc(b0, 128, 256), bl = smem_desc(b0 + kX3BBytes / 2, 128, 256);
                        const uint32_t d = tmem + (uint32_t)c * 256u;
                        mma_tf32(d, ah, bh, idesc, q > 0 ? 1u : 0u);
                        mma_tf32(d, ah, bl, idesc, 1u);
                        mma_tf32(d, al, bh, idesc, 1u);
                    }
                    mma_commit(&empty[st]);   // the stage is free once these MMAs have read it
                }
                if (ok) mma_commit(&acc_full);
            }
            // no MMA may still write the tensor memory when it is freed
            mma_commit(&drain);
            mbar_wait_bounded(&drain, 0, err, 8, 1ll << 26, true);
        }
    } else {
        const int quarter = warp & 3, group = warp >> 2;
        const uint32_t tl = tmem + ((uint32_t)(quarter * 32) << 16);
        for (int it = 0; it < my_tiles; ++it) {
            // one decision for all epilogue warps: they meet at named barriers below
            // each lane quarter (its 4 warps, 32 elements) stages and stores its own rows
            if (group == 0 && lane == 0) bulk_wait_read();   // its previous store has read the staging rows
            if (!named_bar_and(1 + quarter, 128, mbar_wait_bounded(&acc_full, (uint32_t)(it & 1), err, 9))) break;
            tc_fence_after();
            const int tile = blockIdx.x + it * gridDim.x;
            const int el = quarter * 32 + lane, e = tile * kTileT + el;
            float w[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) w[k] = e < E ? __ldg(w6 + (size_t)k * E + e) : 0.0f;
            epi_combine(tl, nl, nl4, 4 * group, 4 * (kX3EpiThreads / 128), w, St + el * epi_stride(nl));
            fence_proxy_async();               // the staging tile is read by the bulk copy
            tc_fence_before();
            mbar_arrive(&acc_empty);           // accumulators read: the next tile's MMAs may start
            named_bar(1 + quarter, 128);       // the quarter's staging rows are complete
            if (group == 0 && lane == 0) {
                const size_t r0 = (size_t)quarter * 32 * epi_stride(nl);
                bulk_s2g(V + (size_t)tile * kTileT * epi_stride(nl) + r0, St + r0, 32u * epi_stride(nl) * 4u);
            }
        }
        if (group == 0 && lane == 0) bulk_wait_all();
    }
    __syncwarp();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, 512);
}

// ----------------------------- tcgen05 split-TF32 apply kernel for wide levels
// The FP32-accurate operator of levels whose six stacked matrices need more than the
// 512 accumulator columns (orders 7 and 8).  One launch applies the matrices
// k0 .. k0 + kc - 1 (the groups of k_mf_apply_tcw): two MMAs of N = nh per part
// product fill 2 nh accumulator columns.  Both operands stream through the ring of
// stages of k_mf_apply_x3, a stage now holding the tile's K step [Uh | Ul] (8 KB)
// and the group's rows of it [Sh | Sl] (2 nh rows each, the same core-matrix
// layout).  The epilogue stores sum_k w_k D_k into V on the first launch and adds it
// on the others, element rows straight to V as in k_mf_apply_tcw.
static_assert(kX3EpiThreads / 128 == 4, "the wide epilogue passes assume four row groups");

__host__ __device__ constexpr uint32_t x3w_stage_bytes(int nh) { return kX3ABytes + 128u * (uint32_t)nh; }

__global__ void __launch_bounds__(kX3Threads, 1)
k_mf_apply_x3w(int E, int nl, int nl4, int kq, int k0, int kc, int nh, int accumulate, const float* __restrict__ w6,
               const float* __restrict__ B3g, const float* __restrict__ U3, float* __restrict__ V, int* err) {
    extern __shared__ float4 smem4[];
    uint8_t* sm = reinterpret_cast<uint8_t*>(smem4);
    const uint32_t b_bytes = 128u * (uint32_t)nh;   // [hi/lo][2 nh][8] floats
    const uint32_t stage_bytes = kX3ABytes + b_bytes;
    __shared__ __align__(8) uint64_t full[kX3Stages], empty[kX3Stages];
    __shared__ __align__(8) uint64_t acc_full, acc_empty, drain;
    __shared__ uint32_t tmem_slot;
    const int n_tiles = (E + kTileT - 1) / kTileT;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int i = 0; i < kX3Stages; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        mbar_init(&acc_full, 1);
        mbar_init(&acc_empty, kX3EpiThreads);
        mbar_init(&drain, 1);
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem_alloc(&tmem_slot, 512);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_slot;
    const int my_tiles = (int)blockIdx.x < n_tiles ? (n_tiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    if (warp == kX3EpiThreads / 32) {
        if (lane == 0) {
            // producer: stage g = it * kq + q over this block's tiles
            const long long total = (long long)my_tiles * kq;
            long long g = 0;
            for (; g < total; ++g) {
                const int st = (int)(g % kX3Stages);
                const long long use = g / kX3Stages;
                if (use > 0 && !mbar_wait_bounded(&empty[st], (uint32_t)((use - 1) & 1), err, 40)) break;
                const int it = (int)(g / kq), q = (int)(g % kq);
                const size_t tile = (size_t)blockIdx.x + (size_t)it * gridDim.x;
                uint8_t* dst = sm + (size_t)st * stage_bytes;
                mbar_expect_tx(&full[st], stage_bytes);
                bulk_g2s(dst, U3 + (tile * kq + q) * (kX3ABytes / 4), kX3ABytes, &full[st]);
                bulk_g2s(dst + kX3ABytes, B3g + (size_t)q * (b_bytes / 4), b_bytes, &full[st]);
            }
            // every copy issued has landed before the block may exit
            for (long long h = g - 1; h >= 0 && h >= g - kX3Stages; --h)
                mbar_wait_bounded(&full[h % kX3Stages], (uint32_t)((h / kX3Stages) & 1), err, 41, 1ll << 26, true);
        }
    } else if (warp == kX3EpiThreads / 32 + 1) {
        if (lane == 0) {
            const uint32_t idesc = idesc_tf32(128, nh);
            long long g = 0;
            bool ok = true;
            for (int it = 0; ok && it < my_tiles; ++it) {
                // the epilogue has read the previous tile's accumulators
                if (it > 0 && !mbar_wait_bounded(&acc_empty, (uint32_t)((it - 1) & 1), err, 42)) break;
                tc_fence_after();
                for (int q = 0; q < kq; ++q, ++g) {
                    const int st = (int)(g % kX3Stages);
                    if (!mbar_wait_bounded(&full[st], (uint32_t)((g / kX3Stages) & 1), err, 43)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t base = smem_u32(sm + (size_t)st * stage_bytes);
                    const uint64_t ah = smem_desc(base, 128, 256), al = smem_desc(base + kX3ABytes / 2, 128, 256);
                    for (int c = 0; c < 2; ++c) {
                        const uint32_t b0 = base + kX3ABytes + (uint32_t)c * 32u * (uint32_t)nh;
                        const uint64_t bh = smem_desc(b0, 128, 256), bl = smem_desc(b0 + 64u * (uint32_t)nh, 128, 256);
                        const uint32_t d = tmem + (uint32_t)(c * nh);
                        mma_tf32(d, ah, bh, idesc, q > 0 ? 1u : 0u);
                        mma_tf32(d, ah, bl, idesc, 1u);
                        mma_tf32(d, al, bh, idesc, 1u);
                    }
                    mma_commit(&empty[st]);   // the stage is free once these MMAs have read it
                }
                if (ok) mma_commit(&acc_full);
            }
            // no MMA may still write the tensor memory when it is freed
            mma_commit(&drain);
            mbar_wait_bounded(&drain, 0, err, 44, 1ll << 26, true);
        }
    } else {
        const int quarter = warp & 3, group = warp >> 2;
        const uint32_t tl = tmem + ((uint32_t)(quarter * 32) << 16);
        const int stride = epi_stride(nl);
        for (int it = 0; it < my_tiles; ++it) {
            const int tile = blockIdx.x + it * gridDim.x;
            const int el = quarter * 32 + lane, e = tile * kTileT + el;
            float* vr = V + (size_t)e * stride;
            float old[kWidePasses][4];
            wide_prefetch(vr, nl, group, accumulate && e < E, old);
            // one decision for the quarter's warps (they meet at a named barrier)
            if (!named_bar_and(1 + quarter, 128, mbar_wait_bounded(&acc_full, (uint32_t)(it & 1), err, 45))) break;
            tc_fence_after();
            float w[kWideKc];
#pragma unroll
            for (int k = 0; k < kWideKc; ++k) w[k] = (e < E && k < kc) ? __ldg(w6 + (size_t)(k0 + k) * E + e) : 0.0f;
            wide_store(tl, nl, nl4, kc, group, w, e < E, old, vr);
            tc_fence_before();
            mbar_arrive(&acc_empty);   // accumulators read: the next tile's MMAs may start
        }
    }
    __syncwarp();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, 512);
}

// U3: split TF32 tiles of kTileT elements, one 8 KB block per K step of 8 modes,
// [tile][q][hi/lo][m/8][K core matrix 2][m%8][4 modes].  One thread writes the hi and
// lo 16-byte rows of one element and 4 consecutive modes.
template <bool UNIT>
__global__ void k_gather_x3(int E, int E_pad, int nl, int kq, int md, const int* __restrict__ gi,
                            const float* __restrict__ gv, const int* __restrict__ gp, const float* __restrict__ x,
                            int64_t nx, float4* __restrict__ U) {
    const int64_t total = (int64_t)E_pad * kq * 2;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int e = (int)(t % E_pad), jc = (int)(t / E_pad);
        float v[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int j = jc * 4 + c;
            float u = 0.0f;
            if (e < E && j < nl) {
                if (UNIT) {
                    u = unit_load(gp[(size_t)j * E + e], x, nx);
                } else {
                    for (int q = 0; q < md; ++q) {
                        const size_t o = ((size_t)j * md + q) * E + e;
                        const int g = gi[o];
                        if (g >= 0 && in_bounds(g, nx, 36)) u += gv[o] * __ldg(x + g);
                    }
                }
            }
            v[c] = u;
        }
        float h[4], l[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            h[c] = __uint_as_float(tf32_round_bits(__float_as_uint(v[c])));
            l[c] = __uint_as_float(tf32_round_bits(__float_as_uint(v[c] - h[c])));
        }
        const int tile = e / kTileT, m = e % kTileT, q = jc >> 1, kc = jc & 1;
        const size_t part = ((size_t)tile * kq + q) * 2;                 // 4 KB parts = 256 float4
        const size_t off = ((size_t)(m / 8) * 2 + kc) * 8 + (m % 8);
        U[part * 256 + off] = make_float4(h[0], h[1], h[2], h[3]);
        U[(part + 1) * 256 + off] = make_float4(l[0], l[1], l[2], l[3]);
    }
}

// y = A x with an FP32 CSR level operator, TPR lanes per row
template <int TPR>
__global__ void k_spmv_f32(int64_t n, const int64_t* __restrict__ rp, const int* __restrict__ ci,
                           const float* __restrict__ va, const float* __restrict__ x, float* __restrict__ y) {
    const int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / TPR;
    const int lane = threadIdx.x % TPR;
    float acc = 0.0f;
    if (r < n)
        for (int64_t k = rp[r] + lane; k < rp[r + 1]; k += TPR)
            if (in_bounds(ci[k], n, 39)) acc += va[k] * __ldg(x + ci[k]);
#pragma unroll
    for (int o = TPR / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, TPR);
    if (r < n && lane == 0) y[r] = acc;
}

// The CSR level operator with the row's Chebyshev update fused in.  The applied
// vector is read at neighbouring rows, so this kernel never writes it: the new
// direction goes to a second buffer dn, and the solution takes each direction one
// step late (xs += d just before d is replaced; the last one is added after the sweep
// by k_f_add), which adds the same terms in the same order as the unfused recurrence.
//   kResid:      v = rhs - A x
//   kChebFirst:  v = rhs - A x,  dn = a dinv v            (x is the solution)
//   kChebStep:   v -= A d,  xs += d,  dn = a d + c dinv v (x = d is the direction)
template <int TPR, int MODE>
__global__ void k_spmv_f32_cheb(int64_t n, const int64_t* __restrict__ rp, const int* __restrict__ ci,
                                const float* __restrict__ va, const float* __restrict__ x, MfPost po0,
                                float* __restrict__ dn) {
    if (po0.st && po0.st->done) return;
    const MfPost po = col_post(po0, (int64_t)blockIdx.y * n);
    x += (int64_t)blockIdx.y * n;
    if (dn) dn += (int64_t)blockIdx.y * n;
    const int64_t r = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / TPR;
    const int lane = threadIdx.x % TPR;
    float acc = 0.0f;
    if (r < n)
        for (int64_t k = rp[r] + lane; k < rp[r + 1]; k += TPR)
            if (in_bounds(ci[k], n, 37)) acc += va[k] * __ldg(x + ci[k]);
#pragma unroll
    for (int o = TPR / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, TPR);
    if (r >= n || lane != 0) return;
    if (MODE == MfPost::kResid) {
        po.v[r] = po.rhs[r] - acc;
    } else if (MODE == MfPost::kChebFirst) {
        const float v = po.rhs[r] - acc;
        po.v[r] = v;
        dn[r] = po.a * po.dinv[r] * v;
    } else {
        const float v = po.v[r] - acc;
        po.v[r] = v;
        const float d = x[r];
        po.xs[r] += d;
        dn[r] = po.a * d + po.c * po.dinv[r] * v;
    }
}

__global__ void k_d2f(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

__global__ void k_bnd_fix(int64_t nb, const int* __restrict__ bnd, const float* __restrict__ d, const float* __restrict__ x,
                          float* y) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nb; i += (int64_t)gridDim.x * blockDim.x)
        y[bnd[i]] += d[i] * x[bnd[i]];
}

static int nb(int64_t n) { return grid_for(n, 256, 152 * 16); }

// SM count and the dynamic shared-memory limit of the GEMM kernels on one device
struct DevLimits {
    int sms = 0;
    size_t smem_optin = 0;
};
constexpr int kMaxDevices = 64;
static DevLimits g_limits[kMaxDevices];
static std::atomic<bool> g_limits_ready[kMaxDevices];
static std::mutex g_limits_mu;

// The current device's limits, read (and the kernels' shared-memory attribute set,
// which is a per-device setting) the first time a device asks; solvers may be
// built from several threads and on several devices.
static const DevLimits& device_limits() {
    int dev = 0, v = 0;
    TSEM_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) throw Error(TSEM_INVALID, "device ordinal out of range");
    DevLimits& lim = g_limits[dev];
    if (g_limits_ready[dev].load(std::memory_order_acquire)) return lim;
    std::lock_guard<std::mutex> lock(g_limits_mu);
    if (g_limits_ready[dev].load(std::memory_order_relaxed)) return lim;
    TSEM_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
    lim.sms = v;
    TSEM_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    // dynamic shared memory may use what the static declarations leave
    cudaFuncAttributes fa{}, fb{};
    TSEM_CUDA(cudaFuncGetAttributes(&fa, k_mf_apply));
    TSEM_CUDA(cudaFuncGetAttributes(&fb, k_mf_apply_tc));
    cudaFuncAttributes fc{}, fd{}, fw{}, fx{};
    TSEM_CUDA(cudaFuncGetAttributes(&fc, k_mf_apply_x3));
    TSEM_CUDA(cudaFuncGetAttributes(&fd, k_mf_apply_tcg));
    TSEM_CUDA(cudaFuncGetAttributes(&fw, k_mf_apply_tcw));
    TSEM_CUDA(cudaFuncGetAttributes(&fx, k_mf_apply_x3w));
    const size_t stat = std::max({fa.sharedSizeBytes, fb.sharedSizeBytes, fc.sharedSizeBytes, fd.sharedSizeBytes,
                                  fw.sharedSizeBytes, fx.sharedSizeBytes}) + 64;
    lim.smem_optin = (size_t)v - stat;
    TSEM_CUDA(cudaFuncSetAttribute(k_mf_apply, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lim.smem_optin));
    TSEM_CUDA(cudaFuncSetAttribute(k_mf_apply_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lim.smem_optin));
    TSEM_CUDA(cudaFuncSetAttribute(k_mf_apply_x3, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lim.smem_optin));
    TSEM_CUDA(cudaFuncSetAttribute(k_mf_apply_tcg, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lim.smem_optin));
    TSEM_CUDA(cudaFuncSetAttribute(k_mf_apply_tcw, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lim.smem_optin));
    TSEM_CUDA(cudaFuncSetAttribute(k_mf_apply_x3w, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lim.smem_optin));
    g_limits_ready[dev].store(true, std::memory_order_release);
    return lim;
}

// the tensor-core path needs the six matrices of every row in 512 accumulator
// columns and both operands in shared memory
static bool tc_fits(int nl) {
    const DevLimits& lim = device_limits();
    const int nl4 = (nl + 3) & ~3, kpad = (nl + 15) & ~15;
    return nl >= 4 && 6 * nl4 <= 512 && (size_t)(512 + 2 * kTileT) * kpad * 2 + epi_bytes(nl) + 1024 <= lim.smem_optin;
}

// wide levels (more than 512 accumulator columns for all six matrices): the most
// matrices per launch whose B rows and two A tiles fit in shared memory, balanced
// over the launches; N per MMA is half the launch's rows, rounded up to 16
static bool tcw_fits(int nl, int& kc_out, int& nh_out) {
    const DevLimits& lim = device_limits();
    const int nl4 = (nl + 3) & ~3, kpad = (nl + 15) & ~15;
    if (nl < 20 || nl4 % 8 != 0) return false;
    auto nh_of = [&](int kc) { return ((kc * nl4 + 1) / 2 + 15) & ~15; };
    auto fits = [&](int kc) {
        const int nh = nh_of(kc);
        return nh <= 256 && (size_t)(2 * nh + 2 * kTileT) * kpad * 2 + 1024 <= lim.smem_optin;
    };
    if (nl > kWideRows) return false;
    int kc = kWideKc;   // the epilogue holds at most kWideKc matrices
    while (kc > 0 && !fits(kc)) --kc;
    if (kc == 0) return false;
    const int launches = (6 + kc - 1) / kc;
    kc = (6 + launches - 1) / launches;
    kc_out = kc;
    nh_out = nh_of(kc);
    return true;
}

// the split-TF32 path streams its operands, so only the accumulator width limits it
static bool x3_fits(int nl) {
    const DevLimits& lim = device_limits();
    const int nl4 = (nl + 3) & ~3;
    return nl >= 4 && 6 * nl4 <= 512 && (size_t)kX3Stages * kX3StageBytes + epi_bytes(nl) + 1024 <= lim.smem_optin;
}

// the split-TF32 path of a wide level: the ring of stages with the group's rows
static bool x3w_fits(int nh) {
    const DevLimits& lim = device_limits();
    return nh % 16 == 0 && nh <= 256 && (size_t)kX3Stages * x3w_stage_bytes(nh) + 1024 <= lim.smem_optin;
}

static float tf32_round_host(float x) {
    uint32_t b;
    std::memcpy(&b, &x, 4);
    b = tf32_round_bits(b);
    std::memcpy(&x, &b, 4);
    return x;
}

enum class GemmPath { kF32, kBf16, kX3, kBf16W, kX3W };
static GemmPath gemm_path(const MfLevel& L, bool low_precision) {
    if (low_precision && L.tc) return GemmPath::kBf16;
    if (low_precision && L.tcw) return GemmPath::kBf16W;
    if (!low_precision && L.x3) return GemmPath::kX3;
    if (!low_precision && L.x3w) return GemmPath::kX3W;
    return GemmPath::kF32;
}

// gather, element GEMMs: the per-element results V of A_level x (matrix-free
// levels); `mid`, when given, is recorded between the gather and the GEMM
void MfOperator::elements(int level, const float* x, cudaStream_t s, bool low_precision, cudaEvent_t mid, int ncol,
                          const PcgScalars* halt) const {
    const MfLevel& L = levels[level];
    const int sms = device_limits().sms;
    if (ncol > cols) throw Error(TSEM_INVALID, "more columns than the operator holds results for");
    const GemmPath path = gemm_path(L, low_precision);
    if (path == GemmPath::kBf16 && L.unit) {
        // gather fused into the GEMM; a block of ncol columns is one launch over (column, tile) pairs
        const int n_tiles = (E + kTileT - 1) / kTileT;
        if (mid) TSEM_CUDA(cudaEventRecord(mid, s));
        const size_t shm = (size_t)(512 + 2 * kTileT) * L.kpad * 2 + epi_bytes(L.nl);
        k_mf_apply_tcg<<<std::min(n_tiles * ncol, sms), kTgThreads, shm, s>>>(
            E, L.nl, L.nl4, L.kpad, L.gp.p, x, w6.p, L.Bt.p, Vbuf.p, err.p, ncol, (int64_t)L.n, vcol, nullptr, 0, 0, halt,
            L.n);
        TSEM_LAUNCHED();
        return;
    }
    for (int c = 0; c < ncol; ++c)
        elements_col(level, x + (int64_t)c * L.n, Vbuf.p + (int64_t)c * vcol, s, (int)path, c == 0 ? mid : nullptr);
}

// one column of the paths without a block launch: gather, then the element GEMM into V
void MfOperator::elements_col(int level, const float* x, float* V, cudaStream_t s, int gpath, cudaEvent_t mid) const {
    const MfLevel& L = levels[level];
    const DevLimits& lim = device_limits();
    const GemmPath path = (GemmPath)gpath;
    if (path == GemmPath::kBf16) {
        // levels with general transforms (unit levels take the fused-gather kernel)
        const int n_tiles = (E + kTileT - 1) / kTileT;
        const int E_pad = n_tiles * kTileT;
        k_gather_bf16<<<grid_for((int64_t)E_pad * (L.kpad / 8), 256), 256, 0, s>>>(E, E_pad, L.nl, L.kpad, L.md, L.gi.p,
                                                                                  L.gv.p, x, L.n, (uint4*)U16.p);
        TSEM_LAUNCHED();
        if (mid) TSEM_CUDA(cudaEventRecord(mid, s));
        const size_t shm = (size_t)(512 + 2 * kTileT) * L.kpad * 2 + epi_bytes(L.nl);
        k_mf_apply_tc<<<std::min(n_tiles, lim.sms), kTcThreads, shm, s>>>(E, L.nl, L.nl4, L.kpad, L.md, L.gi.p, L.gv.p,
                                                                            w6.p, L.Bt.p, U16.p, V, err.p);
        TSEM_LAUNCHED();
    } else if (path == GemmPath::kBf16W) {
        // wide levels: the gathered tiles once, then one launch per group of matrices
        const int n_tiles = (E + kTileT - 1) / kTileT;
        const int E_pad = n_tiles * kTileT;
        k_gather_bf16<<<grid_for((int64_t)E_pad * (L.kpad / 8), 256), 256, 0, s>>>(E, E_pad, L.nl, L.kpad, L.md, L.gi.p,
                                                                                  L.gv.p, x, L.n, (uint4*)U16.p);
        TSEM_LAUNCHED();
        if (mid) TSEM_CUDA(cudaEventRecord(mid, s));
        const size_t shm = (size_t)(2 * L.tcw_nh + 2 * kTileT) * L.kpad * 2;
        for (int k0 = 0; k0 < 6; k0 += L.tcw_kc) {
            const int kc = std::min(L.tcw_kc, 6 - k0);
            k_mf_apply_tcw<<<std::min(n_tiles, lim.sms), kTcThreads, shm, s>>>(E, L.nl, L.nl4, L.kpad, k0, kc, L.tcw_nh,
                                                                               k0 > 0 ? 1 : 0, w6.p, L.Bt.p, U16.p, V,
                                                                               err.p);
            TSEM_LAUNCHED();
        }
    } else if (path == GemmPath::kX3W) {
        // wide levels: the split tiles once, then one launch per group of matrices
        const int n_tiles = (E + kTileT - 1) / kTileT;
        const int E_pad = n_tiles * kTileT;
        const unsigned g = grid_for((int64_t)E_pad * L.kq * 2, 256);
        if (L.unit)
            k_gather_x3<true><<<g, 256, 0, s>>>(E, E_pad, L.nl, L.kq, 1, nullptr, nullptr, L.gp.p, x, L.n, (float4*)U3.p);
        else
            k_gather_x3<false><<<g, 256, 0, s>>>(E, E_pad, L.nl, L.kq, L.md, L.gi.p, L.gv.p, nullptr, x, L.n,
                                                 (float4*)U3.p);
        TSEM_LAUNCHED();
        if (mid) TSEM_CUDA(cudaEventRecord(mid, s));
        const size_t group_floats = (size_t)L.kq * 2 * 2 * L.tcw_nh * 8;
        for (int k0 = 0, gi = 0; k0 < 6; k0 += L.tcw_kc, ++gi) {
            const int kc = std::min(L.tcw_kc, 6 - k0);
            k_mf_apply_x3w<<<std::min(n_tiles, lim.sms), kX3Threads, (size_t)kX3Stages * x3w_stage_bytes(L.tcw_nh), s>>>(
                E, L.nl, L.nl4, L.kq, k0, kc, L.tcw_nh, k0 > 0 ? 1 : 0, w6.p, L.B3.p + (size_t)gi * group_floats, U3.p, V,
                err.p);
            TSEM_LAUNCHED();
        }
    } else if (path == GemmPath::kX3) {
        const int n_tiles = (E + kTileT - 1) / kTileT;
        const int E_pad = n_tiles * kTileT;
        const unsigned g = grid_for((int64_t)E_pad * L.kq * 2, 256);
        if (L.unit)
            k_gather_x3<true><<<g, 256, 0, s>>>(E, E_pad, L.nl, L.kq, 1, nullptr, nullptr, L.gp.p, x, L.n, (float4*)U3.p);
        else
            k_gather_x3<false><<<g, 256, 0, s>>>(E, E_pad, L.nl, L.kq, L.md, L.gi.p, L.gv.p, nullptr, x, L.n,
                                                 (float4*)U3.p);
        TSEM_LAUNCHED();
        if (mid) TSEM_CUDA(cudaEventRecord(mid, s));
        const int nhalf = 6 * L.nl4 > 256 ? 2 : 1;
        k_mf_apply_x3<<<std::min(n_tiles, lim.sms), kX3Threads, (size_t)kX3Stages * kX3StageBytes + epi_bytes(L.nl),
                        s>>>(E, L.nl, L.nl4, L.kq, nhalf, w6.p, L.B3.p, U3.p, V, err.p);
        TSEM_LAUNCHED();
    } else {
        const int n_tiles = (E + kTileE - 1) / kTileE;
        const int E_pad = n_tiles * kTileE;
        if (L.unit)
            k_gather_f32_unit<<<grid_for((int64_t)E_pad * L.nl, 256), 256, 0, s>>>(E, E_pad, L.nl, L.gp.p, x, L.n, U32.p);
        else
            k_gather_f32<<<grid_for((int64_t)E_pad * L.nl, 256), 256, 0, s>>>(E, E_pad, L.nl, L.md, L.gi.p, L.gv.p, x,
                                                                             L.n, U32.p);
        TSEM_LAUNCHED();
        if (mid) TSEM_CUDA(cudaEventRecord(mid, s));
        // rows per pass so that the staged stack and two tiles fit in shared memory
        const size_t fixed = 2 * (size_t)L.nl * kTileE * sizeof(float);
        int rows = L.nl;
        while (rows > 2 && fixed + (size_t)L.nl * ((rows + 1) & ~1) * 6 * sizeof(float) > lim.smem_optin) rows = (rows + 1) / 2;
        for (int r0 = 0; r0 < L.nl; r0 += rows) {
            const int cnt = std::min(rows, L.nl - r0);
            const size_t shm = fixed + (size_t)L.nl * ((cnt + 1) & ~1) * 6 * sizeof(float);
            k_mf_apply<<<std::min(n_tiles, lim.sms), kApplyThreads, shm, s>>>(E, L.nl, L.nlp, L.md, r0, cnt, L.gi.p, L.gv.p,
                                                                                 w6.p, L.S.p, U32.p, V, epi_stride(L.nl), 1,
                                                                                 err.p);
            TSEM_LAUNCHED();
        }
    }
}

// y = A x on a level applied as an assembled FP32 CSR matrix, tpr lanes per row
static void spmv_csr(const MfLevel& L, int tpr, const float* x, float* y, cudaStream_t s) {
    const unsigned g = (unsigned)((L.n * tpr + 255) / 256);
    switch (tpr) {
        case 2: k_spmv_f32<2><<<g, 256, 0, s>>>(L.n, L.crp.p, L.ccol.p, L.cval.p, x, y); break;
        case 4: k_spmv_f32<4><<<g, 256, 0, s>>>(L.n, L.crp.p, L.ccol.p, L.cval.p, x, y); break;
        case 8: k_spmv_f32<8><<<g, 256, 0, s>>>(L.n, L.crp.p, L.ccol.p, L.cval.p, x, y); break;
        case 16: k_spmv_f32<16><<<g, 256, 0, s>>>(L.n, L.crp.p, L.ccol.p, L.cval.p, x, y); break;
        default: k_spmv_f32<32><<<g, 256, 0, s>>>(L.n, L.crp.p, L.ccol.p, L.cval.p, x, y); break;
    }
    TSEM_LAUNCHED();
}

// lanes per row of a CSR level's SpMV: each of 2 .. 32 timed on the level itself
// (CUDA events, best of 8 launches after one warm-up), the fastest kept
static int autotune_csr_tpr(const MfLevel& L, const float* x, float* y, cudaStream_t s) {
    cudaEvent_t a, b;
    TSEM_CUDA(cudaEventCreate(&a));
    TSEM_CUDA(cudaEventCreate(&b));
    int best = 8;
    float best_ms = 1e30f;
    for (int tpr = 2; tpr <= 32; tpr *= 2) {
        spmv_csr(L, tpr, x, y, s);
        float ms_min = 1e30f;
        for (int r = 0; r < 8; ++r) {
            TSEM_CUDA(cudaEventRecord(a, s));
            spmv_csr(L, tpr, x, y, s);
            TSEM_CUDA(cudaEventRecord(b, s));
            TSEM_CUDA(cudaEventSynchronize(b));
            float ms = 0.0f;
            TSEM_CUDA(cudaEventElapsedTime(&ms, a, b));
            ms_min = std::min(ms_min, ms);
        }
        if (ms_min < best_ms) {
            best_ms = ms_min;
            best = tpr;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return best;
}

// CSR levels: A x with the row update `mode` fused in (k_spmv_f32_cheb)
void MfOperator::spmv_cheb(int level, int mode, const float* x, const MfPost& po, float* dn, cudaStream_t s,
                           int ncol) const {
    const MfLevel& L = levels[level];
    if (!L.csr) throw Error(TSEM_INVALID, "level is applied matrix-free");
    const dim3 g((unsigned)((L.n * L.csr_tpr + 255) / 256), (unsigned)ncol);
#define TSEM_SPMV_CHEB(T)                                                                                          \
    if (mode == MfPost::kResid)                                                                                    \
        k_spmv_f32_cheb<T, MfPost::kResid><<<g, 256, 0, s>>>(L.n, L.crp.p, L.ccol.p, L.cval.p, x, po, dn);         \
    else if (mode == MfPost::kChebFirst)                                                                           \
        k_spmv_f32_cheb<T, MfPost::kChebFirst><<<g, 256, 0, s>>>(L.n, L.crp.p, L.ccol.p, L.cval.p, x, po, dn);     \
    else                                                                                                           \
        k_spmv_f32_cheb<T, MfPost::kChebStep><<<g, 256, 0, s>>>(L.n, L.crp.p, L.ccol.p, L.cval.p, x, po, dn);
    switch (L.csr_tpr) {
        case 2: { TSEM_SPMV_CHEB(2) } break;
        case 4: { TSEM_SPMV_CHEB(4) } break;
        case 8: { TSEM_SPMV_CHEB(8) } break;
        case 16: { TSEM_SPMV_CHEB(16) } break;
        default: { TSEM_SPMV_CHEB(32) } break;
    }
#undef TSEM_SPMV_CHEB
    TSEM_LAUNCHED();
}

void MfOperator::apply(int level, const float* x, float* y, cudaStream_t s, bool low_precision) const {
    const MfLevel& L = levels[level];
    if (L.csr) {
        spmv_csr(L, L.csr_tpr, x, y, s);
        return;
    }
    elements(level, x, s, low_precision);
    MfPost po;
    po.y = y;
    scatter(level, const_cast<float*>(x), po, s);
}

void MfOperator::scatter(int level, float* x, const MfPost& po, cudaStream_t s, int ncol) const {
    const MfLevel& L = levels[level];
    const dim3 g((unsigned)nb(L.n), (unsigned)ncol);
#define TSEM_SCATTER(M)                                                                                            \
    if (L.unit)                                                                                                    \
        k_scatter_t<true, M><<<g, 256, 0, s>>>(L.n, L.trp.p, L.tpos.p, nullptr, Vbuf.p, L.bdiag.p, x, po, vcol);   \
    else                                                                                                           \
        k_scatter_t<false, M><<<g, 256, 0, s>>>(L.n, L.trp.p, L.tpos.p, L.tval.p, Vbuf.p, L.bdiag.p, x, po, vcol);
    switch (po.mode) {
        case MfPost::kStore: TSEM_SCATTER(MfPost::kStore) break;
        case MfPost::kResid: TSEM_SCATTER(MfPost::kResid) break;
        case MfPost::kChebFirst: TSEM_SCATTER(MfPost::kChebFirst) break;
        default: TSEM_SCATTER(MfPost::kChebStep) break;
    }
#undef TSEM_SCATTER
    TSEM_LAUNCHED();
}

// Device time of the three kernels of one apply (CUDA events on stream s, averaged
// over reps) and their algorithmic work: out = {ms gather, ms GEMM, ms scatter,
// bytes gather, bytes GEMM, flops GEMM, bytes scatter, ms scatter of a Chebyshev
// step, its bytes}.  The Chebyshev-step scatter (the smoother's update fused in:
// v -= A d, d = a d + c dinv v, xs += d) is the instantiation the V-cycle launches
// most; it runs on the results of the same GEMM, with work vectors of its own.
// Matrix-free levels only.
void MfOperator::profile(int level, bool low_precision, int reps, const float* x, float* y, cudaStream_t s,
                         double* out) const {
    const MfLevel& L = levels[level];
    if (L.csr) throw Error(TSEM_INVALID, "level is applied as an assembled matrix");
    device_limits();
    const GemmPath path = gemm_path(L, low_precision);
    cudaEvent_t ev[5];
    for (auto& e : ev) TSEM_CUDA(cudaEventCreate(&e));
    float t[4] = {0, 0, 0, 0};
    MfPost po;
    po.y = y;
    // the Chebyshev step's vectors: d (applied, updated in place), v, xs
    DBuf<float> dv(L.n), vv(L.n), xsv(L.n);
    TSEM_CUDA(cudaMemcpyAsync(dv.p, x, L.n * sizeof(float), cudaMemcpyDeviceToDevice, s));
    vv.zero(s);
    xsv.zero(s);
    MfPost pc;
    pc.mode = MfPost::kChebStep;
    pc.v = vv.p; pc.xs = xsv.p; pc.dinv = L.dinv.p;
    pc.a = 0.5f; pc.c = 1e-3f;
    for (int r = -1; r < reps; ++r) {   // r = -1 warms up
        TSEM_CUDA(cudaEventRecord(ev[0], s));
        elements(level, x, s, low_precision, ev[1]);
        TSEM_CUDA(cudaEventRecord(ev[2], s));
        scatter(level, const_cast<float*>(x), po, s);
        TSEM_CUDA(cudaEventRecord(ev[3], s));
        scatter(level, dv.p, pc, s);
        TSEM_CUDA(cudaEventRecord(ev[4], s));
        TSEM_CUDA(cudaEventSynchronize(ev[4]));
        if (r >= 0)
            for (int k = 0; k < 4; ++k) {
                float ms = 0;
                TSEM_CUDA(cudaEventElapsedTime(&ms, ev[k], ev[k + 1]));
                t[k] += ms;
            }
    }
    for (auto& e : ev) cudaEventDestroy(e);
    out[7] = reps > 0 ? t[3] / reps : 0.0;
    const double nl = L.nl, Ed = E, n = (double)L.n, nnzT = (double)L.tpos.n;
    const double E_pad_t = (double)((E + kTileT - 1) / kTileT * kTileT);
    const double E_pad_f = (double)((E + kTileE - 1) / kTileE * kTileE);
    for (int k = 0; k < 3; ++k) out[k] = reps > 0 ? t[k] / reps : 0.0;
    const double idx = L.unit ? 4.0 * nl * Ed : 8.0 * nl * L.md * Ed;          // gp, or gi + gv
    // bytes of the gathered tiles U (written by the gather, read by the GEMM)
    const double ub = path == GemmPath::kBf16 ? 2.0 * L.kpad * E_pad_t
                      : (path == GemmPath::kX3 || path == GemmPath::kX3W) ? 2.0 * 4.0 * 8.0 * L.kq * E_pad_t
                                              : 4.0 * nl * E_pad_f;
    if (path == GemmPath::kBf16 && L.unit) {
        // gather fused into the GEMM: indices and x once, V and the weights
        out[3] = 0.0;
        out[4] = idx + 4.0 * n + 4.0 * nl * Ed + 24.0 * Ed;
    } else {
        out[3] = idx + 4.0 * n + ub;                 // + x once
        out[4] = ub + 4.0 * nl * Ed + 24.0 * Ed;     // U, V, w6
    }
    out[5] = 12.0 * nl * nl * Ed;                                                // 6 GEMMs of nl x nl
    out[6] = 4.0 * (n + 1) + 4.0 * nnzT + 4.0 * nnzT + 4.0 * n + (L.unit ? 0.0 : 4.0 * nnzT);  // trp, tpos, V, y
    // Chebyshev step: trp, tpos, V (tval), then v, d, dinv, xs read and v, d, xs written
    out[8] = 4.0 * (n + 1) + 8.0 * nnzT + (L.unit ? 0.0 : 4.0 * nnzT) + 28.0 * n;
}

// A x followed by the vector update `po` (levels without an assembled CSR operator),
// for ncol columns n_level apart
void MfOperator::apply_post(int level, float* x, const MfPost& po, cudaStream_t s, bool low_precision, int ncol) const {
    elements(level, x, s, low_precision, nullptr, ncol, po.st);
    scatter(level, x, po, s, ncol);
}

// room for the per-element results of ncol columns
void MfOperator::ensure_columns(int ncol) {
    if (ncol <= cols) return;
    DBuf<float> nv((size_t)vcol * ncol);
    Vbuf = std::move(nv);
    cols = ncol;
}

// ------------------------------------------------------------------ FP32 kernels
__global__ void k_f_scale_dot(int64_t n, const float* __restrict__ dinv, const float* __restrict__ ay, float* z,
                              const float* __restrict__ y, double* out) {
    double acc[2] = {0, 0};
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const float zj = dinv[j] * ay[j];
        z[j] = zj;
        acc[0] += (double)zj * zj;
        acc[1] += (double)zj * y[j];
    }
    double* const dst[2] = {out, out + 1};
    block_accumulate<2>(acc, dst);
}
__global__ void k_f_normalize(int64_t n, float* x, const double* __restrict__ s) {
    const float f = (float)(1.0 / sqrt(s[0]));
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) x[j] *= f;
}

// first Chebyshev step from x = 0: v = rhs, d = s dinv rhs, x = d (x = 0 when the
// sweep adds each direction one step late, as the fused CSR sweep does)
__global__ void k_f_cheb_zero(int64_t n, const float* __restrict__ dinv, const float* __restrict__ rhs, float* v, float* d,
                              float s, float* x, const PcgScalars* st, int deferred) {
    if (st && st->done) return;
    const int64_t o = (int64_t)blockIdx.y * n;   // column of a block V-cycle
    rhs += o; v += o; d += o; x += o;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        const float r = rhs[j];
        v[j] = r;
        const float dj = dinv[j] * r * s;
        d[j] = dj;
        x[j] = deferred ? 0.0f : dj;
    }
}
// x += d: the last direction of a fused CSR sweep
__global__ void k_f_add(int64_t n, float* x, const float* __restrict__ d, const PcgScalars* st) {
    if (st && st->done) return;
    x += (int64_t)blockIdx.y * n;
    d += (int64_t)blockIdx.y * n;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
        x[j] += d[j];
}
__global__ void k_f_restrict(int64_t nf, int64_t nc, const int* __restrict__ core, const float* __restrict__ v, float* rc,
                             const PcgScalars* st) {
    if (st && st->done) return;
    v += (int64_t)blockIdx.y * nf;
    rc += (int64_t)blockIdx.y * nc;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nf; j += (int64_t)gridDim.x * blockDim.x) {
        const int c = core[j];
        if (c >= 0) rc[c] = v[j];
    }
}
__global__ void k_f_prolong(int64_t nf, int64_t nc, const int* __restrict__ core, const float* __restrict__ xc, float* x,
                            const PcgScalars* st) {
    if (st && st->done) return;
    xc += (int64_t)blockIdx.y * nc;
    x += (int64_t)blockIdx.y * nf;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nf; j += (int64_t)gridDim.x * blockDim.x) {
        const int c = core[j];
        if (c >= 0) x[j] += xc[c];
    }
}
__global__ void k_f_zero(int64_t n, float* x, const PcgScalars* st) {
    if (st && st->done) return;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) x[j] = 0.f;
}

// inner PCG (standard sign convention: r = b - A x)
__global__ void k_in_init(int64_t n, const float* __restrict__ r, const float* __restrict__ z, float* p, PcgScalars* st) {
    double acc[2] = {0, 0};
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        p[j] = z[j];
        acc[0] += (double)r[j] * z[j];
        acc[1] += (double)r[j] * r[j];
    }
    double* const dst[2] = {&st->rty[0], &st->bb};
    block_accumulate<2>(acc, dst);
}
// the bodies of the PCG kernels, shared by the single-solve kernels and the grouped
// one (k_grp_pcg: blockIdx.y is the solve)
__device__ __forceinline__ void in_pq(int64_t n, const float* __restrict__ p, const float* __restrict__ q, PcgScalars* st) {
    if (st->done) return;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const int cur = st->iter & 1;
        st->cur = cur;
        st->rty[cur ^ 1] = 0.0;
        st->rr = 0.0;
    }
    double acc[1] = {0};
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
        acc[0] += (double)p[j] * q[j];
    double* const dst[1] = {&st->pap};
    block_accumulate<1>(acc, dst);
}
__device__ __forceinline__ void in_update(int64_t n, float* x, float* r, const float* __restrict__ p,
                                          const float* __restrict__ q, PcgScalars* st) {
    if (st->done) return;
    const double pq = st->pap;
    if (!(pq > 0.0) || !isfinite(pq)) return;
    const float alpha = (float)(st->rty[st->cur] / pq);
    double acc[1] = {0};
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        x[j] += alpha * p[j];
        const float rj = r[j] - alpha * q[j];
        r[j] = rj;
        acc[0] += (double)rj * rj;
    }
    double* const dst[1] = {&st->rr};
    block_accumulate<1>(acc, dst);
}
__device__ __forceinline__ void in_rz(int64_t n, const float* __restrict__ r, const float* __restrict__ z, PcgScalars* st) {
    if (st->done) return;
    double acc[1] = {0};
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
        acc[0] += (double)r[j] * z[j];
    double* const dst[1] = {&st->rty[st->cur ^ 1]};
    block_accumulate<1>(acc, dst);
}
__device__ __forceinline__ void in_p(int64_t n, float* p, const float* __restrict__ z, PcgScalars* st) {
    if (st->done) return;
    const int cur = st->cur;
    const float beta = (float)(st->rty[cur ^ 1] / st->rty[cur]);
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
        p[j] = z[j] + beta * p[j];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const int it = st->iter + 1;
        st->iter = it;
        const double pq = st->pap;
        if (!(pq > 0.0) || !isfinite(pq)) { st->done = 1; st->status = TSEM_BREAKDOWN; }
        else if (!isfinite(st->rr)) { st->done = 1; st->status = TSEM_NONFINITE; }
        else if (st->rr <= st->tol_rel2 * st->bb) { st->done = 1; st->status = TSEM_OK; }
        else if (it >= st->max_iter) { st->done = 1; st->status = TSEM_MAXIT; }
        st->pap = 0.0;
    }
}
__global__ void k_in_pq(int64_t n, const float* __restrict__ p, const float* __restrict__ q, PcgScalars* st) {
    in_pq(n, p, q, st);
}
__global__ void k_in_update(int64_t n, float* x, float* r, const float* __restrict__ p, const float* __restrict__ q,
                            PcgScalars* st) {
    in_update(n, x, r, p, q, st);
}
__global__ void k_in_rz(int64_t n, const float* __restrict__ r, const float* __restrict__ z, PcgScalars* st) {
    in_rz(n, r, z, st);
}
__global__ void k_in_p(int64_t n, float* p, const float* __restrict__ z, PcgScalars* st) { in_p(n, p, z, st); }

// outer FP64 helpers
__global__ void k_norms(int64_t n, const double* __restrict__ a, double* out) {
    double acc[1] = {0};
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
        acc[0] += a[j] * a[j];
    double* const dst[1] = {out};
    block_accumulate<1>(acc, dst);
}
// out[0] += |b|^2, out[1] += the number of nonzero entries of x
__global__ void k_norm_nz(int64_t n, const double* __restrict__ b, const double* __restrict__ x, double* out) {
    double acc[2] = {0, 0};
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
        acc[0] += b[j] * b[j];
        acc[1] += x[j] != 0.0 ? 1.0 : 0.0;
    }
    double* const dst[2] = {out, out + 1};
    block_accumulate<2>(acc, dst);
}
__global__ void k_to_f32(int64_t n, const double* __restrict__ a, double s, float* b) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
        b[j] = (float)(a[j] * s);
}
__global__ void k_axpy_f32(int64_t n, double s, const float* __restrict__ d, double* x) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
        x[j] += s * (double)d[j];
}

// ------------------------------------------------------------------ build
static void dihedral_host(const double* xyz, const int* nd, double g[6]) {
    double P[4][3];
    for (int k = 0; k < 4; ++k)
        for (int j = 0; j < 3; ++j) P[k][j] = xyz[3 * (size_t)nd[k] + j];
    const int I1[6] = {0, 0, 0, 1, 1, 2}, I2[6] = {1, 2, 3, 2, 3, 3};
    const int Sx[6] = {2, 1, 2, 0, 0, 0}, Tx[6] = {3, 3, 1, 3, 2, 1};
    const int slot[6] = {0, 3, 5, 1, 2, 4};
    for (int q = 0; q < 6; ++q) {
        double a[3], b[3], c[3];
        for (int j = 0; j < 3; ++j) {
            a[j] = P[Tx[q]][j] - P[Sx[q]][j];
            b[j] = P[I1[q]][j] - P[Sx[q]][j];
            c[j] = P[I2[q]][j] - P[Sx[q]][j];
        }
        const double u0 = a[1] * b[2] - a[2] * b[1], u1 = -a[0] * b[2] + a[2] * b[0], u2 = a[0] * b[1] - a[1] * b[0];
        const double v0 = a[1] * c[2] - a[2] * c[1], v1 = -a[0] * c[2] + a[2] * c[0], v2 = a[0] * c[1] - a[1] * c[0];
        const double w = 0.25 * (u0 * v0 + u1 * v1 + u2 * v2);
        g[slot[q]] = std::fabs(w) < 1e-12 ? 0.0 : w;
    }
}

void MfOperator::build(tsem_space_s* sp, const DevCsr& A_bc, int dflag, int step, cudaStream_t s) {
    space_reference(sp);
    const SpaceHost& h = sp->host;
    // element count padded with empty elements (no transform terms, zero weights) to
    // an odd multiple of 32: it is also the stride of every [.][element] array
    const int E_real = h.nt;
    E = odd_multiple(E_real, 32);
    M = h.M;
    n_loc = h.n_loc;
    if (A_bc.n != h.n_dof) throw Error(TSEM_INVALID, "matrix size differs from the space");
    // TSEM_MF_GEMM=fp32 keeps the FP32-accurate applies on the CUDA-core GEMM (the
    // split-TF32 tensor-core GEMM is used otherwise, where a level fits it)
    const char* gemm_env = std::getenv("TSEM_MF_GEMM");
    const bool x3_enabled = !(gemm_env && std::strcmp(gemm_env, "fp32") == 0);
    // element weights
    {
        std::vector<float> w((size_t)6 * E);
        for (int e = 0; e < E_real; ++e) {
            double g[6];
            dihedral_host(h.xyz.data(), &h.ele_node[4 * (size_t)e], g);
            const double c = 2.0 / (3.0 * h.volume[e]);
            for (int k = 0; k < 6; ++k) w[(size_t)k * E + e] = (float)(c * g[k]);
        }
        w6.upload(w, s);
    }
    // Dirichlet DOFs and the FP64 diagonal
    std::vector<uint8_t> isd(h.n_dof, 0);
    if (dflag != 0) {
        auto on = [&](int m) { return dflag == -1 ? m != 0 : m == dflag; };
        for (int v = 0; v < h.nv; ++v) if (on(h.mark_v[v])) isd[h.vdof[v]] = 1;
        for (int g = 0; g < h.ne; ++g) if (on(h.mark_e[g])) for (int i = 0; i < h.ndE; ++i) isd[h.edof[g] + i] = 1;
        for (int f = 0; f < h.nf; ++f) if (on(h.mark_f[f])) for (int i = 0; i < h.ndF; ++i) isd[h.fdof[f] + i] = 1;
    }
    std::vector<double> diag(h.n_dof);
    A_bc.diag.download(diag.data(), h.n_dof, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    // level orders as in init_PMG
    const int np = std::max(1, (M + step - 1) / step - 1 + ((M - 1) % step == 0 ? 0 : 1));
    std::vector<int> order(np + 1);
    order[0] = M;
    order[np] = 1;
    for (int i = 1; i < np; ++i) order[i] = order[i - 1] - step;
    if (M == 1) order = {1};
    levels.clear();
    levels.resize(order.size());
    std::vector<std::vector<int>> lmap(order.size(), std::vector<int>(h.n_dof, -1));
    for (size_t L = 0; L < order.size(); ++L) {
        int c = 0;
        for (int64_t g = 0; g < h.n_dof; ++g)
            if (h.sum_dof[g] <= order[L]) lmap[L][g] = c++;
        levels[L].n = c;
        levels[L].q = order[L];
    }
    const auto& Sref = sp->ref->stiff;   // FP64 [6][n_loc][n_loc]
    for (size_t L = 0; L < order.size(); ++L) {
        MfLevel& lv = levels[L];
        lv.nl = mi_count(lv.q);
        lv.nlp = (lv.nl + 3) & ~3;
        int md = 1;
        for (int e = 0; e < E_real; ++e)
            for (int a = 0; a < lv.nl; ++a) md = std::max(md, h.t_n[(size_t)e * n_loc + a]);
        lv.md = md;
        std::vector<int> gi((size_t)lv.nl * md * E, -1);
        std::vector<float> gv((size_t)lv.nl * md * E, 0.0f);
        for (int e = 0; e < E_real; ++e)
            for (int a = 0; a < lv.nl; ++a) {
                const size_t b = (size_t)e * n_loc + a;
                for (int t = 0; t < h.t_n[b]; ++t) {
                    const int g = h.t_ind[b * h.max_dep + t];
                    const int lg = lmap[L][g];
                    if (lg < 0) throw Error(TSEM_INVALID, "level transform references a DOF of higher degree");
                    const size_t o = ((size_t)a * md + t) * E + e;
                    gi[o] = lg;
                    gv[o] = isd[g] ? 0.0f : (float)h.t_val[b * h.max_dep + t];
                }
            }
        lv.gi.upload(gi, s);
        lv.gv.upload(gv, s);
        // packed index of unit levels and the transposed transform of the scatter
        bool unit = md == 1;
        for (size_t o = 0; unit && o < gi.size(); ++o)
            if (gi[o] >= 0 && gv[o] != 0.0f && std::fabs(gv[o]) != 1.0f) unit = false;
        lv.unit = unit;
        if (unit) {
            std::vector<int> gp((size_t)lv.nl * E);
            for (size_t o = 0; o < gp.size(); ++o)
                gp[o] = (gi[o] < 0 || gv[o] == 0.0f) ? -1 : (gv[o] > 0.0f ? gi[o] : -gi[o] - 2);
            lv.gp.upload(gp, s);
        }
        {
            const int64_t vs = v_stride(E);
            if ((int64_t)epi_stride(lv.nl) * vs >= (int64_t)1 << 31)
                throw Error(TSEM_INVALID, "mesh too large for 32-bit result positions");
            std::vector<int> trp(lv.n + 1, 0);
            for (int a = 0; a < lv.nl; ++a)
                for (int t = 0; t < md; ++t)
                    for (int e = 0; e < E; ++e) {
                        const size_t o = ((size_t)a * md + t) * E + e;
                        if (gi[o] >= 0 && gv[o] != 0.0f) ++trp[gi[o] + 1];
                    }
            for (int64_t g = 0; g < lv.n; ++g) trp[g + 1] += trp[g];
            std::vector<int> cur(trp.begin(), trp.end() - 1), tpos(trp[lv.n]);
            std::vector<float> tval(unit ? 0 : trp[lv.n]);
            for (int a = 0; a < lv.nl; ++a)
                for (int t = 0; t < md; ++t)
                    for (int e = 0; e < E; ++e) {
                        const size_t o = ((size_t)a * md + t) * E + e;
                        if (gi[o] < 0 || gv[o] == 0.0f) continue;
                        const int k = cur[gi[o]]++;
                        const int pos = (int)((int64_t)e * epi_stride(lv.nl) + a);
                        if (unit) tpos[k] = gv[o] > 0.0f ? pos : ~pos;
                        else { tpos[k] = pos; tval[k] = gv[o]; }
                    }
            lv.trp.upload(trp, s);
            lv.tpos.upload(tpos, s);
            if (!unit) lv.tval.upload(tval, s);
        }
        std::vector<float> S((size_t)6 * lv.nl * lv.nlp, 0.0f);
        for (int k = 0; k < 6; ++k)
            for (int i = 0; i < lv.nl; ++i)
                for (int j = 0; j < lv.nl; ++j)
                    S[((size_t)k * lv.nl + i) * lv.nlp + j] = (float)Sref[((size_t)k * n_loc + i) * n_loc + j];
        lv.S.upload(S, s);
        std::vector<int> bnd;
        std::vector<float> bd;
        std::vector<float> dinv(lv.n), bdg(lv.n, 0.0f);
        for (int64_t g = 0; g < h.n_dof; ++g) {
            const int lg = lmap[L][g];
            if (lg < 0) continue;
            dinv[lg] = (float)(1.0 / diag[g]);
            if (isd[g]) { bnd.push_back(lg); bd.push_back((float)diag[g]); bdg[lg] = (float)diag[g]; }
        }
        lv.bnd.upload(bnd, s);
        lv.bnd_diag.upload(bd, s);
        lv.bdiag.upload(bdg, s);
        lv.dinv.upload(dinv, s);
        if (L + 1 < order.size()) {
            std::vector<int> core(lv.n, -1);
            for (int64_t g = 0; g < h.n_dof; ++g)
                if (lmap[L][g] >= 0) core[lmap[L][g]] = lmap[L + 1][g];
            lv.core.upload(core, s);
        }
        lv.x.alloc(lv.n); lv.r.alloc(lv.n); lv.v.alloc(lv.n); lv.t.alloc(lv.n); lv.ad.alloc(lv.n);
        lv.xv = lv.x.p;
        // BF16 operand of the tensor-core path: rows n = k * nl4 + i, K padded to 16,
        // no-swizzle K-major core-matrix layout (16-byte rows, 8 per core matrix)
        lv.nl4 = (lv.nl + 3) & ~3;
        lv.kpad = (lv.nl + 15) & ~15;
        lv.tc = lv.nl >= 20 && tc_fits(lv.nl);
        if (lv.tc) {
            const int kb = lv.kpad / 8;
            std::vector<uint16_t> B((size_t)512 * lv.kpad, 0);
            for (int k = 0; k < 6; ++k)
                for (int i = 0; i < lv.nl; ++i) {
                    const int nrow = k * lv.nl4 + i;
                    for (int j = 0; j < lv.nl; ++j) {
                        const size_t unit = ((size_t)(nrow / 8) * kb + j / 8) * 8 + nrow % 8;
                        const float v = (float)Sref[((size_t)k * n_loc + i) * n_loc + j];
                        B[unit * 8 + j % 8] = __bfloat16_as_ushort(__float2bfloat16(v));
                    }
                }
            lv.Bt.upload(B, s);
        }
        // wide levels: the same layout over all 6 nl4 rows, plus 2 nh zero rows so that
        // the last launch's padded slice stays inside the array
        lv.tcw = !lv.tc && lv.nl >= 20 && tcw_fits(lv.nl, lv.tcw_kc, lv.tcw_nh);
        if (lv.tcw) {
            const int kb = lv.kpad / 8;
            const size_t rows = (size_t)6 * lv.nl4 + 2 * lv.tcw_nh;
            std::vector<uint16_t> B(((rows + 7) / 8) * 8 * lv.kpad, 0);
            for (int k = 0; k < 6; ++k)
                for (int i = 0; i < lv.nl; ++i) {
                    const int nrow = k * lv.nl4 + i;
                    for (int j = 0; j < lv.nl; ++j) {
                        const size_t unit = ((size_t)(nrow / 8) * kb + j / 8) * 8 + nrow % 8;
                        const float v = (float)Sref[((size_t)k * n_loc + i) * n_loc + j];
                        B[unit * 8 + j % 8] = __bfloat16_as_ushort(__float2bfloat16(v));
                    }
                }
            lv.Bt.upload(B, s);
        }
        // split-TF32 operand of the FP32-accurate tensor-core path: the same stacked rows
        // as hi + lo TF32 parts of the FP64 matrices, one [hi/lo][512][8] block per K step
        lv.kq = (lv.nl + 7) / 8;
        lv.x3 = lv.tc && x3_enabled && x3_fits(lv.nl);
        if (lv.x3) {
            std::vector<float> B((size_t)lv.kq * 2 * 512 * 8, 0.0f);
            for (int k = 0; k < 6; ++k)
                for (int i = 0; i < lv.nl; ++i) {
                    const int nrow = k * lv.nl4 + i;
                    for (int j = 0; j < lv.nl; ++j) {
                        const double v = Sref[((size_t)k * n_loc + i) * n_loc + j];
                        const float h = tf32_round_host((float)v);
                        const float l = tf32_round_host((float)(v - (double)h));
                        const size_t at = ((size_t)(nrow / 8) * 2 + (j % 8) / 4) * 32 + (nrow % 8) * 4 + j % 4;
                        B[((size_t)(j / 8) * 2 + 0) * 4096 + at] = h;
                        B[((size_t)(j / 8) * 2 + 1) * 4096 + at] = l;
                    }
                }
            lv.B3.upload(B, s);
        }
        // the same for the wide levels, per group of tcw_kc matrices: [group][kq][hi/lo]
        // [2 tcw_nh][8], the group's rows k * nl4 + i (k counted from the group's first)
        lv.x3w = lv.tcw && x3_enabled && x3w_fits(lv.tcw_nh);
        if (lv.x3w) {
            const int nh2 = 2 * lv.tcw_nh, ng = (6 + lv.tcw_kc - 1) / lv.tcw_kc;
            const size_t blk = (size_t)nh2 * 8;
            std::vector<float> B((size_t)ng * lv.kq * 2 * blk, 0.0f);
            for (int k = 0; k < 6; ++k) {
                const int gi = k / lv.tcw_kc, kr = k % lv.tcw_kc;
                for (int i = 0; i < lv.nl; ++i) {
                    const int nrow = kr * lv.nl4 + i;
                    for (int j = 0; j < lv.nl; ++j) {
                        const double v = Sref[((size_t)k * n_loc + i) * n_loc + j];
                        const float h = tf32_round_host((float)v);
                        const float l = tf32_round_host((float)(v - (double)h));
                        const size_t at = ((size_t)(nrow / 8) * 2 + (j % 8) / 4) * 32 + (nrow % 8) * 4 + j % 4;
                        const size_t q0 = ((size_t)gi * lv.kq + j / 8) * 2;
                        B[(q0 + 0) * blk + at] = h;
                        B[(q0 + 1) * blk + at] = l;
                    }
                }
            }
            lv.B3.upload(B, s);
        }
        // levels without a tensor-core path (few modes per element) are applied as
        // assembled FP32 CSR matrices: one SpMV instead of gather, GEMM and scatter
        if (!lv.tc && !lv.tcw) {
            DevCsr C;
            principal_submatrix(A_bc, lmap[L], lv.n, C, s);
            lv.cval.alloc(C.nnz);
            k_d2f<<<nb(C.nnz), 256, 0, s>>>(C.nnz, C.val.p, lv.cval.p);
            TSEM_LAUNCHED();
            lv.crp = std::move(C.rowptr);
            lv.ccol = std::move(C.col);
            lv.csr = true;
            lv.x.zero(s);
            lv.csr_tpr = autotune_csr_tpr(lv, lv.x.p, lv.ad.p, s);
            TSEM_CUDA(cudaStreamSynchronize(s));
        }
    }
    // scratch tiles shared by all levels
    size_t u32 = 0, u16 = 0, u3 = 0;
    for (auto& lv : levels) {
        u32 = std::max(u32, (size_t)((E + kTileE - 1) / kTileE) * kTileE * lv.nl);
        // BF16 tiles in HBM only for levels with general transforms (unit levels gather in the GEMM)
        if ((lv.tc && !lv.unit) || lv.tcw) u16 = std::max(u16, (size_t)((E + kTileT - 1) / kTileT) * kTileT * lv.kpad);
        if (lv.x3 || lv.x3w) u3 = std::max(u3, (size_t)((E + kTileT - 1) / kTileT) * kTileT * lv.kq * 16);
    }
    U32.alloc(u32);
    if (u16) U16.alloc(u16);
    if (u3) U3.alloc(u3);
    {
        // per-element results V[e][i]
        size_t vb = 0;
        for (auto& lv : levels) vb = std::max(vb, (size_t)v_stride(E) * (size_t)epi_stride(lv.nl));
        Vbuf.alloc(vb);
        vcol = (int64_t)vb;
        cols = 1;
    }
    err.alloc(1);
    err.zero(s);
    // largest eigenvalue of D^{-1} A per level (power iteration)
    for (size_t L = 0; L < levels.size(); ++L) {
        MfLevel& lv = levels[L];
        std::vector<float> y0(lv.n);
        uint64_t st = 0x9E3779B97F4A7C15ull + L;
        for (int64_t i = 0; i < lv.n; ++i) {
            st ^= st << 13; st ^= st >> 7; st ^= st << 17;
            y0[i] = 0.5f + (float)((double)(st >> 11) / (double)(1ull << 53));
        }
        DBuf<float> y, ay, z;
        DBuf<double> acc(2);
        y.upload(y0, s);
        ay.alloc(lv.n);
        z.alloc(lv.n);
        double hacc[2] = {1, 1};
        for (int it = 0; it < 30; ++it) {
            apply((int)L, y.p, ay.p, s);
            acc.zero(s);
            k_f_scale_dot<<<nb(lv.n), 256, 0, s>>>(lv.n, lv.dinv.p, ay.p, z.p, y.p, acc.p);
            TSEM_LAUNCHED();
            k_f_normalize<<<nb(lv.n), 256, 0, s>>>(lv.n, z.p, acc.p);
            TSEM_LAUNCHED();
            std::swap(y.p, z.p);
        }
        acc.download(hacc, 2, s);
        TSEM_CUDA(cudaStreamSynchronize(s));
        lv.lmax = 1.1 * std::sqrt(std::max(hacc[0], 1e-30));
        lv.lmin = lv.lmax / kChebRange;
    }
}

// ------------------------------------------------------------------ solver
MixedSolver::MixedSolver(tsem_space_s* sp, const DevCsr* A_, int dflag, const tsem_solver_opts& o, cudaStream_t s)
    : A(A_), opts(o) {
    smooth = std::max(1, o.smooth_steps);
    lowp = o.smoother == 2;
    op.build(sp, *A, dflag, std::max(1, o.pmg_order_step), s);
    trace_mark("op_build");
    // the outer residual's SpMV: a shape found for a matrix of the same kind serves
    spmv_autotune(const_cast<DevCsr&>(*A), s, true);
    trace_mark("autotune");
    const int64_t n = A->n;
    r64.alloc(n);
    rf.alloc(n); dsol.alloc(n); rw.alloc(n); z.alloc(n); p.alloc(n); q.alloc(n);
    sc.alloc(1);
    red.alloc(4);
    hsc = pinned_slot<PcgScalars>();
    TSEM_CUDA(cudaEventCreate(&ev0));
    TSEM_CUDA(cudaEventCreate(&ev1));
}

MixedSolver::~MixedSolver() {
    if (it_exec) cudaGraphExecDestroy(it_exec);
    for (auto& g : vc_graphs) cudaGraphExecDestroy(g.exec);
    trace_mark("graph_destroy");
    if (cap) cudaStreamDestroy(cap);
    if (hsc) pinned_slot<PcgScalars>(hsc);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
}

// Coefficients of a Chebyshev sweep of `steps` steps on a level (the first-kind
// polynomial of [lmin, lmax], three-term recurrence): the first direction is
// d_0 = s0 dinv r_0, and step k >= 1 sets d_k = a_k d_{k-1} + c_k dinv r_k after
// r_k = r_{k-1} - A d_{k-1}; the solution takes every d_k.
static void cheb_coef(const MfLevel& lv, int steps, double& s0, std::vector<double>& a, std::vector<double>& c) {
    a.assign(steps, 0.0);
    c.assign(steps, 0.0);
    const double theta = 0.5 * (lv.lmax + lv.lmin), delta = 0.5 * (lv.lmax - lv.lmin);
    s0 = 1.0 / theta;
    double rho_old = delta / theta;
    for (int k = 1; k < steps; ++k) {
        const double rho = 1.0 / (2.0 * theta / delta - rho_old);
        a[k] = rho * rho_old;
        c[k] = 2.0 * rho / delta;
        rho_old = rho;
    }
}

// Chebyshev smoothing of A x = rhs from the current x (x_zero: from x = 0, which
// spares the first apply); on matrix-free levels the vector updates ride on the
// scatter of each apply
void MixedSolver::chebyshev(MfLevel& lv, const float* rhs, int steps, const PcgScalars* st, cudaStream_t s,
                            bool x_zero, int ncol) {
    const int64_t n = lv.n;
    const dim3 g((unsigned)nb(n), (unsigned)ncol);
    double s0 = 1.0;
    std::vector<double> ca, cc;
    cheb_coef(lv, steps, s0, ca, cc);
    const int L = (int)(&lv - op.levels.data());
    if (lv.csr) {
        // one fused SpMV per step; directions alternate between t and ad, and the
        // solution takes each one a step late
        float* dc = lv.t.p;
        float* dn = lv.ad.p;
        if (x_zero) {
            k_f_cheb_zero<<<g, 256, 0, s>>>(n, lv.dinv.p, rhs, lv.v.p, dc, (float)s0, lv.xv, st, 1);
            TSEM_LAUNCHED();
        } else {
            MfPost f;
            f.rhs = rhs; f.v = lv.v.p; f.dinv = lv.dinv.p; f.a = (float)s0; f.st = st;
            op.spmv_cheb(L, MfPost::kChebFirst, lv.xv, f, dc, s, ncol);
        }
        for (int k = 1; k < steps; ++k) {
            MfPost c;
            c.v = lv.v.p; c.xs = lv.xv; c.dinv = lv.dinv.p; c.st = st;
            c.a = (float)ca[k]; c.c = (float)cc[k];
            op.spmv_cheb(L, MfPost::kChebStep, dc, c, dn, s, ncol);
            std::swap(dc, dn);
        }
        k_f_add<<<g, 256, 0, s>>>(n, lv.xv, dc, st);
        TSEM_LAUNCHED();
        return;
    }
    if (x_zero) {
        k_f_cheb_zero<<<g, 256, 0, s>>>(n, lv.dinv.p, rhs, lv.v.p, lv.t.p, (float)s0, lv.xv, st, 0);
        TSEM_LAUNCHED();
    } else {
        MfPost f;
        f.mode = MfPost::kChebFirst;
        f.rhs = rhs; f.v = lv.v.p; f.d = lv.t.p; f.dinv = lv.dinv.p; f.a = (float)s0; f.st = st;
        op.apply_post(L, lv.xv, f, s, lowp, ncol);
    }
    for (int k = 1; k < steps; ++k) {
        MfPost c;
        c.mode = MfPost::kChebStep;
        c.v = lv.v.p; c.xs = lv.xv; c.dinv = lv.dinv.p; c.st = st;
        c.a = (float)ca[k]; c.c = (float)cc[k];
        op.apply_post(L, lv.t.p, c, s, lowp, ncol);
    }
}

// Record the launches of `body` on the private capture stream into an executable
// graph (capture mode thread-local: other threads' CUDA calls are unaffected).  The
// launch counter counts the graph's kernels once per replay instead.
template <class F>
cudaGraphExec_t MixedSolver::capture(F&& body, long long& kernels) {
    device_limits();
    if (!cap) TSEM_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    const long long k0 = g_kernel_launches.load();
    TSEM_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    cudaGraph_t g = nullptr;
    try {
        body(cap);
    } catch (...) {
        cudaStreamEndCapture(cap, &g);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    TSEM_CUDA(cudaStreamEndCapture(cap, &g));
    kernels = g_kernel_launches.load() - k0;
    g_kernel_launches.fetch_sub(kernels);
    cudaGraphExec_t ex = nullptr;
    const cudaError_t rc = cudaGraphInstantiate(&ex, g, 0);
    cudaGraphDestroy(g);
    TSEM_CUDA(rc);
    return ex;
}

void MixedSolver::replay(cudaGraphExec_t ex, long long kernels, cudaStream_t s) {
    TSEM_CUDA(cudaGraphLaunch(ex, s));
    g_kernel_launches.fetch_add(kernels);
}

// level vectors for block V-cycles of ncol columns (n_level apart); the captured
// graphs hold the old vectors and are dropped
void MixedSolver::ensure_columns(int ncol, cudaStream_t s) {
    if (ncol <= cols) return;
    TSEM_CUDA(cudaStreamSynchronize(s));
    if (it_exec) {
        cudaGraphExecDestroy(it_exec);
        it_exec = nullptr;
    }
    for (auto& g : vc_graphs) cudaGraphExecDestroy(g.exec);
    vc_graphs.clear();
    for (auto& lv : op.levels) {
        const size_t m = (size_t)lv.n * ncol;
        lv.x.alloc(m); lv.r.alloc(m); lv.v.alloc(m); lv.t.alloc(m); lv.ad.alloc(m);
        lv.xv = lv.x.p;
    }
    op.ensure_columns(ncol);
    cols = ncol;
}

void MixedSolver::vcycle_graph(const float* r0, float* x0, cudaStream_t s, int ncol) {
    ensure_columns(ncol, s);
    for (auto& g : vc_graphs)
        if (g.r == r0 && g.x == x0 && g.ncol == ncol) {
            replay(g.exec, g.kernels, s);
            return;
        }
    if (vc_graphs.size() >= 8) {   // keep the few most recent vector pairs
        cudaGraphExecDestroy(vc_graphs.front().exec);
        vc_graphs.erase(vc_graphs.begin());
    }
    VcGraph g{r0, x0, ncol, nullptr, 0};
    g.exec = capture([&](cudaStream_t c) { vcycle(r0, x0, nullptr, c, ncol); }, g.kernels);
    vc_graphs.push_back(g);
    replay(g.exec, g.kernels, s);
}

// z = V-cycle(r) from z = 0
void MixedSolver::vcycle(const float* r0, float* x0, const PcgScalars* st, cudaStream_t s, int ncol) {
    if (ncol > cols) throw Error(TSEM_INVALID, "block V-cycle wider than the solver's level vectors");
    auto& lv0 = op.levels[0];
    lv0.xv = x0;
    const int nlv = (int)op.levels.size();
    for (int L = 0; L + 1 < nlv; ++L) {
        MfLevel& lv = op.levels[L];
        const float* rhs = L == 0 ? r0 : lv.r.p;
        chebyshev(lv, rhs, smooth, st, s, true, ncol);
        // the residual restricted to the coarser level only feeds the preconditioner:
        // the smoother's operator precision suffices
        MfPost f;
        f.mode = MfPost::kResid;
        f.rhs = rhs; f.v = lv.v.p; f.st = st;
        if (!lv.csr) op.apply_post(L, lv.xv, f, s, lowp, ncol);
        else op.spmv_cheb(L, MfPost::kResid, lv.xv, f, nullptr, s, ncol);
        MfLevel& c = op.levels[L + 1];
        k_f_restrict<<<dim3((unsigned)nb(lv.n), (unsigned)ncol), 256, 0, s>>>(lv.n, c.n, lv.core.p, lv.v.p, c.r.p, st);
        TSEM_LAUNCHED();
    }
    MfLevel& cl = op.levels[nlv - 1];
    chebyshev(cl, nlv == 1 ? r0 : cl.r.p, 4 * smooth, st, s, true, ncol);
    for (int L = nlv - 2; L >= 0; --L) {
        MfLevel& lv = op.levels[L];
        const float* rhs = L == 0 ? r0 : lv.r.p;
        k_f_prolong<<<dim3((unsigned)nb(lv.n), (unsigned)ncol), 256, 0, s>>>(lv.n, op.levels[L + 1].n, lv.core.p,
                                                                             op.levels[L + 1].xv, lv.xv, st);
        TSEM_LAUNCHED();
        chebyshev(lv, rhs, smooth, st, s, false, ncol);
    }
    TSEM_LAUNCH_CHECK();
    lv0.xv = lv0.x.p;
}

// the start of an inner solve of A d = rhs: state on the device, r = rhs, d = 0,
// z = V-cycle(r), p = z (the iterations follow, alone or in a group)
void MixedSolver::inner_begin(const float* rhs, float* dsol, cudaStream_t s) {
    const int64_t n = A->n;
    std::memset(hsc, 0, sizeof(PcgScalars));
    hsc->tol_rel2 = inner_rel * inner_rel;
    hsc->max_iter = inner_max;
    TSEM_CUDA(cudaMemcpyAsync(sc.p, hsc, sizeof(PcgScalars), cudaMemcpyHostToDevice, s));
    PcgScalars* st = sc.p;
    float* r = rw.p;
    TSEM_CUDA(cudaMemcpyAsync(r, rhs, n * sizeof(float), cudaMemcpyDeviceToDevice, s));
    k_f_zero<<<nb(n), 256, 0, s>>>(n, dsol, nullptr);
    TSEM_LAUNCHED();
    vcycle(r, z.p, nullptr, s);
    k_in_init<<<nb(n), 256, 0, s>>>(n, r, z.p, p.p, st);
    TSEM_LAUNCHED();
}

// solve A d = rhs (FP32, d from zero) to relative residual inner_tol; returns iterations
int MixedSolver::inner_pcg(const float* rhs, float* dsol, cudaStream_t s) {
    const int64_t n = A->n;
    inner_begin(rhs, dsol, s);
    PcgScalars* st = sc.p;
    float* r = rw.p;
    // one iteration: operator, the two PCG updates, the V-cycle, the new direction;
    // captured once as a graph (its vectors and scalars are the solver's own)
    if (!it_exec)
        it_exec = capture(
            [&](cudaStream_t c) {
                op.apply(0, p.p, q.p, c);
                k_in_pq<<<nb(n), 256, 0, c>>>(n, p.p, q.p, st);
                TSEM_LAUNCHED();
                k_in_update<<<nb(n), 256, 0, c>>>(n, dsol, r, p.p, q.p, st);
                TSEM_LAUNCHED();
                vcycle(r, z.p, st, c);
                k_in_rz<<<nb(n), 256, 0, c>>>(n, r, z.p, st);
                TSEM_LAUNCHED();
                k_in_p<<<nb(n), 256, 0, c>>>(n, p.p, z.p, st);
                TSEM_LAUNCHED();
            },
            it_kernels);
    for (;;) {
        replay(it_exec, it_kernels, s);
        TSEM_CUDA(cudaMemcpyAsync(hsc, sc.p, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s));
        TSEM_CUDA(cudaStreamSynchronize(s));
        if (hsc->done) break;
    }
    return hsc->iter;
}

// iterative refinement: r = b - A x (FP64 CSR), A d = r / |r| (FP32, matrix-free), x += |r| d
void MixedSolver::solve(const double* b, double* x, tsem_stats* out, cudaStream_t s) {
    const int64_t n = A->n;
    TSEM_CUDA(cudaEventRecord(ev0, s));
    double hbx[2] = {0, 0}, hr = 0;
    red.zero(s);
    k_norm_nz<<<nb(n), 256, 0, s>>>(n, b, x, red.p);
    TSEM_LAUNCHED();
    red.download(hbx, 2, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    const double hb = hbx[0];
    const double bn = std::sqrt(hb);
    // x = 0 (the usual start): the first residual is b itself, without the SpMV
    bool x_zero = hbx[1] == 0.0;
    const double tol = opts.tol_rel > 0 ? opts.tol_rel : 1e-10;
    const int max_outer = opts.max_iter > 0 ? std::min(opts.max_iter, 60) : 60;
    int outer = 0, inner_total = 0, status = TSEM_MAXIT;
    double rel = 1.0;
    for (;;) {
        if (x_zero) {
            TSEM_CUDA(cudaMemcpyAsync(r64.p, b, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s));
            hr = hb;
            x_zero = false;
        } else {
            csr_residual(*A, x, r64.p, b, s);
            red.zero(s);
            k_norms<<<nb(n), 256, 0, s>>>(n, r64.p, red.p);
            TSEM_LAUNCHED();
            red.download(&hr, 1, s);
            TSEM_CUDA(cudaStreamSynchronize(s));
        }
        const double rn = std::sqrt(hr);
        rel = bn > 0 ? rn / bn : rn;
        if (!std::isfinite(rel)) { status = TSEM_NONFINITE; break; }
        if (rel <= tol) { status = TSEM_OK; break; }
        if (outer >= max_outer) { status = TSEM_MAXIT; break; }
        k_to_f32<<<nb(n), 256, 0, s>>>(n, r64.p, 1.0 / rn, rf.p);
        TSEM_LAUNCHED();
        // the inner solve reduces the residual by inner_tol, or by just enough to
        // reach the target when that is less (with a safety factor of 0.3)
        inner_rel = std::min(1e-2, std::max(inner_tol, 0.3 * tol / rel));
        inner_total += inner_pcg(rf.p, dsol.p, s);
        int herr_inner = 0;                       // a bounded wait gave up: reported below
        op.err.download(&herr_inner, 1, s);
        TSEM_CUDA(cudaStreamSynchronize(s));
        if (herr_inner) break;
#ifdef TSEM_CHECK
        {
            CheckState hc{};
            TSEM_CUDA(cudaMemcpyFromSymbol(&hc, g_check, sizeof(hc)));
            if (hc.code)
                throw Error(TSEM_INVALID, "bounds check failed in the matrix-free operator (check " +
                                              std::to_string(hc.code) + ", index " + std::to_string(hc.index) + ")");
        }
#endif
        if (hsc->status == TSEM_NONFINITE || hsc->status == TSEM_BREAKDOWN) { status = hsc->status; break; }
        k_axpy_f32<<<nb(n), 256, 0, s>>>(n, rn, dsol.p, x);
        TSEM_LAUNCHED();
        ++outer;
    }
    last_outer = outer;
    last_inner = inner_total;
    int herr = 0;
    op.err.download(&herr, 1, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    if (herr) {
        op.err.zero(s);
        throw Error(TSEM_TIMEOUT, "a bounded wait of the matrix-free apply gave up (code " + std::to_string(herr) + ")");
    }
    TSEM_CUDA(cudaEventRecord(ev1, s));
    TSEM_CUDA(cudaEventSynchronize(ev1));
    float ms = 0;
    TSEM_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    if (out) {
        out->iterations = inner_total;
        out->status = status;
        out->residual_l1 = 0;
        out->init_l1 = outer;
        out->residual_rel = rel;
        out->device_ms = ms;
    }
}

}  // namespace tsem

namespace tsem {

// ------------------------------------------------ allocation-free FP32 apply
// A variant of the FP32 matrix-free apply for callers that may not allocate
// device memory while they run: a host whose device memory is fully handed to
// its own pool, or a serving loop that must not take the device-wide
// synchronisation a cudaMalloc/cudaFree can imply.  The gathered tiles, the
// per-element results and the wait-failure flag live in one fixed static device
// array instead of the operator's own buffers.  Layout of the array (floats):
//   [0, 64)              failure flag (an int in the first word), reset by every call
//   [64, 64 + u)         gathered tiles U[tile][j][64], u = E_pad * nl rounded up to 64
//   [64 + u, 64 + 2u)    per-element results V[i][e]
// Neither tile area needs to start at zero: the gather writes every tile entry
// (zero past the last element) and the scatter reads only results the GEMM wrote.
// All calls on a device share the one array, so calls that overlap in time (two
// streams, or two solvers) race on it; order them on one stream or with events.
static __device__ __align__(256) float g_noalloc_scratch[kNoAllocScratchBytes / sizeof(float)];

namespace {
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
float* g_noalloc_ptr[kNoAllocMaxDevices] = {};
}  // namespace

// once per device, with that device current: the device address of the array
// (cudaGetSymbolAddress may set up the module, so the first call on a device
// belongs before any stream capture)
static float* noalloc_scratch(int dev) {
    if (dev < 0 || dev >= kNoAllocMaxDevices) throw Error(TSEM_INVALID, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        TSEM_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
        g_noalloc_ptr[dev] = static_cast<float*>(p);
    }
    return g_noalloc_ptr[dev];
}

// y = NaN wherever a bounded wait of this call gave up, so that a failed call
// is visible in its result without a host synchronisation
__global__ void k_nan_on_err(int64_t n, const int* __restrict__ err, float* y) {
    if (*err == 0) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = __int_as_float(0x7fc00000);
}

size_t mf_noalloc_need_bytes(const MfOperator& op, int level) {
    const MfLevel& L = op.levels[level];
    const size_t E_pad = (size_t)((op.E + kTileE - 1) / kTileE) * kTileE;
    const size_t u = (E_pad * (size_t)L.nl + 63) / 64 * 64;
    return (64 + 2 * u) * sizeof(float);
}

void mf_apply_noalloc(const MfOperator& op, int level, const float* x, float* y, cudaStream_t s) {
    const MfLevel& L = op.levels[level];
    const size_t need = mf_noalloc_need_bytes(op, level);
    if (need > kNoAllocScratchBytes)
        throw Error(TSEM_INVALID, "level " + std::to_string(level) + " needs " + std::to_string(need) +
                                      " bytes of scratch; the allocation-free apply holds at most " +
                                      std::to_string(kNoAllocScratchBytes));
    int dev = 0;
    TSEM_CUDA(cudaGetDevice(&dev));
    float* base = noalloc_scratch(dev);
    const DevLimits& lim = device_limits();
    const int E = op.E;
    const int n_tiles = (E + kTileE - 1) / kTileE;
    const int E_pad = n_tiles * kTileE;
    const size_t u = ((size_t)E_pad * L.nl + 63) / 64 * 64;
    int* err = reinterpret_cast<int*>(base);
    float* U = base + 64;
    float* V = U + u;
    TSEM_CUDA(cudaMemsetAsync(err, 0, sizeof(int), s));
    TSEM_CUDA(cudaMemsetAsync(y, 0, L.n * sizeof(float), s));
    k_gather_f32<<<grid_for((int64_t)E_pad * L.nl, 256), 256, 0, s>>>(E, E_pad, L.nl, L.md, L.gi.p, L.gv.p, x, L.n, U);
    TSEM_LAUNCHED();
    const size_t fixed = 2 * (size_t)L.nl * kTileE * sizeof(float);
    int rows = L.nl;
    while (rows > 2 && fixed + (size_t)L.nl * ((rows + 1) & ~1) * 6 * sizeof(float) > lim.smem_optin) rows = (rows + 1) / 2;
    for (int r0 = 0; r0 < L.nl; r0 += rows) {
        const int cnt = std::min(rows, L.nl - r0);
        const size_t shm = fixed + (size_t)L.nl * ((cnt + 1) & ~1) * 6 * sizeof(float);
        k_mf_apply<<<std::min(n_tiles, lim.sms), kApplyThreads, shm, s>>>(E, L.nl, L.nlp, L.md, r0, cnt, L.gi.p, L.gv.p,
                                                                             op.w6.p, L.S.p, U, V, 1, E_pad, err);
        TSEM_LAUNCHED();
    }
    k_scatter<<<grid_for((int64_t)E * L.nl, 256), 256, 0, s>>>(E, E_pad, L.nl, L.md, L.gi.p, L.gv.p, V, y, L.n);
    TSEM_LAUNCHED();
    if (L.bnd.n) {
        k_bnd_fix<<<nb(L.bnd.n), 256, 0, s>>>((int64_t)L.bnd.n, L.bnd.p, L.bnd_diag.p, x, y);
        TSEM_LAUNCHED();
    }
    k_nan_on_err<<<nb(L.n), 256, 0, s>>>((int64_t)L.n, err, y);
    TSEM_LAUNCHED();
}

// ============================================================== groups of solves
// Several mixed solvers of the same order run their inner PCG iterations together:
// each step of the V-cycle is one launch over a ragged table of all members' levels
// (GroupLevel, one entry per member and a sentinel whose g0 is the total; a thread
// finds its member by binary search over g0), the BF16 element GEMM one launch over
// all members' element tiles (TcgOp).  The arithmetic per DOF and per element is the
// single solver's.

__device__ __forceinline__ int grp_find(const GroupLevel* __restrict__ T, int nops, int64_t g) {
    int lo = 0, hi = nops - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (T[mid].g0 <= g) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Chebyshev start from x = 0: v = rhs, t = s0 dinv rhs, x = t (x = 0 on assembled
// levels, which add each direction a step late) -- k_f_cheb_zero per member
__global__ void k_grp_cheb_zero(const GroupLevel* __restrict__ T, int nops, int64_t total, int deferred) {
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x) {
        const GroupLevel& L = T[grp_find(T, nops, g)];
        if (L.st && L.st->done) continue;
        const int64_t j = g - L.g0;
        const float r = L.rhs[j];
        L.v[j] = r;
        const float d = L.dinv[j] * r * L.s0;
        L.t[j] = d;
        L.x[j] = deferred ? 0.0f : d;
    }
}

// the transposed scatter of the members' element results with the update MODE fused
// in (k_scatter_t on unit levels): kResid v = rhs - A x; kChebFirst v = rhs - A x,
// t = s0 dinv v, x += t; kChebStep (step k) v -= A t, t = a_k t + c_k dinv v, x += t
template <int MODE>
__global__ void k_grp_scatter(const GroupLevel* __restrict__ T, int nops, int64_t total, int k) {
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x) {
        const GroupLevel& L = T[grp_find(T, nops, g)];
        if (L.st && L.st->done) continue;
        const int64_t j = g - L.g0;
        float* xa = MODE == MfPost::kChebStep ? L.t : L.x;   // the applied vector
        const int b = L.trp[j], e = L.trp[j + 1];
        const float acc = b == e ? L.bdiag[j] * xa[j] : scatter_row<true>(b, e, L.tpos, nullptr, L.V, L.vlen);
        if (MODE == MfPost::kResid) {
            L.v[j] = L.rhs[j] - acc;
        } else if (MODE == MfPost::kChebFirst) {
            const float v = L.rhs[j] - acc;
            L.v[j] = v;
            const float d = L.dinv[j] * v * L.s0;
            L.t[j] = d;
            L.x[j] += d;
        } else {
            const float v = L.v[j] - acc;
            L.v[j] = v;
            const float d = L.a[k] * xa[j] + L.c[k] * L.dinv[j] * v;
            xa[j] = d;
            L.x[j] += d;
        }
    }
}

// assembled levels: A x with the row update MODE fused in (k_spmv_f32_cheb per
// member); the directions alternate between t and ad, step k reading t when k is odd
template <int TPR, int MODE>
__global__ void k_grp_spmv_cheb(const GroupLevel* __restrict__ T, int nops, int64_t total, int k) {
    const int64_t gr = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / TPR;
    const int lane = threadIdx.x % TPR;
    const GroupLevel* L = gr < total ? &T[grp_find(T, nops, gr)] : nullptr;
    // rows of several members may share a warp: no early return before the shuffle
    const bool live = L && !(L->st && L->st->done);
    const int64_t j = live ? gr - L->g0 : 0;
    const float* xa = !live ? nullptr : MODE == MfPost::kChebStep ? ((k & 1) ? L->t : L->ad) : L->x;
    float acc = 0.0f;
    if (live)
        for (int64_t q = L->crp[j] + lane; q < L->crp[j + 1]; q += TPR)
            if (in_bounds(L->ccol[q], L->n, 38)) acc += L->cval[q] * __ldg(xa + L->ccol[q]);
#pragma unroll
    for (int o = TPR / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o, TPR);
    if (!live || lane != 0) return;
    if (MODE == MfPost::kResid) {
        L->v[j] = L->rhs[j] - acc;
    } else if (MODE == MfPost::kChebFirst) {
        const float v = L->rhs[j] - acc;
        L->v[j] = v;
        L->t[j] = L->s0 * L->dinv[j] * v;
    } else {
        const float v = L->v[j] - acc;
        L->v[j] = v;
        const float d = xa[j];
        L->x[j] += d;
        float* dn = (k & 1) ? L->ad : L->t;
        dn[j] = L->a[k] * d + L->c[k] * L->dinv[j] * v;
    }
}

// x += the last direction of an assembled level's sweep
__global__ void k_grp_f_add(const GroupLevel* __restrict__ T, int nops, int64_t total, int use_ad) {
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x) {
        const GroupLevel& L = T[grp_find(T, nops, g)];
        if (L.st && L.st->done) continue;
        const int64_t j = g - L.g0;
        L.x[j] += use_ad ? L.ad[j] : L.t[j];
    }
}
// injection to the next coarser level: rc[core[j]] = v[j]
__global__ void k_grp_restrict(const GroupLevel* __restrict__ T, int nops, int64_t total) {
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x) {
        const GroupLevel& L = T[grp_find(T, nops, g)];
        if (L.st && L.st->done) continue;
        const int64_t j = g - L.g0;
        const int c = L.core[j];
        if (c >= 0) L.rc[c] = L.v[j];
    }
}
// x[j] += xc[core[j]]
__global__ void k_grp_prolong(const GroupLevel* __restrict__ T, int nops, int64_t total) {
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x) {
        const GroupLevel& L = T[grp_find(T, nops, g)];
        if (L.st && L.st->done) continue;
        const int64_t j = g - L.g0;
        const int c = L.core[j];
        if (c >= 0) L.x[j] += L.xc[c];
    }
}
// the inner PCG's vector updates of every member (blockIdx.y): phase 0 p.q, 1 x and r,
// 2 r.z, 3 the new direction and the test
__global__ void k_grp_pcg(int phase, const GroupPcg* __restrict__ P) {
    const GroupPcg& g = P[blockIdx.y];
    if (phase == 0) in_pq(g.n, g.p, g.q, g.st);
    else if (phase == 1) in_update(g.n, g.x, g.r, g.p, g.q, g.st);
    else if (phase == 2) in_rz(g.n, g.r, g.z, g.st);
    else in_p(g.n, g.p, g.z, g.st);
}

void group_elements(const MfLevel& L, const TcgOp* ops, int nops, int units, int* err, cudaStream_t s) {
    const size_t shm = (size_t)(512 + 2 * kTileT) * L.kpad * 2 + epi_bytes(L.nl);
    k_mf_apply_tcg<<<std::min(units, device_limits().sms), kTgThreads, shm, s>>>(
        0, L.nl, L.nl4, L.kpad, nullptr, nullptr, nullptr, L.Bt.p, nullptr, err, 1, 0, 0, ops, nops, units, nullptr, 0);
    TSEM_LAUNCHED();
}
void group_cheb_zero(const GroupLevel* T, int nops, int64_t total, bool deferred, cudaStream_t s) {
    k_grp_cheb_zero<<<nb(total), 256, 0, s>>>(T, nops, total, deferred ? 1 : 0);
    TSEM_LAUNCHED();
}
void group_scatter(int mode, int k, const GroupLevel* T, int nops, int64_t total, cudaStream_t s) {
    if (mode == MfPost::kResid) k_grp_scatter<MfPost::kResid><<<nb(total), 256, 0, s>>>(T, nops, total, k);
    else if (mode == MfPost::kChebFirst) k_grp_scatter<MfPost::kChebFirst><<<nb(total), 256, 0, s>>>(T, nops, total, k);
    else k_grp_scatter<MfPost::kChebStep><<<nb(total), 256, 0, s>>>(T, nops, total, k);
    TSEM_LAUNCHED();
}
void group_spmv_cheb(int tpr, int mode, int k, const GroupLevel* T, int nops, int64_t total, cudaStream_t s) {
    const unsigned g = (unsigned)((total * tpr + 255) / 256);
#define TSEM_GRP_SPMV(TP)                                                                                          \
    if (mode == MfPost::kResid) k_grp_spmv_cheb<TP, MfPost::kResid><<<g, 256, 0, s>>>(T, nops, total, k);          \
    else if (mode == MfPost::kChebFirst) k_grp_spmv_cheb<TP, MfPost::kChebFirst><<<g, 256, 0, s>>>(T, nops, total, k); \
    else k_grp_spmv_cheb<TP, MfPost::kChebStep><<<g, 256, 0, s>>>(T, nops, total, k);
    switch (tpr) {
        case 2: { TSEM_GRP_SPMV(2) } break;
        case 4: { TSEM_GRP_SPMV(4) } break;
        case 8: { TSEM_GRP_SPMV(8) } break;
        case 16: { TSEM_GRP_SPMV(16) } break;
        default: { TSEM_GRP_SPMV(32) } break;
    }
#undef TSEM_GRP_SPMV
    TSEM_LAUNCHED();
}
void group_f_add(bool use_ad, const GroupLevel* T, int nops, int64_t total, cudaStream_t s) {
    k_grp_f_add<<<nb(total), 256, 0, s>>>(T, nops, total, use_ad ? 1 : 0);
    TSEM_LAUNCHED();
}
void group_restrict(const GroupLevel* T, int nops, int64_t total, cudaStream_t s) {
    k_grp_restrict<<<nb(total), 256, 0, s>>>(T, nops, total);
    TSEM_LAUNCHED();
}
void group_prolong(const GroupLevel* T, int nops, int64_t total, cudaStream_t s) {
    k_grp_prolong<<<nb(total), 256, 0, s>>>(T, nops, total);
    TSEM_LAUNCHED();
}
void group_pcg(int phase, const GroupPcg* P, int nops, int64_t nmax, cudaStream_t s) {
    k_grp_pcg<<<dim3((unsigned)nb(nmax), (unsigned)nops), 256, 0, s>>>(phase, P);
    TSEM_LAUNCHED();
}

// every matrix-free level takes the fused-gather BF16 GEMM (unit transforms, tensor
// cores, BF16 smoother), and the Chebyshev sweeps fit a group record
bool groupable(const MixedSolver& S) {
    if (!S.lowp) return false;
    const int nlv = (int)S.op.levels.size();
    for (int L = 0; L < nlv; ++L) {
        const MfLevel& lv = S.op.levels[L];
        if (!lv.csr && !(lv.unit && lv.tc)) return false;
    }
    return 4 * S.smooth <= kChebMax;
}

// levels of the same sizes per element and the same kind: one group launch serves both
bool same_shape(const MixedSolver& a, const MixedSolver& b) {
    if (a.smooth != b.smooth || a.op.levels.size() != b.op.levels.size() || a.op.M != b.op.M) return false;
    for (size_t L = 0; L < a.op.levels.size(); ++L) {
        const MfLevel &x = a.op.levels[L], &y = b.op.levels[L];
        if (x.csr != y.csr || x.nl != y.nl || x.kpad != y.kpad || x.nl4 != y.nl4 || x.unit != y.unit || x.tc != y.tc)
            return false;
    }
    return true;
}

// The tables and the round of one membership.  A group object is reused as members
// come and go: its device tables only grow, a new membership rewrites them
// (asynchronous uploads, no allocation once grown), and the round is launched
// directly until the same members have run two rounds together; then it is
// captured once as a CUDA graph and replayed while the membership holds.
struct MixedGroup {
    std::vector<int64_t> key;                   // the members' tickets
    int stable = 0;                             // rounds run with these members
    std::vector<MixedSolver*> m;
    int nlv = 0, nops = 0;
    std::vector<DBuf<GroupLevel>> lv;           // per level: nops entries and the sentinel
    std::vector<int64_t> total;                 // DOFs of a level over all members
    std::vector<DBuf<TcgOp>> ops_x, ops_t;      // element GEMM tables applying x / t
    std::vector<int> units;                     // element tiles of a level over all members
    std::vector<int> tpr;                       // lanes per row of assembled levels
    DBuf<GroupPcg> pcg;
    int64_t nmax = 0;
    DBuf<int> err;                              // a bounded wait of a group GEMM gave up
    cudaGraphExec_t exec = nullptr;
    long long kernels = 0;

    ~MixedGroup() {
        if (exec) cudaGraphExecDestroy(exec);
    }

    void build(const std::vector<MixedSolver*>& members, cudaStream_t s) {
        if (exec) {
            cudaGraphExecDestroy(exec);
            exec = nullptr;
        }
        stable = 0;
        m = members;
        nops = (int)m.size();
        if (nops < 1 || nops > kGroupMax) throw Error(TSEM_INVALID, "group size out of range");
        nlv = (int)m[0]->op.levels.size();
        lv.resize(nlv);
        ops_x.resize(nlv);
        ops_t.resize(nlv);
        total.assign(nlv, 0);
        units.assign(nlv, 0);
        tpr.assign(nlv, 8);
        for (int L = 0; L < nlv; ++L) {
            std::vector<GroupLevel> T(nops + 1);
            std::vector<TcgOp> ox(nops), ot(nops);
            const int steps = L == nlv - 1 ? 4 * m[0]->smooth : m[0]->smooth;
            int64_t g0 = 0;
            int tile0 = 0;
            for (int i = 0; i < nops; ++i) {
                MixedSolver& S = *m[i];
                MfLevel& l = S.op.levels[L];
                GroupLevel& G = T[i];
                G = GroupLevel{};
                G.g0 = g0;
                G.n = l.n;
                G.trp = l.trp.p; G.tpos = l.tpos.p; G.V = S.op.Vbuf.p; G.vlen = S.op.vcol; G.bdiag = l.bdiag.p;
                G.crp = l.crp.p; G.ccol = l.ccol.p; G.cval = l.cval.p; G.dinv = l.dinv.p;
                G.rhs = L == 0 ? S.rw.p : l.r.p;
                G.x = L == 0 ? S.z.p : l.x.p;
                G.t = l.t.p; G.ad = l.ad.p; G.v = l.v.p;
                G.core = l.core.p;
                G.rc = L + 1 < nlv ? S.op.levels[L + 1].r.p : nullptr;
                G.xc = L + 1 < nlv ? S.op.levels[L + 1].x.p : nullptr;
                G.st = S.sc.p;
                double s0 = 1.0;
                std::vector<double> ca, cc;
                cheb_coef(l, steps, s0, ca, cc);
                G.s0 = (float)s0;
                for (int k = 0; k < steps; ++k) { G.a[k] = (float)ca[k]; G.c[k] = (float)cc[k]; }
                g0 += l.n;
                if (!l.csr) {
                    const int tiles = (S.op.E + kTileT - 1) / kTileT;
                    ox[i] = TcgOp{l.gp.p, G.x, S.op.w6.p, S.op.Vbuf.p, l.n, S.op.E, tile0};
                    ot[i] = TcgOp{l.gp.p, l.t.p, S.op.w6.p, S.op.Vbuf.p, l.n, S.op.E, tile0};
                    tile0 += tiles;
                }
            }
            T[nops] = GroupLevel{};
            T[nops].g0 = g0;
            total[L] = g0;
            units[L] = tile0;
            tpr[L] = m[0]->op.levels[L].csr_tpr;
            lv[L].upload(T, s);
            if (!m[0]->op.levels[L].csr) {
                ops_x[L].upload(ox, s);
                ops_t[L].upload(ot, s);
            }
        }
        std::vector<GroupPcg> P(nops);
        nmax = 0;
        for (int i = 0; i < nops; ++i) {
            MixedSolver& S = *m[i];
            P[i] = GroupPcg{S.A->n, S.dsol.p, S.rw.p, S.p.p, S.q.p, S.z.p, S.sc.p};
            nmax = std::max(nmax, S.A->n);
        }
        pcg.upload(P, s);
        if (!err.p) err.alloc(1);
        err.zero(s);
    }

    // one round on s: direct launches, or the graph once the membership has held
    // (captured on `cap`, a stream of the engine)
    void run(cudaStream_t s, cudaStream_t cap) {
        if (!exec && stable >= 2) {
            const long long k0 = g_kernel_launches.load();
            TSEM_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
            cudaGraph_t g = nullptr;
            try {
                iteration(cap);
            } catch (...) {
                cudaStreamEndCapture(cap, &g);
                if (g) cudaGraphDestroy(g);
                throw;
            }
            TSEM_CUDA(cudaStreamEndCapture(cap, &g));
            kernels = g_kernel_launches.load() - k0;
            g_kernel_launches.fetch_sub(kernels);
            const cudaError_t rc = cudaGraphInstantiate(&exec, g, 0);
            cudaGraphDestroy(g);
            TSEM_CUDA(rc);
        }
        if (exec) {
            TSEM_CUDA(cudaGraphLaunch(exec, s));
            g_kernel_launches.fetch_add(kernels);
        } else {
            iteration(s);
        }
        ++stable;
    }

   private:
    void chebyshev(int L, int steps, bool x_zero, cudaStream_t c) {
        const GroupLevel* T = lv[L].p;
        const MfLevel& l0 = m[0]->op.levels[L];
        if (l0.csr) {
            if (x_zero) group_cheb_zero(T, nops, total[L], true, c);
            else group_spmv_cheb(tpr[L], MfPost::kChebFirst, 0, T, nops, total[L], c);
            for (int k = 1; k < steps; ++k) group_spmv_cheb(tpr[L], MfPost::kChebStep, k, T, nops, total[L], c);
            group_f_add(((steps - 1) & 1) != 0, T, nops, total[L], c);
            return;
        }
        if (x_zero) {
            group_cheb_zero(T, nops, total[L], false, c);
        } else {
            group_elements(l0, ops_x[L].p, nops, units[L], err.p, c);
            group_scatter(MfPost::kChebFirst, 0, T, nops, total[L], c);
        }
        for (int k = 1; k < steps; ++k) {
            group_elements(l0, ops_t[L].p, nops, units[L], err.p, c);
            group_scatter(MfPost::kChebStep, k, T, nops, total[L], c);
        }
    }
    // z = V-cycle(r) of every member (MixedSolver::vcycle)
    void vcycle(cudaStream_t c) {
        const int smooth = m[0]->smooth;
        for (int L = 0; L + 1 < nlv; ++L) {
            chebyshev(L, smooth, true, c);
            const MfLevel& l0 = m[0]->op.levels[L];
            if (!l0.csr) {
                group_elements(l0, ops_x[L].p, nops, units[L], err.p, c);
                group_scatter(MfPost::kResid, 0, lv[L].p, nops, total[L], c);
            } else {
                group_spmv_cheb(tpr[L], MfPost::kResid, 0, lv[L].p, nops, total[L], c);
            }
            group_restrict(lv[L].p, nops, total[L], c);
        }
        chebyshev(nlv - 1, 4 * smooth, true, c);
        for (int L = nlv - 2; L >= 0; --L) {
            group_prolong(lv[L].p, nops, total[L], c);
            chebyshev(L, smooth, false, c);
        }
    }
    // one inner iteration of every member (the body of MixedSolver::inner_pcg)
    void iteration(cudaStream_t c) {
        for (MixedSolver* S : m) S->op.apply(0, S->p.p, S->q.p, c);   // Krylov operator, FP32-accurate
        group_pcg(0, pcg.p, nops, nmax, c);
        group_pcg(1, pcg.p, nops, nmax, c);
        vcycle(c);
        group_pcg(2, pcg.p, nops, nmax, c);
        group_pcg(3, pcg.p, nops, nmax, c);
    }
};

// ---- continuous batching.  An entry follows MixedSolver::solve step by step: the
// FP64 refinement steps run per system between rounds, the inner iterations in the
// groups' rounds.
struct BatchEngine::Entry {
    int64_t ticket = 0;
    BatchItem* it = nullptr;
    int phase = 0;                 // 0 waiting, 1 in an inner solve, 2 retired
    bool cancelled = false, x_zero = false;
    double hb = 0, bn = 0, rn = 0, rel = 1, tol = 1e-10;
    int outer = 0, inner_total = 0, max_outer = 60, status = TSEM_MAXIT;
    cudaEvent_t start = nullptr, end = nullptr;
    ~Entry() {
        if (start) cudaEventDestroy(start);
        if (end) cudaEventDestroy(end);
    }
};

BatchEngine::BatchEngine(cudaStream_t s_) : s(s_) {}
BatchEngine::~BatchEngine() {
    slots.clear();
    if (cap) cudaStreamDestroy(cap);
}

int64_t BatchEngine::submit(BatchItem* it) {
    auto e = std::make_unique<Entry>();
    e->ticket = ++last_ticket;
    e->it = it;
    pending.push_back(std::move(e));
    return last_ticket;
}

bool BatchEngine::cancel(int64_t ticket) {
    for (auto& e : pending)
        if (e->ticket == ticket) { e->cancelled = true; return true; }
    for (auto& e : active)
        if (e->ticket == ticket && e->phase != 2) { e->cancelled = true; return true; }
    return false;
}

int BatchEngine::in_flight() const { return (int)(pending.size() + active.size()); }

// the FP64 residual of an entry and the next inner solve, or its end
static void batch_outer_step(BatchEngine::Entry& e, cudaStream_t s) {
    MixedSolver& S = *e.it->S;
    const int64_t n = S.A->n;
    double hr = 0.0;
    if (e.x_zero) {
        TSEM_CUDA(cudaMemcpyAsync(S.r64.p, e.it->b, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        hr = e.hb;
        e.x_zero = false;
    } else {
        csr_residual(*S.A, e.it->x, S.r64.p, e.it->b, s);
        S.red.zero(s);
        k_norms<<<nb(n), 256, 0, s>>>(n, S.r64.p, S.red.p);
        TSEM_LAUNCHED();
        S.red.download(&hr, 1, s);
        TSEM_CUDA(cudaStreamSynchronize(s));
    }
    const double rn = std::sqrt(hr);
    e.rel = e.bn > 0 ? rn / e.bn : rn;
    if (!std::isfinite(e.rel)) { e.status = TSEM_NONFINITE; e.phase = 2; return; }
    if (e.rel <= e.tol) { e.status = TSEM_OK; e.phase = 2; return; }
    if (e.outer >= e.max_outer) { e.status = TSEM_MAXIT; e.phase = 2; return; }
    k_to_f32<<<nb(n), 256, 0, s>>>(n, S.r64.p, 1.0 / rn, S.rf.p);
    TSEM_LAUNCHED();
    S.inner_rel = std::min(1e-2, std::max(S.inner_tol, 0.3 * e.tol / e.rel));
    S.inner_begin(S.rf.p, S.dsol.p, s);
    e.rn = rn;
    e.phase = 1;
}

std::vector<std::pair<int64_t, BatchItem*>> BatchEngine::round() {
    std::vector<std::pair<int64_t, BatchItem*>> done;
    auto retire = [&](Entry& e) {
        BatchItem& it = *e.it;
        float ms = 0.0f;
        if (e.start) {
            TSEM_CUDA(cudaEventCreate(&e.end));
            TSEM_CUDA(cudaEventRecord(e.end, s));
            TSEM_CUDA(cudaEventSynchronize(e.end));
            TSEM_CUDA(cudaEventElapsedTime(&ms, e.start, e.end));
        }
        it.stats = tsem_stats{};
        it.stats.iterations = e.inner_total;
        it.stats.status = e.status;
        it.stats.init_l1 = e.outer;
        it.stats.residual_rel = e.rel;
        it.stats.device_ms = ms;
        it.S->last_outer = e.outer;
        it.S->last_inner = e.inner_total;
        e.phase = 2;
        done.emplace_back(e.ticket, e.it);
    };
    // admit: systems no group launch serves solve on their own at once; the others
    // measure |b| and x's support and take their first refinement step
    while (!pending.empty()) {
        std::unique_ptr<Entry> e = std::move(pending.front());
        pending.pop_front();
        BatchItem& it = *e->it;
        if (e->cancelled) {
            e->status = TSEM_INVALID;
            retire(*e);
            continue;
        }
        if (!groupable(*it.S)) {
            it.S->solve(it.b, it.x, &it.stats, s);
            done.emplace_back(e->ticket, e->it);
            continue;
        }
        MixedSolver& S = *it.S;
        const int64_t n = S.A->n;
        TSEM_CUDA(cudaEventCreate(&e->start));
        TSEM_CUDA(cudaEventRecord(e->start, s));
        double hbx[2] = {0, 0};
        S.red.zero(s);
        k_norm_nz<<<nb(n), 256, 0, s>>>(n, it.b, it.x, S.red.p);
        TSEM_LAUNCHED();
        S.red.download(hbx, 2, s);
        TSEM_CUDA(cudaStreamSynchronize(s));
        e->hb = hbx[0];
        e->bn = std::sqrt(hbx[0]);
        e->x_zero = hbx[1] == 0.0;
        e->tol = S.opts.tol_rel > 0 ? S.opts.tol_rel : 1e-10;
        e->max_outer = S.opts.max_iter > 0 ? std::min(S.opts.max_iter, 60) : 60;
        batch_outer_step(*e, s);
        if (e->phase == 2) retire(*e);
        else active.push_back(std::move(e));
    }
    for (auto& e : active)
        if (e->phase == 1 && e->cancelled) { e->status = TSEM_INVALID; retire(*e); }
    // groups of the systems in an inner solve, one round each
    std::vector<std::vector<Entry*>> gs;
    for (auto& e : active) {
        if (e->phase != 1) continue;
        bool placed = false;
        for (auto& g : gs)
            if ((int)g.size() < kGroupMax && same_shape(*g[0]->it->S, *e->it->S)) { g.push_back(e.get()); placed = true; break; }
        if (!placed) gs.push_back({e.get()});
    }
    std::vector<MixedGroup*> ran;
    if (!gs.empty() && !cap) TSEM_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    for (size_t i = 0; i < gs.size(); ++i) {
        if (slots.size() <= i) slots.push_back(std::make_unique<MixedGroup>());
        MixedGroup& G = *slots[i];
        std::vector<int64_t> key;
        for (Entry* e : gs[i]) key.push_back(e->ticket);
        if (G.key != key) {
            std::vector<MixedSolver*> mem;
            for (Entry* e : gs[i]) mem.push_back(e->it->S);
            G.build(mem, s);
            G.key = key;
        }
        G.run(s, cap);
        ran.push_back(&G);
    }
    // the members' states and the groups' error words, one synchronisation
    for (auto& g : gs)
        for (Entry* e : g) {
            MixedSolver& S = *e->it->S;
            TSEM_CUDA(cudaMemcpyAsync(S.hsc, S.sc.p, sizeof(PcgScalars), cudaMemcpyDeviceToHost, s));
        }
    std::vector<int> gerr(ran.size(), 0);
    for (size_t i = 0; i < ran.size(); ++i) ran[i]->err.download(&gerr[i], 1, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    for (size_t i = 0; i < gs.size(); ++i) {
        if (gerr[i]) {
            ran[i]->err.zero(s);
            for (Entry* e : gs[i]) { e->status = TSEM_TIMEOUT; retire(*e); }
            continue;
        }
        for (Entry* e : gs[i]) {
            MixedSolver& S = *e->it->S;
            if (!S.hsc->done) continue;
            e->inner_total += S.hsc->iter;
            if (S.hsc->status == TSEM_NONFINITE || S.hsc->status == TSEM_BREAKDOWN) {
                e->status = S.hsc->status;
                retire(*e);
                continue;
            }
            k_axpy_f32<<<nb(S.A->n), 256, 0, s>>>(S.A->n, e->rn, S.dsol.p, e->it->x);
            TSEM_LAUNCHED();
            ++e->outer;
            batch_outer_step(*e, s);
            if (e->phase == 2) retire(*e);
        }
    }
    std::vector<std::unique_ptr<Entry>> keep;
    for (auto& e : active)
        if (e->phase != 2) keep.push_back(std::move(e));
    active.swap(keep);
    return done;
}

void solve_batch(std::vector<BatchItem>& items, cudaStream_t s) {
    BatchEngine eng(s);
    for (auto& it : items) eng.submit(&it);
    size_t left = items.size();
    while (left > 0) left -= eng.round().size();
}

// the bounds checks of the checked build on the current device: sets the divisor of
// every bound when shrink >= 1, returns and clears the first failure
bool bounds_check(int shrink, int* code, long long* index) {
    CheckState h{};
    TSEM_CUDA(cudaMemcpyFromSymbol(&h, g_check, sizeof(h)));
    if (code) *code = h.code;
    if (index) *index = h.index;
    h.code = 0;
    h.index = 0;
    if (shrink >= 1) h.shrink = shrink;
    TSEM_CUDA(cudaMemcpyToSymbol(g_check, &h, sizeof(h)));
    TSEM_CUDA(cudaDeviceSynchronize());
#ifdef TSEM_CHECK
    return true;
#else
    return false;
#endif
}

// poll limit of the bounded waits that may give up, on the current device (polls <= 0:
// the default 2^26)
void set_wait_polls(long long polls) {
    const long long v = polls > 0 ? polls : (1ll << 26);
    TSEM_CUDA(cudaMemcpyToSymbol(g_wait_polls, &v, sizeof(v)));
    TSEM_CUDA(cudaDeviceSynchronize());
}

}  // namespace tsem
