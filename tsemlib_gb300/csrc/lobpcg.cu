// Block LOBPCG (TSEMSolver::solve_LOBPCG, src/TSEMSolver.cpp:2071-2222 for one
// vector and :2225-2406 for a block) on the device.
//
// The basis S = [X W P] of every iteration lives row-major in one n x 3k array
// (columns [0,k) X, [k,2k) W, [2k,3k) P), with A S and M S beside it: the block
// products (CSR times a block, Gram matrices S^T A S and S^T M S, and the Ritz
// combinations S C) then read whole rows.  Gram matrices and the Rayleigh-Ritz
// problem are FP64; the small generalized eigenproblem is solved on the host.
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

constexpr int kMaxBlock = 40;     // columns of one block (X, W or P)
constexpr int kGramRows = 32;     // rows per shared-memory stage of the Gram kernel
constexpr int kGramThreads = 256;

// ---- FP64 products on the FP32 pipe.  GB300 runs FP64 FMAs at a small fraction of
// its FP32 rate; the block kernels below take their FP64 operands as (hi, lo) FP32
// pairs and form every product and sum with exact FP32 error terms (about 2^-48
// relative per product, compensated sums), FP64 only at the ends.
__device__ __forceinline__ float2 split2(double d) {
    const float hi = __double2float_rn(d);
    return make_float2(hi, __double2float_rn(d - (double)hi));
}
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

// Xs[i][j] = split(X[i][j]) for j < kc
__global__ void k_split_block(int64_t n, int kc, const double* __restrict__ X, int ldx, float2* __restrict__ Xs) {
    const int64_t total = n * kc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x)
        Xs[t] = split2(X[(size_t)(t / kc) * ldx + t % kc]);
}

// Y[i][j] = sum_c A[i][c] X[c][j] on split operands (values of A and the block Xs)
template <int L>
__global__ void k_spmm_split(int64_t n, const int64_t* __restrict__ rp, const int* __restrict__ ci,
                             const float2* __restrict__ va, const float2* __restrict__ Xs, int kc, double* __restrict__ Y,
                             int ldy) {
    const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / L;
    const int lane = threadIdx.x % L;
    if (row >= n || lane >= kc) return;
    const bool two = lane + 32 < kc;
    float sh = 0.f, sl = 0.f, sh2 = 0.f, sl2 = 0.f;
    const int64_t e = rp[row + 1];
    int64_t k = rp[row];
    for (; k + 4 <= e; k += 4) {
        float2 a[4];
        const float2* xr[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            a[u] = va[k + u];
            xr[u] = Xs + (size_t)ci[k + u] * kc;
        }
        float2 x[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) x[u] = xr[u][lane];
#pragma unroll
        for (int u = 0; u < 4; ++u) acc2(a[u], x[u], sh, sl);
        if (two)
#pragma unroll
            for (int u = 0; u < 4; ++u) acc2(a[u], xr[u][lane + 32], sh2, sl2);
    }
    for (; k < e; ++k) {
        const float2 a = va[k];
        const float2* xr = Xs + (size_t)ci[k] * kc;
        acc2(a, xr[lane], sh, sl);
        if (two) acc2(a, xr[lane + 32], sh2, sl2);
    }
    Y[(size_t)row * ldy + lane] = (double)sh + (double)sl;
    if (two) Y[(size_t)row * ldy + lane + 32] = (double)sh2 + (double)sl2;
}

// G[a][b] += sum_i S[i][a] T[i][b] (a < m1, b < m2; with `upper` only b >= a), FP64
// on the FP32 pipe (split products, compensated sums).  A block streams kGramRows
// rows of both blocks through shared memory (split, zero-padded to multiples of 4
// columns); each thread owns 4 x 4 tiles of G in registers, so eight 16-byte loads
// per row feed sixteen products; the block's partial sums go to G by FP64 atomics.
__global__ void __launch_bounds__(kGramThreads)
k_gram(int64_t n, int m1, int m2, const double* __restrict__ S, int lds, const double* __restrict__ T, int ldt, int upper,
       double* G) {
    extern __shared__ float4 shs4[];
    const int m1p = (m1 + 3) & ~3, m2p = (m2 + 3) & ~3;
    float2* Ss = reinterpret_cast<float2*>(shs4);
    float2* Ts = Ss + kGramRows * m1p;
    const int ta_n = m1p / 4, tb_n = m2p / 4;
    // the tiles: all of them, or (upper, m1 == m2) those with tb >= ta
    const int n_tiles = upper ? ta_n * (ta_n + 1) / 2 : ta_n * tb_n;
    for (int tile0 = 0; tile0 < n_tiles; tile0 += kGramThreads) {
        const int tile = tile0 + threadIdx.x;
        int ta = 0, tb = 0;
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
        const bool active = tile < n_tiles;
        float ah[4][4], al[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) ah[i][j] = al[i][j] = 0.0f;
        for (int64_t r0 = (int64_t)blockIdx.x * kGramRows; r0 < n; r0 += (int64_t)gridDim.x * kGramRows) {
            __syncthreads();
            for (int idx = threadIdx.x; idx < kGramRows * m1p; idx += blockDim.x) {
                const int64_t r = r0 + idx / m1p;
                const int c = idx % m1p;
                Ss[idx] = (r < n && c < m1) ? split2(S[(size_t)r * lds + c]) : make_float2(0.f, 0.f);
            }
            for (int idx = threadIdx.x; idx < kGramRows * m2p; idx += blockDim.x) {
                const int64_t r = r0 + idx / m2p;
                const int c = idx % m2p;
                Ts[idx] = (r < n && c < m2) ? split2(T[(size_t)r * ldt + c]) : make_float2(0.f, 0.f);
            }
            __syncthreads();
            if (active) {
                const int rows = (int)min((int64_t)kGramRows, n - r0);
                for (int r = 0; r < rows; ++r) {
                    const float4* sp = reinterpret_cast<const float4*>(Ss + r * m1p + 4 * ta);
                    const float4* tp = reinterpret_cast<const float4*>(Ts + r * m2p + 4 * tb);
                    const float4 s01 = sp[0], s23 = sp[1], t01 = tp[0], t23 = tp[1];
                    const float2 sv[4] = {make_float2(s01.x, s01.y), make_float2(s01.z, s01.w),
                                          make_float2(s23.x, s23.y), make_float2(s23.z, s23.w)};
                    const float2 tv[4] = {make_float2(t01.x, t01.y), make_float2(t01.z, t01.w),
                                          make_float2(t23.x, t23.y), make_float2(t23.z, t23.w)};
#pragma unroll
                    for (int i = 0; i < 4; ++i)
#pragma unroll
                        for (int j = 0; j < 4; ++j) acc2(sv[i], tv[j], ah[i][j], al[i][j]);
                }
            }
        }
        if (active) {
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int a = 4 * ta + i, b = 4 * tb + j;
                    if (a < m1 && b < m2 && (!upper || b >= a))
                        atomicAdd(G + (size_t)a * m2 + b, (double)ah[i][j] + (double)al[i][j]);
                }
        }
    }
}

// Y[i][j] = sum_a S[i][a0 + a] C[a][j] for a < m, j < kc (C row-major m x kc)
// S: the m columns of the basis, already split (n x m pairs)
__global__ void k_combo(int64_t n, int m, int kc, const float2* __restrict__ S, const double* __restrict__ C,
                        double* __restrict__ Y, int ldy) {
    extern __shared__ float2 Cs[];
    for (int idx = threadIdx.x; idx < m * kc; idx += blockDim.x) Cs[idx] = split2(C[idx]);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; row < n; row += warps) {
        const float2* sr = S + (size_t)row * m;
        for (int j = lane; j < kc; j += 32) {
            float h = 0.f, l = 0.f;
            for (int a = 0; a < m; ++a) acc2(sr[a], Cs[a * kc + j], h, l);
            Y[(size_t)row * ldy + j] = (double)h + (double)l;
        }
    }
}

// R[i][j] = AX[i][j] - lambda_j MX[i][j]; nrm[j] += R^2, nrm[k + j] += MX^2
__global__ void k_block_resid(int64_t n, int kc, const double* __restrict__ AX, const double* __restrict__ MX, int ld,
                              const double* __restrict__ lam, double* __restrict__ R, int ldr, double* nrm) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int j = lane; j < kc; j += 32) {
        double rr = 0.0, mm = 0.0;
        const double l = lam[j];
        for (int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; row < n; row += warps) {
            const double mx = MX[(size_t)row * ld + j];
            const double r = AX[(size_t)row * ld + j] - l * mx;
            R[(size_t)row * ldr + j] = r;
            rr += r * r;
            mm += mx * mx;
        }
        atomicAdd(nrm + j, rr);
        atomicAdd(nrm + kc + j, mm);
    }
}

// column j of a row-major block <-> a contiguous vector
__global__ void k_col_get(int64_t n, const double* __restrict__ B, int ld, double* __restrict__ v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v[i] = B[(size_t)i * ld];
}
__global__ void k_col_put(int64_t n, const double* __restrict__ v, double* __restrict__ B, int ld) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        B[(size_t)i * ld] = v[i];
}
// the k columns of B (row stride ld) as FP32 columns n apart, column j scaled by sc[j]
__global__ void k_block_get_f32(int64_t n, int k, const double* __restrict__ B, int ld, const double* __restrict__ sc,
                                float* __restrict__ v) {
    const int j = blockIdx.y;
    const double f = sc[j];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v[(size_t)j * n + i] = (float)(B[(size_t)i * ld + j] * f);
}
// back: B[i][j] = v[j][i] * sc[j]
__global__ void k_block_put_f32(int64_t n, int k, const float* __restrict__ v, const double* __restrict__ sc,
                                double* __restrict__ B, int ld) {
    const int j = blockIdx.y;
    const double f = sc[j];
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        B[(size_t)i * ld + j] = (double)v[(size_t)j * n + i] * f;
}
__global__ void k_jacobi_col(int64_t n, const double* __restrict__ d, double* v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v[i] /= d[i];
}
// column-major n x k block <-> columns [0, k) of a row-major block
__global__ void k_cm_to_rm(int64_t n, int kc, const double* __restrict__ X, double* __restrict__ B, int ld) {
    const int64_t total = n * kc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / kc;
        const int j = (int)(t % kc);
        B[(size_t)i * ld + j] = X[(size_t)j * n + i];
    }
}
__global__ void k_rm_to_cm(int64_t n, int kc, const double* __restrict__ B, int ld, double* __restrict__ X) {
    const int64_t total = n * kc;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int j = (int)(t / n);
        const int64_t i = t % n;
        X[(size_t)j * n + i] = B[(size_t)i * ld + j];
    }
}

int nblk(int64_t n) { return grid_for(n, 256, 152 * 16); }

// dynamic shared memory of the Gram kernel beyond the 48 KB default (blocks of up to 3 x 40 columns)
void gram_smem_limit() {
    static std::once_flag once;
    std::call_once(once, [] {
        TSEM_CUDA(cudaFuncSetAttribute(k_gram, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(kGramRows * 2 * 3 * kMaxBlock * sizeof(double))));
    });
}

// Y = A X on split operands: A's (hi, lo) values (kept with the matrix) and the block
// split into `scratch` (n x kc pairs)
void spmm_split(const DevCsr& A, const double* X, int ldx, int kc, double* Y, int ldy, DBuf<float2>& scratch,
                cudaStream_t s) {
    csr_split_values(A, s);
    if (scratch.n < (size_t)A.n * kc) scratch.alloc((size_t)A.n * kc);
    k_split_block<<<nblk(A.n * kc), 256, 0, s>>>(A.n, kc, X, ldx, scratch.p);
    TSEM_LAUNCHED();
    const int L = kc <= 4 ? 4 : kc <= 8 ? 8 : kc <= 16 ? 16 : 32;
    const unsigned g = (unsigned)((A.n * L + 255) / 256);
    const float2* va = A.vsplit.p;
    if (L == 4) k_spmm_split<4><<<g, 256, 0, s>>>(A.n, A.rowptr.p, A.col.p, va, scratch.p, kc, Y, ldy);
    else if (L == 8) k_spmm_split<8><<<g, 256, 0, s>>>(A.n, A.rowptr.p, A.col.p, va, scratch.p, kc, Y, ldy);
    else if (L == 16) k_spmm_split<16><<<g, 256, 0, s>>>(A.n, A.rowptr.p, A.col.p, va, scratch.p, kc, Y, ldy);
    else k_spmm_split<32><<<g, 256, 0, s>>>(A.n, A.rowptr.p, A.col.p, va, scratch.p, kc, Y, ldy);
    TSEM_LAUNCHED();
}


}  // namespace

// ---------------------------------------------------------------- host side
void sym_eig_small(int m, const std::vector<double>& a_in, std::vector<double>& w, std::vector<double>& V) {
    std::vector<double> a(a_in);
    V.assign((size_t)m * m, 0.0);
    for (int i = 0; i < m; ++i) V[(size_t)i * m + i] = 1.0;
    double scale = 0.0;
    for (double x : a) scale = std::max(scale, std::fabs(x));
    if (scale == 0.0) scale = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0;
        for (int p = 0; p < m; ++p)
            for (int q = p + 1; q < m; ++q) off += a[(size_t)p * m + q] * a[(size_t)p * m + q];
        if (std::sqrt(off) <= 1e-17 * scale * m) break;
        for (int p = 0; p < m; ++p)
            for (int q = p + 1; q < m; ++q) {
                const double apq = a[(size_t)p * m + q];
                if (std::fabs(apq) <= 1e-300) continue;
                const double app = a[(size_t)p * m + p], aqq = a[(size_t)q * m + q];
                // rotation angle that zeroes a[p][q]
                const double tau = (aqq - app) / (2.0 * apq);
                const double t = (tau >= 0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
                const double c = 1.0 / std::sqrt(1.0 + t * t), sn = t * c;
                for (int r = 0; r < m; ++r) {
                    const double arp = a[(size_t)r * m + p], arq = a[(size_t)r * m + q];
                    a[(size_t)r * m + p] = c * arp - sn * arq;
                    a[(size_t)r * m + q] = sn * arp + c * arq;
                }
                for (int r = 0; r < m; ++r) {
                    const double apr = a[(size_t)p * m + r], aqr = a[(size_t)q * m + r];
                    a[(size_t)p * m + r] = c * apr - sn * aqr;
                    a[(size_t)q * m + r] = sn * apr + c * aqr;
                }
                for (int r = 0; r < m; ++r) {
                    const double vrp = V[(size_t)r * m + p], vrq = V[(size_t)r * m + q];
                    V[(size_t)r * m + p] = c * vrp - sn * vrq;
                    V[(size_t)r * m + q] = sn * vrp + c * vrq;
                }
            }
    }
    std::vector<int> idx(m);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](int i, int j) { return a[(size_t)i * m + i] < a[(size_t)j * m + j]; });
    w.resize(m);
    std::vector<double> Vs((size_t)m * m);
    for (int j = 0; j < m; ++j) {
        w[j] = a[(size_t)idx[j] * m + idx[j]];
        for (int i = 0; i < m; ++i) Vs[(size_t)i * m + j] = V[(size_t)i * m + idx[j]];
    }
    V.swap(Vs);
}

int rayleigh_ritz_small(int m, const std::vector<double>& GA_in, const std::vector<double>& GB_in,
                        std::vector<double>& theta, std::vector<double>& C) {
    // scale the basis to unit B-norm first (D GA D, D GB D with D = diag(GB)^(-1/2)):
    // residual directions shrink as the iteration converges, and unscaled they
    // would fall under the rank threshold below
    std::vector<double> dsc(m), GA(GA_in), GB(GB_in);
    for (int i = 0; i < m; ++i) {
        const double g = GB_in[(size_t)i * m + i];
        dsc[i] = g > 0 ? 1.0 / std::sqrt(g) : 0.0;
    }
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j) {
            GA[(size_t)i * m + j] *= dsc[i] * dsc[j];
            GB[(size_t)i * m + j] *= dsc[i] * dsc[j];
        }
    std::vector<double> wb, U;
    sym_eig_small(m, GB, wb, U);
    double mx = 0.0;
    for (double x : wb) mx = std::max(mx, std::fabs(x));
    std::vector<int> keep;
    for (int j = 0; j < m; ++j)
        if (wb[j] > 1e-13 * mx) keep.push_back(j);
    const int r = (int)keep.size();
    // Q = U_keep diag(wb_keep)^(-1/2): a GB-orthonormal basis of the kept directions
    std::vector<double> Q((size_t)m * r), T((size_t)m * r, 0.0), H((size_t)r * r, 0.0);
    for (int a = 0; a < r; ++a) {
        const double f = 1.0 / std::sqrt(wb[keep[a]]);
        for (int i = 0; i < m; ++i) Q[(size_t)i * r + a] = U[(size_t)i * m + keep[a]] * f;
    }
    for (int i = 0; i < m; ++i)
        for (int b = 0; b < r; ++b) {
            double t = 0.0;
            for (int j = 0; j < m; ++j) t += GA[(size_t)i * m + j] * Q[(size_t)j * r + b];
            T[(size_t)i * r + b] = t;
        }
    for (int a = 0; a < r; ++a)
        for (int b = 0; b < r; ++b) {
            double t = 0.0;
            for (int i = 0; i < m; ++i) t += Q[(size_t)i * r + a] * T[(size_t)i * r + b];
            H[(size_t)a * r + b] = t;
        }
    for (int a = 0; a < r; ++a)
        for (int b = 0; b < a; ++b) {
            const double t = 0.5 * (H[(size_t)a * r + b] + H[(size_t)b * r + a]);
            H[(size_t)a * r + b] = H[(size_t)b * r + a] = t;
        }
    std::vector<double> Y;
    sym_eig_small(r, H, theta, Y);
    C.assign((size_t)m * r, 0.0);
    for (int i = 0; i < m; ++i)
        for (int b = 0; b < r; ++b) {
            double t = 0.0;
            for (int a = 0; a < r; ++a) t += Q[(size_t)i * r + a] * Y[(size_t)a * r + b];
            C[(size_t)i * r + b] = t * dsc[i];
        }
    return r;
}

namespace {

// full symmetric m x m Gram matrix S^T T of the first m columns (upper triangle computed)
void gram(int64_t n, int m, const double* S, const double* T, int ld, DBuf<double>& G, std::vector<double>& h,
          cudaStream_t s) {
    TSEM_CUDA(cudaMemsetAsync(G.p, 0, (size_t)m * m * sizeof(double), s));
    const size_t shm = (size_t)kGramRows * 2 * ((m + 3) & ~3) * sizeof(float2);
    const int blocks = (int)std::min<int64_t>(152 * 8, (n + kGramRows - 1) / kGramRows);
    k_gram<<<std::max(blocks, 1), kGramThreads, shm, s>>>(n, m, m, S, ld, T, ld, 1, G.p);
    TSEM_LAUNCHED();
    h.resize((size_t)m * m);
    G.download(h.data(), (size_t)m * m, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    for (int a = 0; a < m; ++a)
        for (int b = 0; b < a; ++b) h[(size_t)a * m + b] = h[(size_t)b * m + a];
}

// Y = S[:, a0 : a0 + m] C (C m x kc), the columns split into `scratch` first
void combo(int64_t n, int m, int kc, const double* S, int lds, int a0, const DBuf<double>& C, double* Y, int ldy,
           DBuf<float2>& scratch, cudaStream_t s) {
    if (scratch.n < (size_t)n * m) scratch.alloc((size_t)n * m);
    k_split_block<<<nblk(n * m), 256, 0, s>>>(n, m, S + a0, lds, scratch.p);
    TSEM_LAUNCHED();
    k_combo<<<nblk(n * 32), 256, (size_t)m * kc * sizeof(float2), s>>>(n, m, kc, scratch.p, C.p, Y, ldy);
    TSEM_LAUNCHED();
}

}  // namespace

// G = S^T T of k x k blocks (row-major, rows over S's columns), on the host
void gram_block(int64_t n, int kb, const double* S, const double* T, int ld, DBuf<double>& G, std::vector<double>& h,
                bool upper, cudaStream_t s) {
    TSEM_CUDA(cudaMemsetAsync(G.p, 0, (size_t)kb * kb * sizeof(double), s));
    const size_t shm = (size_t)kGramRows * 2 * ((kb + 3) & ~3) * sizeof(float2);
    const int blocks = (int)std::min<int64_t>(152 * 8, (n + kGramRows - 1) / kGramRows);
    k_gram<<<std::max(blocks, 1), kGramThreads, shm, s>>>(n, kb, kb, S, ld, T, ld, upper ? 1 : 0, G.p);
    TSEM_LAUNCHED();
    h.resize((size_t)kb * kb);
    G.download(h.data(), (size_t)kb * kb, s);
    TSEM_CUDA(cudaStreamSynchronize(s));
    if (upper)
        for (int a = 0; a < kb; ++a)
            for (int b = 0; b < a; ++b) h[(size_t)a * kb + b] = h[(size_t)b * kb + a];
}

LobpcgResult lobpcg(const DevCsr& A, const DevCsr& M, Solver* plain, MixedSolver* mixed, int k, int n_want, double* X,
                    double* lambda, double tol, int max_it, cudaStream_t s) {
    const int64_t n = A.n;
    if (M.n != n) throw Error(TSEM_INVALID, "A and M differ in size");
    if (k < 1 || k > kMaxBlock) throw Error(TSEM_INVALID, "block size must be 1.." + std::to_string(kMaxBlock));
    if (n_want < 1 || n_want > k) throw Error(TSEM_INVALID, "n_want must be 1..k");
    if (n < 3 * (int64_t)k) throw Error(TSEM_INVALID, "block too large for the problem");
    gram_smem_limit();
    LobpcgResult res;
    cudaEvent_t e0, e1;
    TSEM_CUDA(cudaEventCreate(&e0));
    TSEM_CUDA(cudaEventCreate(&e1));
    TSEM_CUDA(cudaEventRecord(e0, s));
    const int ld = 3 * k;
    DBuf<double> S((size_t)n * ld), AS((size_t)n * ld), MS((size_t)n * ld);
    DBuf<double> S2((size_t)n * ld), AS2((size_t)n * ld), MS2((size_t)n * ld);
    DBuf<double> G((size_t)ld * ld), dC((size_t)ld * k), dlam(k), nrm(2 * k), col(n);
    DBuf<float> cf, zf;
    DBuf<float2> xs;         // split copy of the block a product reads
    DBuf<double> bsc(2 * k);   // per-column scales of the block V-cycle (1/|r_j| in, |r_j| out)
    DBuf<double> dK((size_t)2 * k * k);
    std::vector<double> hC;
    if (mixed) { cf.alloc((size_t)n * k); zf.alloc((size_t)n * k); }
    std::vector<double> GA, GB, theta, C, hn(2 * k), hsc(2 * k);

    // Ritz update of the first m columns: X = S C[:, :k], P = S[:, k:m] C[k:m, :k]
    auto update = [&](int m, bool with_p) {
        std::vector<double> Ck((size_t)m * k);
        const int r = (int)(C.size() / m);
        for (int i = 0; i < m; ++i)
            for (int j = 0; j < k; ++j) Ck[(size_t)i * k + j] = C[(size_t)i * r + j];
        dC.upload(Ck, s);
        combo(n, m, k, S.p, ld, 0, dC, S2.p, ld, xs, s);
        combo(n, m, k, AS.p, ld, 0, dC, AS2.p, ld, xs, s);
        combo(n, m, k, MS.p, ld, 0, dC, MS2.p, ld, xs, s);
        if (with_p) {
            DBuf<double> dCp((size_t)(m - k) * k);
            dCp.upload(Ck.data() + (size_t)k * k, (size_t)(m - k) * k, s);
            combo(n, m - k, k, S.p, ld, k, dCp, S2.p + 2 * k, ld, xs, s);
            // A P and M P from P itself: combined like P they would lose their
            // relative accuracy when P is small, and the next Gram matrices would
            // no longer describe the same vectors
            spmm_split(A, S2.p + 2 * k, ld, k, AS2.p + 2 * k, ld, xs, s);
            spmm_split(M, S2.p + 2 * k, ld, k, MS2.p + 2 * k, ld, xs, s);
            TSEM_CUDA(cudaStreamSynchronize(s));
        }
        std::swap(S.p, S2.p);
        std::swap(AS.p, AS2.p);
        std::swap(MS.p, MS2.p);
        for (int j = 0; j < k; ++j) lambda[j] = theta[j];
        dlam.upload(lambda, k, s);
    };

    // initial Rayleigh-Ritz on X
    k_cm_to_rm<<<nblk(n * k), 256, 0, s>>>(n, k, X, S.p, ld);
    TSEM_LAUNCHED();
    spmm_split(A, S.p, ld, k, AS.p, ld, xs, s);
    spmm_split(M, S.p, ld, k, MS.p, ld, xs, s);
    gram(n, k, S.p, AS.p, ld, G, GA, s);
    gram(n, k, S.p, MS.p, ld, G, GB, s);
    // the k x k Gram of the first k columns sits in the leading block of a ld-strided
    // layout only when m == ld; here m == k and the matrices are k x k
    if (rayleigh_ritz_small(k, GA, GB, theta, C) < k) throw Error(TSEM_INVALID, "initial block is rank deficient");
    update(k, false);
    int np = 0;
    int it = 0;
    res.status = TSEM_MAXIT;
    for (;; ++it) {
        // residual block into the W columns, and its relative norms
        nrm.zero(s);
        k_block_resid<<<nblk(n * 32), 256, 0, s>>>(n, k, AS.p, MS.p, ld, dlam.p, S.p + k, ld, nrm.p);
        TSEM_LAUNCHED();
        nrm.download(hn.data(), 2 * k, s);
        TSEM_CUDA(cudaStreamSynchronize(s));
        double worst = 0.0;
        bool finite = true;
        for (int j = 0; j < n_want; ++j) {
            const double rel = std::sqrt(hn[j]) / (std::fabs(lambda[j]) * std::sqrt(hn[k + j]));
            if (!std::isfinite(rel)) finite = false;
            worst = std::max(worst, rel);
        }
        res.residual = worst;
        if (!finite) { res.status = TSEM_NONFINITE; break; }
        if (worst < tol) { res.status = TSEM_OK; break; }
        if (it >= max_it) break;
        // W = preconditioned residual: the mixed solver's V-cycle takes the whole block in
        // one pass of launches (each column scaled to unit norm in FP32); the plain
        // form's runs column by column
        if (mixed) {
            for (int j = 0; j < k; ++j) {
                const double rn = std::sqrt(hn[j]);
                hsc[j] = rn > 0 ? 1.0 / rn : 1.0;
                hsc[k + j] = rn > 0 ? rn : 1.0;
            }
            bsc.upload(hsc, s);
            const dim3 g((unsigned)nblk(n), (unsigned)k);
            k_block_get_f32<<<g, 256, 0, s>>>(n, k, S.p + k, ld, bsc.p, cf.p);
            TSEM_LAUNCHED();
            mixed->vcycle_graph(cf.p, zf.p, s, k);
            k_block_put_f32<<<g, 256, 0, s>>>(n, k, zf.p, bsc.p + k, S.p + k, ld);
            TSEM_LAUNCHED();
        }
        for (int j = 0; j < k && !mixed; ++j) {
            double* wj = S.p + k + j;
            k_col_get<<<nblk(n), 256, 0, s>>>(n, wj, ld, col.p);
            TSEM_LAUNCHED();
            if (plain && plain->pmg) {
                DBuf<double>& z = plain->y;   // scratch of the PCG, unused between solves
                // the V-cycle (ite_PMG) works on z in place: from z = 0 it is one fixed
                // linear preconditioner for every column
                TSEM_CUDA(cudaMemsetAsync(z.p, 0, (size_t)n * sizeof(double), s));
                plain->pmg->vcycle(z.p, col.p, nullptr, s);
                k_col_put<<<nblk(n), 256, 0, s>>>(n, z.p, wj, ld);
            } else {
                k_jacobi_col<<<nblk(n), 256, 0, s>>>(n, A.diag.p, col.p);
                TSEM_LAUNCHED();
                k_col_put<<<nblk(n), 256, 0, s>>>(n, col.p, wj, ld);
            }
            TSEM_LAUNCHED();
        }
        // W <- W - X ((M X)^T W): the preconditioned residuals M-orthogonal to X (which is
        // M-orthonormal after the previous Rayleigh-Ritz step), formed on the vectors so
        // that the Gram matrices below need not resolve W's small part outside span(X)
        // next to its large part inside it; A W and M W then come from the projected W
        {
            gram_block(n, k, MS.p, S.p + k, ld, G, hC, false, s);
            std::vector<double> K1((size_t)2 * k * k, 0.0);
            for (int a = 0; a < k; ++a)
                for (int b = 0; b < k; ++b) K1[(size_t)a * k + b] = -hC[(size_t)a * k + b];
            for (int b = 0; b < k; ++b) K1[(size_t)(k + b) * k + b] = 1.0;
            dK.upload(K1, s);
            combo(n, 2 * k, k, S.p, ld, 0, dK, S.p + k, ld, xs, s);
        }
        spmm_split(A, S.p + k, ld, k, AS.p + k, ld, xs, s);
        spmm_split(M, S.p + k, ld, k, MS.p + k, ld, xs, s);
        const int m = 2 * k + np;
        // Gram matrices of the m = 2k + np columns
        {
            const size_t shm = (size_t)kGramRows * 2 * ((m + 3) & ~3) * sizeof(float2);
            const int blocks = (int)std::min<int64_t>(152 * 8, (n + kGramRows - 1) / kGramRows);
            for (int w = 0; w < 2; ++w) {
                TSEM_CUDA(cudaMemsetAsync(G.p, 0, (size_t)m * m * sizeof(double), s));
                k_gram<<<std::max(blocks, 1), kGramThreads, shm, s>>>(n, m, m, S.p, ld, w == 0 ? AS.p : MS.p, ld, 1,
                                                                       G.p);
                TSEM_LAUNCHED();
                std::vector<double>& h = w == 0 ? GA : GB;
                h.resize((size_t)m * m);
                G.download(h.data(), (size_t)m * m, s);
                TSEM_CUDA(cudaStreamSynchronize(s));
                for (int a = 0; a < m; ++a)
                    for (int b = 0; b < a; ++b) h[(size_t)a * m + b] = h[(size_t)b * m + a];
            }
        }
        if (rayleigh_ritz_small(m, GA, GB, theta, C) < k) { res.status = TSEM_BREAKDOWN; break; }
        update(m, true);
        np = k;
    }
    res.iterations = it;
    k_rm_to_cm<<<nblk(n * k), 256, 0, s>>>(n, k, S.p, ld, X);
    TSEM_LAUNCHED();
    TSEM_CUDA(cudaEventRecord(e1, s));
    TSEM_CUDA(cudaEventSynchronize(e1));
    TSEM_CUDA(cudaEventElapsedTime(&res.device_ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return res;
}

}  // namespace tsem
