// CSR SpMV and fused vector kernels (FP64).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace tsem {

// Device scalars of one PCG run.  Accumulators are zeroed by the kernel that
// precedes their producer; `cur` is latched once per iteration by the SpMV kernel
// so that every block of the later kernels sees the same slot.
struct PcgScalars {
    double rty[2];      // r^T y of the current / next iteration
    double pap;         // p^T A p
    double l1, rr;      // ||r||_1, ||r||_2^2 of the latest residual
    double bb;          // ||b||_2^2
    double init_l1;
    double tol_abs, tol_rel2;
    int iter, max_iter;
    int cur;
    int done, status;
    int rel_mode;
};

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// block-wide sum of up to three values, atomically added to the targets by thread 0
template <int NV>
__device__ __forceinline__ void block_accumulate(double (&v)[NV], double* const (&dst)[NV]) {
    __shared__ double sh[NV][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int k = 0; k < NV; ++k) v[k] = warp_sum(v[k]);
    if (lane == 0)
        for (int k = 0; k < NV; ++k) sh[k][wid] = v[k];
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        for (int k = 0; k < NV; ++k) {
            double t = lane < nw ? sh[k][lane] : 0.0;
            t = warp_sum(t);
            if (lane == 0 && dst[k]) atomicAdd(dst[k], t);
        }
    }
}

}  // namespace tsem
