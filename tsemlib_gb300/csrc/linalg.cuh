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

// d as an FP32 pair (hi, lo), hi the nearest float and |lo| at most half an ulp of
// hi: about 2^-48 relative.  FP64 arithmetic and every conversion instruction run at
// a small fraction of the FP32 rate on this GPU, so the split works on the double's
// bits with integer and FP32 operations only: hi from the exponent and the upper 23
// mantissa bits (rounded to nearest; a carry into the exponent is the correct
// result); lo from the 29 low bits minus the rounding, an integer below 2^28 in
// magnitude that becomes a float as two exact 16-bit halves (2^23 + x - 2^23) joined
// by one rounding FMA, scaled by 2^(e - 52).  Zero, values below 2^-74 or above
// 2^126, and non-finite values take FP64 conversions.
__device__ __forceinline__ float2 split_f64(double d) {
    const unsigned long long u = (unsigned long long)__double_as_longlong(d);
    const unsigned hi32 = (unsigned)(u >> 32);
    const int ex = (int)((hi32 >> 20) & 0x7ffu) - 1023;
    if (ex < -74 || ex > 126) {
        const float hi = __double2float_rn(d);
        return make_float2(hi, __double2float_rn(d - (double)hi));
    }
    const unsigned long long man = u & 0xfffffffffffffull;
    const unsigned up = (unsigned)(man >> 28) & 1u;
    const unsigned hb = ((unsigned)(ex + 127) << 23) + (unsigned)(man >> 29) + up;
    const int rl = (int)(unsigned)(man & 0x1fffffffull) - (int)(up << 29);
    const unsigned x = (unsigned)(rl < 0 ? -rl : rl);
    const float f1 = __fsub_rn(__uint_as_float(0x4B000000u | (x >> 16)), 8388608.0f);
    const float f0 = __fsub_rn(__uint_as_float(0x4B000000u | (x & 0xffffu)), 8388608.0f);
    const float mag = __fmul_rn(__fmaf_rn(f1, 65536.0f, f0), __uint_as_float((unsigned)(ex - 52 + 127) << 23));
    const unsigned sign = hi32 & 0x80000000u;
    return make_float2(__uint_as_float(hb | sign), __uint_as_float(__float_as_uint(mag) ^ (sign ^ (rl < 0 ? 0x80000000u : 0u))));
}

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
