// Bounds checks of the checked build (compiled with -DTSEM_CHECK).  The matrix-free
// operator's gathers and scatters and the mixed solver's FP32 SpMVs check every index
// they read from a table against the length of the vector it addresses; an index
// outside records the first failure (a code naming the kernel, and the index) in
// g_check and its access is skipped: nothing traps, and the host turns the record
// into TSEM_INVALID.  g_check.shrink divides every bound: a test hook with which valid
// indices fail the check, so that the error path runs while every access that still
// happens is inside its vector.  Without TSEM_CHECK the checks compile to nothing.
#pragma once
#include <cstdint>

namespace tsem {

struct CheckState {
    int code;             // first failing check (0 = none)
    int shrink;           // divisor of every bound (1 = the real bounds)
    long long index;      // its index
};

static __device__ CheckState g_check = {0, 1, 0};

__device__ __forceinline__ bool in_bounds(long long i, long long n, int code) {
#ifdef TSEM_CHECK
    const int sh = g_check.shrink;
    const long long lim = sh > 1 ? n / sh : n;
    if (i >= 0 && i < lim) return true;
    if (atomicCAS(&g_check.code, 0, code) == 0) g_check.index = i;
    return false;
#else
    (void)i; (void)n; (void)code;
    return true;
#endif
}

}  // namespace tsem
