// Error handling and device-memory helpers shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>

#include <atomic>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/tsem_gpu.h"

namespace tsem {

// Exceptions carry a tsem_status to the C boundary.
struct Error : std::runtime_error {
    tsem_status status;
    Error(tsem_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline void cuda_check(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return;
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        throw Error(TSEM_OOM_REFUSED, std::string(what) + ": " + cudaGetErrorString(e));
    }
    throw Error(TSEM_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
}
#define TSEM_CUDA(x) ::tsem::cuda_check((x), #x)
#define TSEM_LAUNCH_CHECK() ::tsem::cuda_check(cudaGetLastError(), "kernel launch")

// kernels this process has launched (one count per launch site passed)
inline std::atomic<long long> g_kernel_launches{0};
#define TSEM_LAUNCHED() \
    (::tsem::g_kernel_launches.fetch_add(1, std::memory_order_relaxed), TSEM_LAUNCH_CHECK())

// Owning device buffer.
template <class T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    DBuf() = default;
    explicit DBuf(size_t count) { alloc(count); }
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    DBuf& operator=(DBuf&& o) noexcept {
        if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
        return *this;
    }
    ~DBuf() { release(); }
    void alloc(size_t count) {
        release();
        n = count;
        if (count) TSEM_CUDA(cudaMalloc((void**)&p, count * sizeof(T)));
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void upload(const T* h, size_t count, cudaStream_t s) {
        if (count > n) alloc(count);
        if (count) TSEM_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void upload(const std::vector<T>& v, cudaStream_t s) { upload(v.data(), v.size(), s); }
    void download(T* h, size_t count, cudaStream_t s) const {
        if (count) TSEM_CUDA(cudaMemcpyAsync(h, p, count * sizeof(T), cudaMemcpyDeviceToHost, s));
    }
    void zero(cudaStream_t s) {
        if (n) TSEM_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
    }
};

inline int grid_for(int64_t n, int block, int max_blocks = 152 * 32) {
    int64_t g = (n + block - 1) / block;
    if (g > max_blocks) g = max_blocks;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace tsem
