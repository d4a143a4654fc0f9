// Error handling and device-memory helpers shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>

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

// Timing marks inside a unit of work, for a caller that traces its phases (the
// service's opt-in trace): the caller installs a sink on its thread, and library code
// marks the ends of its inner phases.  Without a sink a mark costs one load.
struct TraceSink {
    virtual void mark(const char* name) = 0;
};
inline thread_local TraceSink* t_trace = nullptr;
inline void trace_mark(const char* name) {
    if (TraceSink* t = t_trace) t->mark(name);
}

// Allocation scope of one unit of work on a thread that shares the device with other
// threads' long-running work (a request of the service).  cudaMalloc and cudaFree
// wait for all work queued on the device, so a set-up that makes many temporary
// buffers would wait behind the other requests' solves at every one of them.  Inside
// a scope, buffers come from the stream-ordered pool (cudaMallocAsync on the scope's
// own stream, which only that allocation waits for) and their frees are deferred to
// the end of the scope, where they return to the pool without waiting.  The owner of
// a scope promises that by its end the host has seen every use of its buffers
// complete: the library's calls synchronise the streams they used before returning,
// and every destroy synchronises its object's stream.  (A device-wide synchronisation
// here would be wrong as well as slow: it is invalid while another thread captures a
// graph.)
struct AllocScope;
inline thread_local AllocScope* t_alloc_scope = nullptr;

struct AllocScope {
    cudaStream_t stream = nullptr;
    std::vector<void*> deferred;
    AllocScope* prev = nullptr;
    AllocScope() {
        if (cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking) != cudaSuccess) {
            cudaGetLastError();
            stream = nullptr;
            return;   // no scope: buffers use cudaMalloc / cudaFree
        }
        prev = t_alloc_scope;
        t_alloc_scope = this;
    }
    ~AllocScope() {
        if (!stream) return;
        t_alloc_scope = prev;
        for (void* q : deferred) cudaFreeAsync(q, stream);
        cudaStreamDestroy(stream);
    }
    AllocScope(const AllocScope&) = delete;
    AllocScope& operator=(const AllocScope&) = delete;
};

// Owning device buffer.
template <class T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    bool pooled = false;   // from the stream-ordered pool (allocated inside an AllocScope)
    DBuf() = default;
    explicit DBuf(size_t count) { alloc(count); }
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept : p(o.p), n(o.n), pooled(o.pooled) { o.p = nullptr; o.n = 0; o.pooled = false; }
    DBuf& operator=(DBuf&& o) noexcept {
        if (this != &o) {
            release();
            p = o.p; n = o.n; pooled = o.pooled;
            o.p = nullptr; o.n = 0; o.pooled = false;
        }
        return *this;
    }
    ~DBuf() { release(); }
    void alloc(size_t count) {
        release();
        n = count;
        if (!count) return;
        if (AllocScope* sc = t_alloc_scope) {
            TSEM_CUDA(cudaMallocAsync((void**)&p, count * sizeof(T), sc->stream));
            TSEM_CUDA(cudaStreamSynchronize(sc->stream));
            pooled = true;
        } else {
            TSEM_CUDA(cudaMalloc((void**)&p, count * sizeof(T)));
        }
    }
    void release() {
        if (p) {
            if (!pooled) {
                cudaFree(p);
            } else if (AllocScope* sc = t_alloc_scope) {
                sc->deferred.push_back(p);
            } else {
                // outside any scope: cudaFree waits for every use, then returns it to the pool
                cudaFree(p);
            }
        }
        p = nullptr;
        n = 0;
        pooled = false;
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

// Pinned host slots for small records the host reads back every iteration (a
// solver's scalar block): taken from slabs of page-locked memory that live as long as
// the process, so that making and destroying a solver never calls cudaMallocHost or
// cudaFreeHost (both wait for the whole device).  give = nullptr takes a slot.
template <class T>
T* pinned_slot(T* give = nullptr) {
    static std::mutex mu;
    static std::vector<T*> free_list;
    std::lock_guard<std::mutex> lock(mu);
    if (give) {
        free_list.push_back(give);
        return nullptr;
    }
    if (free_list.empty()) {
        constexpr int kSlab = 256;
        T* slab = nullptr;
        TSEM_CUDA(cudaMallocHost((void**)&slab, kSlab * sizeof(T)));
        for (int i = kSlab - 1; i >= 0; --i) free_list.push_back(slab + i);
    }
    T* q = free_list.back();
    free_list.pop_back();
    return q;
}

inline int grid_for(int64_t n, int block, int max_blocks = 152 * 32) {
    int64_t g = (n + block - 1) / block;
    if (g > max_blocks) g = max_blocks;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace tsem
