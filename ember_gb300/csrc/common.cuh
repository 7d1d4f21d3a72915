// Shared host/device helpers of libember_gpu: error reporting, CUDA checks,
// stream-ordered scratch buffers and host<->device staging for the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/ember_gpu.h"

namespace ember {

// Last error message of the calling thread (ember_last_error()).
void set_error(const char* fmt, ...);
const std::string& last_error();

// Run `expr` (a cudaError_t expression); on failure record the message and
// return EMBER_ECUDA from the enclosing function.
#define EMBER_CUDA_TRY(expr)                                                     \
    do {                                                                         \
        cudaError_t ember_err_ = (expr);                                         \
        if (ember_err_ != cudaSuccess) {                                         \
            ::ember::set_error("%s failed: %s (%s:%d)", #expr,                  \
                               cudaGetErrorString(ember_err_), __FILE__, __LINE__); \
            return EMBER_ECUDA;                                                  \
        }                                                                        \
    } while (0)

#define EMBER_CHECK_ARG(cond, ...)                                               \
    do {                                                                         \
        if (!(cond)) {                                                           \
            ::ember::set_error(__VA_ARGS__);                                     \
            return EMBER_EINVAL;                                                 \
        }                                                                        \
    } while (0)

#define EMBER_TRY(expr)                                                          \
    do {                                                                         \
        int ember_rc_ = (expr);                                                  \
        if (ember_rc_ != EMBER_OK) return ember_rc_;                             \
    } while (0)

inline cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

// Make sure the calling thread has a usable device.
int ensure_device();

// The library's own stream-ordered memory pool of the current device (freed
// blocks are kept for reuse; the default pool is not touched).
int scratch_pool(cudaMemPool_t* pool);

// Raise (never lower) a kernel's dynamic shared memory limit on the current
// device to `bytes`.
int raise_dynamic_smem(const void* func, size_t bytes);

// Stream-ordered device scratch (allocated from the library's pool with
// cudaMallocFromPoolAsync, freed with cudaFreeAsync on the call's stream). Freed when the object goes out of scope; the free is
// ordered after every kernel already queued on that stream.
//
// Arena mode (the second constructor): allocations are carved in order out of
// a caller-owned device buffer and nothing is freed; no allocation call is
// made, so launches that take a Scratch can be captured into a CUDA graph and
// replayed with the same buffers.
class Scratch {
public:
    explicit Scratch(cudaStream_t s) : stream_(s) {}
    Scratch(cudaStream_t s, void* arena, size_t arena_bytes)
        : stream_(s), arena_(static_cast<char*>(arena)), arena_bytes_(arena_bytes) {}
    ~Scratch() { release(); }
    Scratch(const Scratch&) = delete;
    Scratch& operator=(const Scratch&) = delete;

    static size_t rounded(size_t bytes) {
        bytes = ((bytes + 255) / 256) * 256;
        return bytes == 0 ? 256 : bytes;
    }

    // Allocate `bytes` (rounded up to 256) and return the device pointer in *p.
    template <class T>
    int alloc(T** p, size_t count) {
        size_t bytes = rounded(count * sizeof(T));
        if (arena_) {
            if (arena_used_ + bytes > arena_bytes_) {
                set_error("scratch arena too small (%zu of %zu bytes used, %zu more requested)", arena_used_,
                          arena_bytes_, bytes);
                return EMBER_ENOMEM;
            }
            *p = reinterpret_cast<T*>(arena_ + arena_used_);
            arena_used_ += bytes;
            return EMBER_OK;
        }
        void* q = nullptr;
        cudaMemPool_t pool = nullptr;
        EMBER_TRY(scratch_pool(&pool));
        cudaError_t e = cudaMallocFromPoolAsync(&q, bytes, pool, stream_);
        if (e != cudaSuccess) {
            set_error("cudaMallocFromPoolAsync(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
            return (e == cudaErrorMemoryAllocation) ? EMBER_ENOMEM : EMBER_ECUDA;
        }
        ptrs_.push_back(q);
        *p = static_cast<T*>(q);
        return EMBER_OK;
    }

    void release() {
        for (void* q : ptrs_) cudaFreeAsync(q, stream_);
        ptrs_.clear();
    }

private:
    cudaStream_t stream_;
    std::vector<void*> ptrs_;
    char* arena_ = nullptr;
    size_t arena_bytes_ = 0;
    size_t arena_used_ = 0;
};

// View an argument array on the device: for EMBER_MEM_DEVICE the pointer is
// used as is; for EMBER_MEM_HOST a scratch copy is made on `stream`.
template <class T>
int stage_in(Scratch& sc, const T* src, size_t count, int mem, cudaStream_t stream, const T** dev) {
    if (src == nullptr || mem == EMBER_MEM_DEVICE) {
        *dev = src;
        return EMBER_OK;
    }
    T* d = nullptr;
    EMBER_TRY(sc.alloc(&d, count));
    if (count) EMBER_CUDA_TRY(cudaMemcpyAsync(d, src, count * sizeof(T), cudaMemcpyHostToDevice, stream));
    *dev = d;
    return EMBER_OK;
}

// Output array: device pointer as is, or a scratch buffer to copy back later
// with stage_out().
template <class T>
int stage_buffer(Scratch& sc, T* dst, size_t count, int mem, T** dev) {
    if (dst == nullptr || mem == EMBER_MEM_DEVICE) {
        *dev = dst;
        return EMBER_OK;
    }
    return sc.alloc(dev, count);
}

template <class T>
int stage_out(T* dst, const T* dev, size_t count, int mem, cudaStream_t stream) {
    if (dst == nullptr || mem == EMBER_MEM_DEVICE || count == 0) return EMBER_OK;
    EMBER_CUDA_TRY(cudaMemcpyAsync(dst, dev, count * sizeof(T), cudaMemcpyDeviceToHost, stream));
    return EMBER_OK;
}

// Check the launch and, for host-memory calls, wait for the stream.
int finish_call(int mem, cudaStream_t stream);

inline int blocks_for(int64_t n, int threads) {
    return static_cast<int>((n + threads - 1) / threads);
}

}  // namespace ember
