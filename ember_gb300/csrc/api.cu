// Library-wide entry points of libember_gpu: error text, version, device setup.
#include "common.cuh"

#include <cstring>
#include <mutex>

namespace ember {

static thread_local std::string g_last_error;

void set_error(const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
}

const std::string& last_error() { return g_last_error; }

int ensure_device() {
    static std::once_flag once;
    static int rc = EMBER_OK;
    std::call_once(once, [] {
        int n = 0;
        cudaError_t e = cudaGetDeviceCount(&n);
        if (e != cudaSuccess || n == 0) {
            rc = EMBER_ECUDA;
            return;
        }
        int dev = 0;
        cudaGetDevice(&dev);
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t threshold = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &threshold);
        }
    });
    if (rc != EMBER_OK) set_error("no CUDA device is available");
    return rc;
}

int finish_call(int mem, cudaStream_t stream) {
    EMBER_CUDA_TRY(cudaGetLastError());
    if (mem == EMBER_MEM_HOST) EMBER_CUDA_TRY(cudaStreamSynchronize(stream));
    return EMBER_OK;
}

}  // namespace ember

extern "C" int ember_last_error(char* buf, size_t n) {
    const std::string& s = ember::last_error();
    if (buf && n) {
        size_t m = s.size() < n - 1 ? s.size() : n - 1;
        std::memcpy(buf, s.data(), m);
        buf[m] = '\0';
    }
    return static_cast<int>(s.size());
}

extern "C" int ember_version(void) { return 100; }

extern "C" int ember_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}
