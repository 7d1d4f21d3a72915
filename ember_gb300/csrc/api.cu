// Library-wide entry points of libember_gpu: error text, version, device setup.
#include "common.cuh"

#include <cstring>
#include <map>
#include <mutex>
#include <utility>

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
        if (e != cudaSuccess || n == 0) rc = EMBER_ECUDA;
    });
    if (rc != EMBER_OK) set_error("no CUDA device is available");
    return rc;
}

// One memory pool per device, owned by the library: freed scratch blocks stay
// in it (release threshold: never) so that later calls allocate without
// driver calls, and the process's default pool is left as the application
// configured it.
int scratch_pool(cudaMemPool_t* pool) {
    static std::mutex mu;
    static std::map<int, cudaMemPool_t> pools;
    int dev = 0;
    EMBER_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    auto it = pools.find(dev);
    if (it != pools.end()) {
        *pool = it->second;
        return EMBER_OK;
    }
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t p = nullptr;
    EMBER_CUDA_TRY(cudaMemPoolCreate(&p, &props));
    uint64_t threshold = UINT64_MAX;
    EMBER_CUDA_TRY(cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &threshold));
    pools.emplace(dev, p);
    *pool = p;
    return EMBER_OK;
}

// cudaFuncAttributeMaxDynamicSharedMemorySize is a per-function, per-device
// setting shared by every handle and by graphs captured earlier: it is only
// ever raised, so that a launch sized for a small problem cannot invalidate
// the launches (or graph replays) of a larger one.
int raise_dynamic_smem(const void* func, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, size_t> set_to;
    int dev = 0;
    EMBER_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    size_t& cur = set_to[{func, dev}];
    if (bytes <= cur) return EMBER_OK;
    EMBER_CUDA_TRY(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)));
    cur = bytes;
    return EMBER_OK;
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
