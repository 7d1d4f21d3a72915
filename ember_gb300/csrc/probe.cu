// Device throughput probes used as roofline denominators: the FP64 FMA pipe
// (DFMA) and the FP64 tensor path (DMMA m8n8k4). Both run a fixed amount of
// independent work on every SM and are timed with CUDA events.
#include "common.cuh"

namespace ember {

template <int CHAINS>
__global__ void k_probe_dfma(double* out, int iters, double s) {
    double acc[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) acc[c] = threadIdx.x * 1e-3 + c;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < CHAINS; ++c) acc[c] = fma(acc[c], s, 0.25);
    }
    double r = 0.0;
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) r += acc[c];
    if (r == 1234.5) out[0] = r;  // keep the work observable
}

__global__ void k_probe_dmma(double* out, int iters) {
    double a = 1.0 + threadIdx.x * 1e-6, b = 0.5;
    double c0 = 0.0, c1 = 0.0, c2 = 0.0, c3 = 0.0;
    for (int i = 0; i < iters; ++i) {
        asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                     : "+d"(c0), "+d"(c1)
                     : "d"(a), "d"(b));
        asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                     : "+d"(c2), "+d"(c3)
                     : "d"(b), "d"(a));
    }
    if (c0 + c1 + c2 + c3 == 1234.5) out[0] = c0;
}

}  // namespace ember

using namespace ember;

extern "C" int ember_probe_fp64_rate(int kind, double* flops_per_second) {
    EMBER_CHECK_ARG(flops_per_second != nullptr, "null output");
    EMBER_CHECK_ARG(kind == 0 || kind == 1, "kind must be 0 (DFMA) or 1 (DMMA)");
    EMBER_TRY(ensure_device());
    int dev = 0, sms = 0;
    EMBER_CUDA_TRY(cudaGetDevice(&dev));
    EMBER_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    double* out = nullptr;
    EMBER_CUDA_TRY(cudaMalloc(&out, sizeof(double)));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int threads = 256, blocks = sms * 8;
    const int iters = kind == 0 ? 4096 : 8192;
    float best_ms = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        if (kind == 0)
            k_probe_dfma<8><<<blocks, threads>>>(out, iters, 0.999999);
        else
            k_probe_dmma<<<blocks, threads>>>(out, iters);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best_ms) best_ms = ms;
    }
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) {
        set_error("probe kernel failed: %s", cudaGetErrorString(err));
        return EMBER_ECUDA;
    }
    double flops;
    if (kind == 0)
        flops = 2.0 * 8.0 * iters * double(threads) * blocks;
    else
        flops = 1024.0 * iters * double(threads / 32) * blocks;  // 2 mma (8x8x4, 512 flop each) per iter per warp
    *flops_per_second = flops / (best_ms * 1e-3);
    return EMBER_OK;
}
