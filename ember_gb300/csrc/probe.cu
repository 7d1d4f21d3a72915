// Device throughput probes used as roofline denominators: the FP64 FMA pipe
// (DFMA) and the FP64 tensor path (DMMA m8n8k4), both run as a fixed amount
// of independent work on every SM and timed with CUDA events; and the issue
// cost of single FP64 warp instructions (clock64 per CTA), which shows how
// the pipe is shared between warps and lanes. Also the kinetics kernels'
// exp / log functions evaluated on an array, for their parity tests.
#include "common.cuh"
#include "emath.cuh"

#include <algorithm>
#include <vector>

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

// Issue cost of FP64 warp instructions: one CTA of `warps` warps per SM,
// lanes below `active` running `iters` x CHAINS operations (MODE 0: DFMA,
// 1: DADD, 2: DMUL, 3: division, 4: fmax, 5: compare-and-select, 6: the
// reciprocal 1.0 / x, 7: the reciprocal as __drcp_rn), clocked per CTA with
// clock64.
template <int CHAINS, int MODE>
__global__ void k_probe_issue(double* sink, long long* cyc, int iters, int active) {
    const int lane = threadIdx.x & 31;
    double acc[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) acc[c] = 1.0 + threadIdx.x * 1e-3 + c;
    const double s = 0.999999;
    __syncthreads();
    long long t0;
    asm volatile("mov.u64 %0, %%clock64;" : "=l"(t0));
    if (lane < active) {
        for (int i = 0; i < iters; ++i) {
#pragma unroll
            for (int c = 0; c < CHAINS; ++c) {
                if (MODE == 0) acc[c] = fma(acc[c], s, 0.25);
                else if (MODE == 1) acc[c] = acc[c] + s;
                else if (MODE == 2) acc[c] = acc[c] * s;
                else if (MODE == 3) acc[c] = s / acc[c];
                else if (MODE == 4) acc[c] = fmax(acc[c] - s, s * 0.5);
                else if (MODE == 5) acc[c] = (acc[c] < s) ? acc[c] + s : acc[c] - s;
                else if (MODE == 6) acc[c] = 1.0 / acc[c];
                else acc[c] = __drcp_rn(acc[c]);
            }
        }
    }
    __syncthreads();
    long long t1;
    asm volatile("mov.u64 %0, %%clock64;" : "=l"(t1));
    double r = 0.0;
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) r += acc[c];
    if (r == 1234.5) sink[0] = r;
    if (threadIdx.x == 0) cyc[blockIdx.x] = t1 - t0;
}

// y[i] = em_exp, em_log, em_log10 or em_exp10 (op 0..3) of x[i]
__global__ void k_math_eval(int op, const double* x, double* y, int64_t n) {
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = x[i];
    y[i] = op == 0 ? em_exp(v) : op == 1 ? em_log(v) : op == 2 ? em_log10(v) : em_exp10(v);
}

}  // namespace ember

using namespace ember;

extern "C" int ember_probe_fp64_issue(int op, int chains, int warps, int active_lanes, double* cycles_per_inst) {
    EMBER_CHECK_ARG(cycles_per_inst != nullptr, "null output");
    EMBER_CHECK_ARG(op >= 0 && op <= 7,
                    "op must be 0 (DFMA), 1 (DADD), 2 (DMUL), 3 (division), 4 (fmax + DADD), 5 (compare + DADD), "
                    "6 (1.0 / x) or 7 (__drcp_rn)");
    EMBER_CHECK_ARG(chains == 1 || chains == 8, "chains must be 1 or 8");
    EMBER_CHECK_ARG(warps >= 1 && warps <= 32, "warps must be 1..32");
    EMBER_CHECK_ARG(active_lanes >= 1 && active_lanes <= 32, "active_lanes must be 1..32");
    EMBER_TRY(ensure_device());
    int dev = 0, sms = 0;
    EMBER_CUDA_TRY(cudaGetDevice(&dev));
    EMBER_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    double* sink = nullptr;
    long long* cyc = nullptr;
    EMBER_CUDA_TRY(cudaMalloc(&sink, sizeof(double)));
    if (cudaMalloc(&cyc, sizeof(long long) * sms) != cudaSuccess) {
        cudaFree(sink);
        set_error("probe: no device memory");
        return EMBER_ECUDA;
    }
    const int iters = (op == 3 || op >= 6) ? 256 : 1024;
    void (*kern)(double*, long long*, int, int) = nullptr;
    switch (op * 2 + (chains == 8)) {
        case 0: kern = k_probe_issue<1, 0>; break;
        case 1: kern = k_probe_issue<8, 0>; break;
        case 2: kern = k_probe_issue<1, 1>; break;
        case 3: kern = k_probe_issue<8, 1>; break;
        case 4: kern = k_probe_issue<1, 2>; break;
        case 5: kern = k_probe_issue<8, 2>; break;
        case 6: kern = k_probe_issue<1, 3>; break;
        case 7: kern = k_probe_issue<8, 3>; break;
        case 8: kern = k_probe_issue<1, 4>; break;
        case 9: kern = k_probe_issue<8, 4>; break;
        case 10: kern = k_probe_issue<1, 5>; break;
        case 11: kern = k_probe_issue<8, 5>; break;
        case 12: kern = k_probe_issue<1, 6>; break;
        case 13: kern = k_probe_issue<8, 6>; break;
        case 14: kern = k_probe_issue<1, 7>; break;
        default: kern = k_probe_issue<8, 7>; break;
    }
    for (int rep = 0; rep < 2; ++rep) kern<<<sms, warps * 32>>>(sink, cyc, iters, active_lanes);
    cudaError_t err = cudaDeviceSynchronize();
    std::vector<long long> h(sms);
    if (err == cudaSuccess) err = cudaMemcpy(h.data(), cyc, sizeof(long long) * sms, cudaMemcpyDeviceToHost);
    cudaFree(sink);
    cudaFree(cyc);
    if (err != cudaSuccess) {
        set_error("probe kernel failed: %s", cudaGetErrorString(err));
        return EMBER_ECUDA;
    }
    std::sort(h.begin(), h.end());
    *cycles_per_inst = double(h[sms / 2]) / (double(iters) * chains);
    return EMBER_OK;
}

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

extern "C" int ember_math_eval(int op, const double* x, double* y, int64_t n) {
    EMBER_CHECK_ARG(op >= 0 && op <= 3, "op must be 0 (exp), 1 (log), 2 (log10) or 3 (exp10), got %d", op);
    EMBER_CHECK_ARG(n >= 0 && n <= (int64_t(1) << 26), "n must be in [0, 2^26], got %lld", (long long)n);
    EMBER_CHECK_ARG(n == 0 || (x != nullptr && y != nullptr), "null array");
    if (n == 0) return EMBER_OK;
    EMBER_TRY(ensure_device());
    double* d = nullptr;
    EMBER_CUDA_TRY(cudaMalloc(&d, sizeof(double) * 2 * size_t(n)));
    cudaError_t err = cudaMemcpy(d, x, sizeof(double) * size_t(n), cudaMemcpyHostToDevice);
    if (err == cudaSuccess) {
        k_math_eval<<<unsigned((n + 255) / 256), 256>>>(op, d, d + n, n);
        err = cudaGetLastError();
    }
    if (err == cudaSuccess) err = cudaMemcpy(y, d + n, sizeof(double) * size_t(n), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (err != cudaSuccess) {
        set_error("math kernel failed: %s", cudaGetErrorString(err));
        return EMBER_ECUDA;
    }
    return EMBER_OK;
}
