// Batched tridiagonal integrator and diffusion stage (sm_103a, FP64).
//
// Scheme (reference: src/integrator.cpp:37-47, 133-204): the first step after
// initialize() is 8 first-order BDF sub-steps of h/8 sharing one Thomas
// factorisation of (A - 8/h I); later steps are second-order BDF with
// (A - 3/(2h) I) factorised once at the second step. Matrix rows come from
// DiffusionSystem::get_A / get_k (src/diffusionSystem.cpp:10-76) and the step
// size from FlameSolver::setDiffusionSolverState (src/flameSolver.cpp:702-718).
//
// The kernels here follow the reference's operation order with explicitly
// rounded intrinsics (no FMA contraction), so a system integrated by
// tri_step_serial is bitwise identical to the CPU restatement compiled with
// -ffp-contract=off.
#include "common.cuh"
#include "tridiag.cuh"

#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

namespace ember {

// ---------------------------------------------------------------- kernels --

__global__ void k_tridiag_step(TriBatchView v) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= v.n_systems) return;
    TriSys sys = v.system(s);
    int sc = v.step_count[s];
    double t = v.t[s];
    tri_step_serial(sys, t, v.h[s], sc, v.lu_b0[s]);
    v.step_count[s] = sc;
    v.t[s] = t;
}

__global__ void k_tridiag_integrate(TriBatchView v, const double* __restrict__ t_end) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= v.n_systems) return;
    TriSys sys = v.system(s);
    int sc = v.step_count[s];
    double t = v.t[s];
    double h = v.h[s];
    int st = tri_integrate_serial(sys, t, h, sc, v.lu_b0[s], t_end[s]);
    v.step_count[s] = sc;
    v.t[s] = t;
    v.h[s] = h;
    if (v.status) v.status[s] = st;
}

__global__ void k_tridiag_ydot(TriBatchView v, double* __restrict__ ydot) {
    int s = blockIdx.y;
    const int64_t o = v.off[s];
    const int N = static_cast<int>(v.off[s + 1] - o);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const double* a = v.a + o;
        const double* b = v.b + o;
        const double* c = v.c + o;
        const double* y = v.y + o;
        double r;
        if (i == 0) {
            r = __dadd_rn(__dadd_rn(__dmul_rn(b[0], y[0]), __dmul_rn(c[0], y[1])), v.k[o]);
        } else if (i == N - 1) {
            r = __dadd_rn(__dadd_rn(__dmul_rn(a[i], y[i - 1]), __dmul_rn(b[i], y[i])), v.k[o + i]);
        } else {
            r = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(a[i], y[i - 1]), __dmul_rn(b[i], y[i])),
                                    __dmul_rn(c[i], y[i + 1])),
                          v.k[o + i]);
        }
        ydot[o + i] = r;
    }
}

// Rows of DiffusionSystem::get_A / get_k for every (flame, variable) system.
// One thread per matrix row; each row is what the reference's sequence of
// writes (left BC, right BC, interior loop) leaves in it, starting from the
// zeroed arrays of TridiagonalIntegrator::resize.
__global__ void k_diffusion_rows(DiffusionView v) {
    for (int s = blockIdx.y; s < v.n_systems; s += gridDim.y) {
        const DiffSysInfo info = v.info[s];
        const int N = info.n;
        const double* x = v.x + info.grid_off;
        const int64_t o = info.off;
        const double* B = v.B + o;
        const double* D = v.D + o;
        for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < N; j += gridDim.x * blockDim.x) {
            DiffRow row = diffusion_row(j, N, x, info.alpha, info.left_bc, info.right_bc, B, D,
                                        v.wall_const ? v.wall_const[s] : 0.0);
            double k = v.split_const ? v.split_const[o + j] : 0.0;
            if (j == 0 && info.left_bc == EMBER_BC_WALL_FLUX) {
                double hh0 = __dsub_rn(x[1], x[0]);
                double wc = v.wall_const ? v.wall_const[s] : 0.0;
                double yi = v.y_inf ? v.y_inf[s] : 0.0;
                k = __dadd_rn(k, __dmul_rn(__dmul_rn(__ddiv_rn(__dmul_rn(B[0], static_cast<double>(info.alpha + 1)), hh0), wc), yi));
            }
            v.a[o + j] = row.a;
            v.b[o + j] = row.b;
            v.c[o + j] = row.c;
            v.k[o + j] = k;
        }
    }
}

// Step size rule of setDiffusionSolverState followed by initialize(t0, h) and
// integrateToTime(t1), one thread per system.
__global__ void k_diffusion_integrate_serial(DiffusionView v, TriBatchView tb, StageTime tm, double mult,
                                             double gdt) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= v.n_systems) return;
    double t0, t1;
    tm.get(t0, t1);
    const DiffSysInfo info = v.info[s];
    double h;
    if (v.h) {
        h = v.h[s];
    } else {
        h = diffusion_step_size(info.n, v.x + info.grid_off, v.B + info.off, v.D + info.off, mult, gdt);
    }
    TriSys sys = tb.system(s);
    int sc = 0;
    double t = t0;
    double lu_b0 = 0.0;
    int st = tri_integrate_serial(sys, t, h, sc, lu_b0, t1);
    if (v.status) v.status[s] = st;
}

// Adjoint of the stage of k_diffusion_integrate_serial, one thread per system.
__global__ void k_diffusion_adjoint(DiffusionView v, TriBatchView tb, StageTime tm, double mult, double gdt) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= v.n_systems) return;
    double t0, t1;
    tm.get(t0, t1);
    const DiffSysInfo info = v.info[s];
    double h;
    if (v.h) {
        h = v.h[s];
    } else {
        h = diffusion_step_size(info.n, v.x + info.grid_off, v.B + info.off, v.D + info.off, mult, gdt);
    }
    TriSys sys = tb.system(s);
    const int st = tri_integrate_adjoint(sys, t0, h, t1);
    if (v.status) v.status[s] = st;
}

}  // namespace ember

// ------------------------------------------------------------ C ABI: batch --

using namespace ember;

struct ember_tridiag_s {
    int n_systems = 0;
    int64_t n_total = 0;
    std::vector<int64_t> h_off;
    int64_t* off = nullptr;
    double* arr = nullptr;  // a b c k y yprev luc inv  (8 * n_total)
    double* sys = nullptr;  // t h lu_b0                (3 * n_systems)
    int* step_count = nullptr;
    int* status = nullptr;

    TriBatchView view() const {
        TriBatchView v;
        v.n_systems = n_systems;
        v.off = off;
        v.a = arr;
        v.b = arr + n_total;
        v.c = arr + 2 * n_total;
        v.k = arr + 3 * n_total;
        v.y = arr + 4 * n_total;
        v.yprev = arr + 5 * n_total;
        v.luc = arr + 6 * n_total;
        v.inv = arr + 7 * n_total;
        v.t = sys;
        v.h = sys + n_systems;
        v.lu_b0 = sys + 2 * n_systems;
        v.step_count = step_count;
        v.status = status;
        return v;
    }
};

static int check_batch(ember_tridiag b) {
    EMBER_CHECK_ARG(b != nullptr, "null ember_tridiag handle");
    return EMBER_OK;
}

static int copy_in(double* dst, const double* src, size_t n, int mem, cudaStream_t st) {
    EMBER_CHECK_ARG(src != nullptr, "null array argument");
    EMBER_CHECK_ARG(mem == EMBER_MEM_HOST || mem == EMBER_MEM_DEVICE, "bad mem flag %d", mem);
    EMBER_CUDA_TRY(cudaMemcpyAsync(dst, src, n * sizeof(double),
                                   mem == EMBER_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, st));
    return EMBER_OK;
}

extern "C" int ember_tridiag_create(int n_systems, const int64_t* offsets, ember_tridiag* out) {
    EMBER_CHECK_ARG(out != nullptr, "null output handle pointer");
    *out = nullptr;
    EMBER_CHECK_ARG(n_systems > 0, "n_systems must be positive (got %d)", n_systems);
    EMBER_CHECK_ARG(offsets != nullptr, "null offsets");
    EMBER_CHECK_ARG(offsets[0] == 0, "offsets[0] must be 0");
    for (int s = 0; s < n_systems; ++s)
        EMBER_CHECK_ARG(offsets[s + 1] - offsets[s] >= 2, "system %d has %lld points; at least 2 are needed", s,
                        (long long)(offsets[s + 1] - offsets[s]));
    EMBER_CHECK_ARG(offsets[n_systems] - offsets[n_systems - 1] < (int64_t(1) << 31), "system too large");
    EMBER_TRY(ensure_device());
    auto* b = new ember_tridiag_s;
    b->n_systems = n_systems;
    b->n_total = offsets[n_systems];
    b->h_off.assign(offsets, offsets + n_systems + 1);
    cudaError_t e = cudaMalloc(&b->off, sizeof(int64_t) * (n_systems + 1));
    if (e == cudaSuccess) e = cudaMalloc(&b->arr, sizeof(double) * 8 * b->n_total);
    if (e == cudaSuccess) e = cudaMalloc(&b->sys, sizeof(double) * 3 * n_systems);
    if (e == cudaSuccess) e = cudaMalloc(&b->step_count, sizeof(int) * n_systems);
    if (e == cudaSuccess) e = cudaMalloc(&b->status, sizeof(int) * n_systems);
    if (e == cudaSuccess) e = cudaMemcpy(b->off, offsets, sizeof(int64_t) * (n_systems + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(b->arr, 0, sizeof(double) * 8 * b->n_total);
    if (e == cudaSuccess) e = cudaMemset(b->sys, 0, sizeof(double) * 3 * n_systems);
    if (e == cudaSuccess) e = cudaMemset(b->step_count, 0, sizeof(int) * n_systems);
    if (e == cudaSuccess) e = cudaMemset(b->status, 0, sizeof(int) * n_systems);
    if (e != cudaSuccess) {
        set_error("ember_tridiag_create: %s", cudaGetErrorString(e));
        ember_tridiag_destroy(b);
        return e == cudaErrorMemoryAllocation ? EMBER_ENOMEM : EMBER_ECUDA;
    }
    *out = b;
    return EMBER_OK;
}

extern "C" int ember_tridiag_destroy(ember_tridiag b) {
    if (!b) return EMBER_OK;
    cudaFree(b->off);
    cudaFree(b->arr);
    cudaFree(b->sys);
    cudaFree(b->step_count);
    cudaFree(b->status);
    delete b;
    return EMBER_OK;
}

extern "C" int ember_tridiag_set_coefficients(ember_tridiag b, const double* a, const double* bb, const double* c,
                                              const double* k, int mem, void* stream) {
    EMBER_TRY(check_batch(b));
    cudaStream_t st = as_stream(stream);
    EMBER_TRY(copy_in(b->arr, a, b->n_total, mem, st));
    EMBER_TRY(copy_in(b->arr + b->n_total, bb, b->n_total, mem, st));
    EMBER_TRY(copy_in(b->arr + 2 * b->n_total, c, b->n_total, mem, st));
    EMBER_TRY(copy_in(b->arr + 3 * b->n_total, k, b->n_total, mem, st));
    return finish_call(mem, st);
}

extern "C" int ember_tridiag_set_y0(ember_tridiag b, const double* y0, int mem, void* stream) {
    EMBER_TRY(check_batch(b));
    cudaStream_t st = as_stream(stream);
    TriBatchView v = b->view();
    EMBER_TRY(copy_in(v.y, y0, b->n_total, mem, st));
    EMBER_CUDA_TRY(cudaMemsetAsync(b->step_count, 0, sizeof(int) * b->n_systems, st));
    return finish_call(mem, st);
}

extern "C" int ember_tridiag_initialize(ember_tridiag b, const double* t0, const double* h, int mem, void* stream) {
    EMBER_TRY(check_batch(b));
    cudaStream_t st = as_stream(stream);
    TriBatchView v = b->view();
    EMBER_TRY(copy_in(v.t, t0, b->n_systems, mem, st));
    EMBER_TRY(copy_in(v.h, h, b->n_systems, mem, st));
    EMBER_CUDA_TRY(cudaMemsetAsync(b->step_count, 0, sizeof(int) * b->n_systems, st));
    return finish_call(mem, st);
}

extern "C" int ember_tridiag_step(ember_tridiag b, void* stream) {
    EMBER_TRY(check_batch(b));
    cudaStream_t st = as_stream(stream);
    k_tridiag_step<<<blocks_for(b->n_systems, 128), 128, 0, st>>>(b->view());
    return finish_call(EMBER_MEM_DEVICE, st);
}

extern "C" int ember_tridiag_integrate_to_time(ember_tridiag b, const double* t_end, int mem, void* stream) {
    EMBER_TRY(check_batch(b));
    EMBER_CHECK_ARG(t_end != nullptr, "null t_end");
    cudaStream_t st = as_stream(stream);
    Scratch sc(st);
    const double* d_tend = nullptr;
    EMBER_TRY(stage_in(sc, t_end, b->n_systems, mem, st, &d_tend));
    k_tridiag_integrate<<<blocks_for(b->n_systems, 128), 128, 0, st>>>(b->view(), d_tend);
    EMBER_TRY(finish_call(mem, st));
    if (mem == EMBER_MEM_HOST) {
        std::vector<int> status(b->n_systems);
        EMBER_CUDA_TRY(cudaMemcpy(status.data(), b->status, sizeof(int) * b->n_systems, cudaMemcpyDeviceToHost));
        for (int s = 0; s < b->n_systems; ++s) {
            if (status[s] != 0) {
                set_error("system %d: integrate_to_time failed with status %d", s, status[s]);
                return EMBER_EFAIL;
            }
        }
    }
    return EMBER_OK;
}

extern "C" int ember_tridiag_get_state(ember_tridiag b, double* y, double* t, double* h, int mem, void* stream) {
    EMBER_TRY(check_batch(b));
    EMBER_CHECK_ARG(mem == EMBER_MEM_HOST || mem == EMBER_MEM_DEVICE, "bad mem flag %d", mem);
    cudaStream_t st = as_stream(stream);
    TriBatchView v = b->view();
    cudaMemcpyKind kind = mem == EMBER_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (y) EMBER_CUDA_TRY(cudaMemcpyAsync(y, v.y, sizeof(double) * b->n_total, kind, st));
    if (t) EMBER_CUDA_TRY(cudaMemcpyAsync(t, v.t, sizeof(double) * b->n_systems, kind, st));
    if (h) EMBER_CUDA_TRY(cudaMemcpyAsync(h, v.h, sizeof(double) * b->n_systems, kind, st));
    return finish_call(mem, st);
}

extern "C" int ember_tridiag_get_ydot(ember_tridiag b, double* ydot, int mem, void* stream) {
    EMBER_TRY(check_batch(b));
    EMBER_CHECK_ARG(ydot != nullptr, "null ydot");
    cudaStream_t st = as_stream(stream);
    Scratch sc(st);
    double* d_ydot = nullptr;
    EMBER_TRY(stage_buffer(sc, ydot, b->n_total, mem, &d_ydot));
    EMBER_CHECK_ARG(b->n_systems <= 65535, "get_ydot supports at most 65535 systems");
    int64_t nmax = 0;
    for (int s = 0; s < b->n_systems; ++s) nmax = std::max(nmax, b->h_off[s + 1] - b->h_off[s]);
    dim3 grid(std::min(blocks_for(nmax, 256), 64), b->n_systems);
    k_tridiag_ydot<<<grid, 256, 0, st>>>(b->view(), d_ydot);
    EMBER_TRY(stage_out(ydot, d_ydot, b->n_total, mem, st));
    return finish_call(mem, st);
}

// ------------------------------------------------------ C ABI: diffusion --

namespace ember {

int diffusion_serial_run(const DiffusionView& dv_in, double* y, double* work, int64_t n_vals, int nmax,
                         const StageTime& tm, double mult, double gdt, cudaStream_t st) {
    // Matrix rows and integrator workspace (a b c k | y_prev lu_c 1/den).
    DiffusionView dv = dv_in;
    dv.a = work;
    dv.b = work + n_vals;
    dv.c = work + 2 * n_vals;
    dv.k = work + 3 * n_vals;
    const int n_sys = dv.n_systems;
    dim3 grid_rows(std::min(blocks_for(nmax, 256), 32), std::min(n_sys, 65535));
    k_diffusion_rows<<<grid_rows, 256, 0, st>>>(dv);
    TriBatchView tb;
    tb.n_systems = n_sys;
    tb.off = nullptr;
    tb.info = dv.info;
    tb.a = dv.a;
    tb.b = dv.b;
    tb.c = dv.c;
    tb.k = dv.k;
    tb.y = y;
    tb.yprev = work + 4 * n_vals;
    tb.luc = work + 5 * n_vals;
    tb.inv = work + 6 * n_vals;
    k_diffusion_integrate_serial<<<blocks_for(n_sys, 64), 64, 0, st>>>(dv, tb, tm, mult, gdt);
    EMBER_CUDA_TRY(cudaGetLastError());
    return EMBER_OK;
}

int diffusion_adjoint_run(const DiffusionView& dv_in, double* y, double* work, int64_t n_vals, int nmax,
                          const StageTime& tm, double mult, double gdt, cudaStream_t st) {
    DiffusionView dv = dv_in;
    dv.a = work;
    dv.b = work + n_vals;
    dv.c = work + 2 * n_vals;
    dv.k = work + 3 * n_vals;
    const int n_sys = dv.n_systems;
    dim3 grid_rows(std::min(blocks_for(nmax, 256), 32), std::min(n_sys, 65535));
    k_diffusion_rows<<<grid_rows, 256, 0, st>>>(dv);
    TriBatchView tb;
    tb.n_systems = n_sys;
    tb.off = nullptr;
    tb.info = dv.info;
    tb.a = dv.a;
    tb.b = dv.b;
    tb.c = dv.c;
    tb.k = dv.k;
    tb.y = y;
    tb.yprev = work + 4 * n_vals;
    tb.luc = work + 5 * n_vals;
    tb.inv = work + 6 * n_vals;
    k_diffusion_adjoint<<<blocks_for(n_sys, 64), 64, 0, st>>>(dv, tb, tm, mult, gdt);
    EMBER_CUDA_TRY(cudaGetLastError());
    return EMBER_OK;
}

}  // namespace ember

namespace ember {

static bool pinned_host(const void* p) {
    if (!p) return true;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();  // a plain host pointer is no error
        return false;
    }
    return at.type == cudaMemoryTypeHost;
}

// A host-memory call on page-locked arrays, split into groups of flames that
// each copy in, integrate and copy out on a stream of their own, so that one
// group's copies overlap another's kernels. Each system is integrated by the
// same kernels as in one call, so the results are the same.
constexpr int kDiffusionPipelineChunks = 4;

static int diffusion_pipelined(int n_flames, const ember_diffusion_grid* grids, int n_vars, const double* x, const double* B,
                        const double* D, const double* split_const, double* y, const ember_diffusion_options* opts,
                        int* status, cudaStream_t st) {
    const int K = kDiffusionPipelineChunks;
    const int n_sys = n_flames * n_vars;
    std::vector<int64_t> pt(n_flames + 1, 0);
    for (int f = 0; f < n_flames; ++f) pt[f + 1] = pt[f] + grids[f].n_points;
    const int64_t n_pts = pt[n_flames], n_vals = n_pts * n_vars;
    // flame boundaries of the chunks, by values
    std::vector<int> fb(1, 0);
    for (int c = 1; c < K; ++c) {
        int f = fb.back();
        while (f < n_flames && pt[f] * K < pt[n_flames] * c) ++f;
        if (f > fb.back() && f < n_flames) fb.push_back(f);
    }
    fb.push_back(n_flames);
    const int nc = static_cast<int>(fb.size()) - 1;
    Scratch sc(st);
    double *dx, *dB, *dD, *dS = nullptr, *dy, *dh = nullptr, *dw = nullptr, *dyi = nullptr;
    int* dstat;
    EMBER_TRY(sc.alloc(&dx, size_t(n_pts)));
    EMBER_TRY(sc.alloc(&dB, size_t(n_vals)));
    EMBER_TRY(sc.alloc(&dD, size_t(n_vals)));
    if (split_const) EMBER_TRY(sc.alloc(&dS, size_t(n_vals)));
    EMBER_TRY(sc.alloc(&dy, size_t(n_vals)));
    if (opts->h) EMBER_TRY(sc.alloc(&dh, size_t(n_sys)));
    if (opts->wall_const) EMBER_TRY(sc.alloc(&dw, size_t(n_sys)));
    if (opts->y_inf) EMBER_TRY(sc.alloc(&dyi, size_t(n_sys)));
    EMBER_TRY(sc.alloc(&dstat, size_t(n_sys)));
    cudaStream_t cs[kDiffusionPipelineChunks] = {};
    cudaEvent_t ready = nullptr, done[kDiffusionPipelineChunks] = {};
    int rc = EMBER_OK;
    auto cu = [&](cudaError_t e, const char* what) {
        if (e != cudaSuccess && rc == EMBER_OK) {
            set_error("%s failed: %s", what, cudaGetErrorString(e));
            rc = EMBER_ECUDA;
        }
    };
    cu(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming), "cudaEventCreate");
    cu(cudaEventRecord(ready, st), "cudaEventRecord");  // after the allocations above
    for (int c = 0; c < nc && rc == EMBER_OK; ++c) {
        cu(cudaStreamCreateWithFlags(&cs[c], cudaStreamNonBlocking), "cudaStreamCreate");
        cu(cudaEventCreateWithFlags(&done[c], cudaEventDisableTiming), "cudaEventCreate");
        if (rc != EMBER_OK) break;
        cu(cudaStreamWaitEvent(cs[c], ready, 0), "cudaStreamWaitEvent");
        const int f0 = fb[c], f1 = fb[c + 1];
        const int64_t p0 = pt[f0], p1 = pt[f1], v0 = p0 * n_vars, v1 = p1 * n_vars;
        const int s0 = f0 * n_vars, s1 = f1 * n_vars;
        const size_t dbl = sizeof(double);
        cu(cudaMemcpyAsync(dx + p0, x + p0, dbl * (p1 - p0), cudaMemcpyHostToDevice, cs[c]), "cudaMemcpyAsync");
        cu(cudaMemcpyAsync(dB + v0, B + v0, dbl * (v1 - v0), cudaMemcpyHostToDevice, cs[c]), "cudaMemcpyAsync");
        cu(cudaMemcpyAsync(dD + v0, D + v0, dbl * (v1 - v0), cudaMemcpyHostToDevice, cs[c]), "cudaMemcpyAsync");
        if (dS) cu(cudaMemcpyAsync(dS + v0, split_const + v0, dbl * (v1 - v0), cudaMemcpyHostToDevice, cs[c]),
                   "cudaMemcpyAsync");
        cu(cudaMemcpyAsync(dy + v0, y + v0, dbl * (v1 - v0), cudaMemcpyHostToDevice, cs[c]), "cudaMemcpyAsync");
        ember_diffusion_options oc = *opts;
        if (dh) {
            cu(cudaMemcpyAsync(dh + s0, opts->h + s0, dbl * (s1 - s0), cudaMemcpyHostToDevice, cs[c]), "cudaMemcpyAsync");
            oc.h = dh + s0;
        }
        if (dw) {
            cu(cudaMemcpyAsync(dw + s0, opts->wall_const + s0, dbl * (s1 - s0), cudaMemcpyHostToDevice, cs[c]),
               "cudaMemcpyAsync");
            oc.wall_const = dw + s0;
        }
        if (dyi) {
            cu(cudaMemcpyAsync(dyi + s0, opts->y_inf + s0, dbl * (s1 - s0), cudaMemcpyHostToDevice, cs[c]),
               "cudaMemcpyAsync");
            oc.y_inf = dyi + s0;
        }
        if (rc != EMBER_OK) break;
        rc = ember_diffusion_integrate(f1 - f0, grids + f0, n_vars, dx + p0, dB + v0, dD + v0, dS ? dS + v0 : nullptr,
                                       dy + v0, &oc, dstat + s0, EMBER_MEM_DEVICE, cs[c]);
        if (rc != EMBER_OK) break;
        cu(cudaMemcpyAsync(y + v0, dy + v0, dbl * (v1 - v0), cudaMemcpyDeviceToHost, cs[c]), "cudaMemcpyAsync");
        cu(cudaEventRecord(done[c], cs[c]), "cudaEventRecord");
        cu(cudaStreamWaitEvent(st, done[c], 0), "cudaStreamWaitEvent");
    }
    std::vector<int> h_status(n_sys);
    if (rc == EMBER_OK && status)
        cu(cudaMemcpyAsync(h_status.data(), dstat, sizeof(int) * n_sys, cudaMemcpyDeviceToHost, st), "cudaMemcpyAsync");
    sc.release();
    if (rc == EMBER_OK) rc = finish_call(EMBER_MEM_HOST, st);
    else cudaStreamSynchronize(st);
    for (int c = 0; c < nc; ++c) {
        if (cs[c]) {
            cudaStreamSynchronize(cs[c]);
            cudaStreamDestroy(cs[c]);
        }
        if (done[c]) cudaEventDestroy(done[c]);
    }
    if (ready) cudaEventDestroy(ready);
    if (rc != EMBER_OK || !status) return rc;
    int bad = 0;
    for (int k = 0; k < n_sys; ++k) {
        status[k] = h_status[k];
        bad += h_status[k] != 0;
    }
    if (bad) {
        set_error("%d of %d diffusion systems failed (see status)", bad, n_sys);
        return EMBER_EFAIL;
    }
    return EMBER_OK;
}

}  // namespace ember

extern "C" int ember_diffusion_integrate(int n_flames, const ember_diffusion_grid* grids, int n_vars,
                                         const double* x, const double* B, const double* D,
                                         const double* split_const, double* y,
                                         const ember_diffusion_options* opts, int* status, int mem,
                                         void* stream) {
    EMBER_CHECK_ARG(n_flames > 0 && grids != nullptr, "need at least one flame");
    EMBER_CHECK_ARG(n_vars > 0, "n_vars must be positive");
    EMBER_CHECK_ARG(x && B && D && y && opts, "null array or options argument");
    EMBER_CHECK_ARG(mem == EMBER_MEM_HOST || mem == EMBER_MEM_DEVICE, "bad mem flag %d", mem);
    EMBER_TRY(ensure_device());
    const int n_sys = n_flames * n_vars;
    std::vector<DiffSysInfo> info(n_sys);
    int64_t n_pts = 0, n_vals = 0;
    for (int f = 0; f < n_flames; ++f) {
        const ember_diffusion_grid& g = grids[f];
        EMBER_CHECK_ARG(g.n_points >= 3, "flame %d: n_points must be >= 3 (got %d)", f, g.n_points);
        EMBER_CHECK_ARG(g.left_bc >= 0 && g.left_bc <= 4, "flame %d: bad left_bc %d", f, g.left_bc);
        EMBER_CHECK_ARG(g.right_bc == EMBER_BC_FIXED_VALUE || g.right_bc == EMBER_BC_ZERO_GRADIENT ||
                            g.right_bc == EMBER_BC_FLOATING,
                        "flame %d: bad right_bc %d", f, g.right_bc);
        EMBER_CHECK_ARG(g.alpha >= 0, "flame %d: bad alpha %d", f, g.alpha);
        for (int v = 0; v < n_vars; ++v) {
            DiffSysInfo& s = info[f * n_vars + v];
            s.n = g.n_points;
            s.left_bc = g.left_bc;
            s.right_bc = g.right_bc;
            s.alpha = g.alpha;
            s.grid_off = n_pts;
            s.off = n_vals + int64_t(v) * g.n_points;
        }
        n_pts += g.n_points;
        n_vals += int64_t(n_vars) * g.n_points;
    }
    EMBER_CHECK_ARG(opts->h != nullptr || (opts->dt_multiplier > 0 && opts->global_timestep > 0),
                    "without explicit h, dt_multiplier and global_timestep must be positive");
    EMBER_CHECK_ARG(opts->t_end > opts->t_start, "t_end must exceed t_start");
    EMBER_CHECK_ARG(opts->algorithm == EMBER_DIFFUSION_PARALLEL || opts->algorithm == EMBER_DIFFUSION_SERIAL,
                    "bad diffusion algorithm %d", opts->algorithm);

    cudaStream_t st = as_stream(stream);
    // large host-memory calls on page-locked arrays: copies overlap the kernels of other flame groups
    if (mem == EMBER_MEM_HOST && n_flames >= 2 * kDiffusionPipelineChunks && n_vals >= (int64_t(1) << 20) &&
        pinned_host(B) && pinned_host(D) && pinned_host(y) && pinned_host(split_const))
        return diffusion_pipelined(n_flames, grids, n_vars, x, B, D, split_const, y, opts, status, st);
    Scratch sc(st);
    DiffSysInfo* d_info = nullptr;
    EMBER_TRY(sc.alloc(&d_info, n_sys));
    EMBER_CUDA_TRY(cudaMemcpyAsync(d_info, info.data(), sizeof(DiffSysInfo) * n_sys, cudaMemcpyHostToDevice, st));

    DiffusionView dv;
    dv.n_systems = n_sys;
    dv.info = d_info;
    EMBER_TRY(stage_in(sc, x, n_pts, mem, st, &dv.x));
    EMBER_TRY(stage_in(sc, B, n_vals, mem, st, &dv.B));
    EMBER_TRY(stage_in(sc, D, n_vals, mem, st, &dv.D));
    EMBER_TRY(stage_in(sc, split_const, n_vals, mem, st, &dv.split_const));
    EMBER_TRY(stage_in(sc, opts->h, n_sys, mem, st, &dv.h));
    EMBER_TRY(stage_in(sc, opts->wall_const, n_sys, mem, st, &dv.wall_const));
    EMBER_TRY(stage_in(sc, opts->y_inf, n_sys, mem, st, &dv.y_inf));
    int* d_status = nullptr;
    EMBER_TRY(sc.alloc(&d_status, n_sys));
    dv.status = d_status;

    // State in/out.
    double* d_y = nullptr;
    if (mem == EMBER_MEM_DEVICE) {
        d_y = y;
    } else {
        EMBER_TRY(sc.alloc(&d_y, n_vals));
        EMBER_CUDA_TRY(cudaMemcpyAsync(d_y, y, sizeof(double) * n_vals, cudaMemcpyHostToDevice, st));
    }

    StageTime tm;
    tm.t0 = opts->t_start;
    tm.t1 = opts->t_end;
    if (opts->algorithm == EMBER_DIFFUSION_PARALLEL) {
        DiffusionWarpPlan plan;
        EMBER_TRY(diffusion_warp_plan_init(&plan, info, n_flames, n_vars, n_pts, sc, st));
        EMBER_TRY(diffusion_warp_geometry(plan, d_info, dv.x, st));
        EMBER_TRY(diffusion_warp_run(plan, dv, d_y, tm, opts->dt_multiplier, opts->global_timestep, st));
    } else {
        double* work = nullptr;
        EMBER_TRY(sc.alloc(&work, size_t(7) * n_vals));
        int nmax = 0;
        for (int f = 0; f < n_flames; ++f) nmax = std::max(nmax, grids[f].n_points);
        EMBER_TRY(diffusion_serial_run(dv, d_y, work, n_vals, nmax, tm, opts->dt_multiplier, opts->global_timestep,
                                       st));
    }
    if (mem == EMBER_MEM_HOST) {
        EMBER_CUDA_TRY(cudaMemcpyAsync(y, d_y, sizeof(double) * n_vals, cudaMemcpyDeviceToHost, st));
    }
    std::vector<int> h_status(n_sys);
    EMBER_CUDA_TRY(cudaGetLastError());
    if (status) {
        if (mem == EMBER_MEM_HOST) {
            EMBER_CUDA_TRY(cudaMemcpyAsync(h_status.data(), d_status, sizeof(int) * n_sys, cudaMemcpyDeviceToHost, st));
        } else {
            EMBER_CUDA_TRY(cudaMemcpyAsync(status, d_status, sizeof(int) * n_sys, cudaMemcpyDeviceToDevice, st));
        }
    }
    sc.release();
    EMBER_TRY(finish_call(mem, st));
    if (status && mem == EMBER_MEM_HOST) {
        int bad = 0;
        for (int s = 0; s < n_sys; ++s) {
            status[s] = h_status[s];
            if (h_status[s] != 0) ++bad;
        }
        if (bad) {
            set_error("%d of %d diffusion systems failed (see status)", bad, n_sys);
            return EMBER_EFAIL;
        }
    }
    return EMBER_OK;
}

// ------------------------------------------------- C ABI: diffusion adjoint --

extern "C" int ember_diffusion_adjoint(int n_flames, const ember_diffusion_grid* grids, int n_vars, const double* x,
                                       const double* B, const double* D, double* ybar,
                                       const ember_diffusion_options* opts, int* status, int mem, void* stream) {
    EMBER_CHECK_ARG(n_flames > 0 && grids != nullptr, "need at least one flame");
    EMBER_CHECK_ARG(n_vars > 0, "n_vars must be positive");
    EMBER_CHECK_ARG(x && B && D && ybar && opts, "null array or options argument");
    EMBER_CHECK_ARG(mem == EMBER_MEM_HOST || mem == EMBER_MEM_DEVICE, "bad mem flag %d", mem);
    EMBER_CHECK_ARG(opts->h != nullptr || (opts->dt_multiplier > 0 && opts->global_timestep > 0),
                    "without explicit h, dt_multiplier and global_timestep must be positive");
    EMBER_CHECK_ARG(opts->t_end > opts->t_start, "t_end must exceed t_start");
    EMBER_TRY(ensure_device());
    const int n_sys = n_flames * n_vars;
    std::vector<DiffSysInfo> info(n_sys);
    int64_t n_pts = 0, n_vals = 0;
    int nmax = 0;
    for (int f = 0; f < n_flames; ++f) {
        const ember_diffusion_grid& g = grids[f];
        EMBER_CHECK_ARG(g.n_points >= 3, "flame %d: n_points must be >= 3 (got %d)", f, g.n_points);
        EMBER_CHECK_ARG(g.left_bc >= 0 && g.left_bc <= 4, "flame %d: bad left_bc %d", f, g.left_bc);
        EMBER_CHECK_ARG(g.right_bc == EMBER_BC_FIXED_VALUE || g.right_bc == EMBER_BC_ZERO_GRADIENT ||
                            g.right_bc == EMBER_BC_FLOATING,
                        "flame %d: bad right_bc %d", f, g.right_bc);
        EMBER_CHECK_ARG(g.alpha >= 0, "flame %d: bad alpha %d", f, g.alpha);
        for (int v = 0; v < n_vars; ++v) {
            DiffSysInfo& s = info[f * n_vars + v];
            s.n = g.n_points;
            s.left_bc = g.left_bc;
            s.right_bc = g.right_bc;
            s.alpha = g.alpha;
            s.grid_off = n_pts;
            s.off = n_vals + int64_t(v) * g.n_points;
        }
        n_pts += g.n_points;
        n_vals += int64_t(n_vars) * g.n_points;
        nmax = std::max(nmax, g.n_points);
    }
    cudaStream_t st = as_stream(stream);
    Scratch sc(st);
    DiffSysInfo* d_info = nullptr;
    EMBER_TRY(sc.alloc(&d_info, n_sys));
    EMBER_CUDA_TRY(cudaMemcpyAsync(d_info, info.data(), sizeof(DiffSysInfo) * n_sys, cudaMemcpyHostToDevice, st));
    DiffusionView dv{};
    dv.n_systems = n_sys;
    dv.info = d_info;
    EMBER_TRY(stage_in(sc, x, n_pts, mem, st, &dv.x));
    EMBER_TRY(stage_in(sc, B, n_vals, mem, st, &dv.B));
    EMBER_TRY(stage_in(sc, D, n_vals, mem, st, &dv.D));
    EMBER_TRY(stage_in(sc, opts->h, n_sys, mem, st, &dv.h));
    EMBER_TRY(stage_in(sc, opts->wall_const, n_sys, mem, st, &dv.wall_const));
    int* d_status = nullptr;
    EMBER_TRY(stage_buffer(sc, status, n_sys, mem, &d_status));
    if (!d_status) EMBER_TRY(sc.alloc(&d_status, n_sys));
    dv.status = d_status;
    double* d_y = nullptr;
    if (mem == EMBER_MEM_DEVICE) {
        d_y = ybar;
    } else {
        EMBER_TRY(sc.alloc(&d_y, n_vals));
        EMBER_CUDA_TRY(cudaMemcpyAsync(d_y, ybar, sizeof(double) * n_vals, cudaMemcpyHostToDevice, st));
    }
    double* work = nullptr;
    EMBER_TRY(sc.alloc(&work, size_t(7) * n_vals));
    StageTime tm;
    tm.t0 = opts->t_start;
    tm.t1 = opts->t_end;
    EMBER_TRY(diffusion_adjoint_run(dv, d_y, work, n_vals, nmax, tm, opts->dt_multiplier, opts->global_timestep, st));
    if (mem == EMBER_MEM_HOST) {
        EMBER_CUDA_TRY(cudaMemcpyAsync(ybar, d_y, sizeof(double) * n_vals, cudaMemcpyDeviceToHost, st));
    }
    EMBER_TRY(stage_out(status, d_status, n_sys, mem, st));
    sc.release();
    return finish_call(mem, st);
}

// ------------------------------------------ allocation-free diffusion stage --
//
// Some callers cannot allocate device memory while they run a time step: a
// solver embedded in an application whose device memory is owned by another
// allocator (a framework's caching pool, a fixed budget set at start-up), or
// code that must keep its footprint constant after initialisation. For them,
// ember_diffusion_integrate_noalloc runs the same kernels as
// ember_diffusion_integrate with its workspace in the file-scope device array
// below instead of stream-ordered allocations. The array is sized for
// EMBER_NOALLOC_MAX_VALUES values and EMBER_NOALLOC_MAX_SYSTEMS systems and is
// held by every GPU that loads the library until the process exits.

namespace {

constexpr size_t kNoAllocWorkBytes = size_t(7) * EMBER_NOALLOC_MAX_VALUES * sizeof(double);
constexpr size_t kNoAllocInfoBytes = size_t(EMBER_NOALLOC_MAX_SYSTEMS) * sizeof(ember::DiffSysInfo);
constexpr size_t kNoAllocStatusBytes = size_t(EMBER_NOALLOC_MAX_SYSTEMS) * sizeof(int);
constexpr size_t kNoAllocBytes = kNoAllocWorkBytes + kNoAllocInfoBytes + kNoAllocStatusBytes;

// Workspace of the allocation-free entry point: matrix rows a, b, c, k and
// integrator arrays y_prev, lu_c, 1/denominator (7 doubles per value), then
// the per-system descriptors and status words.
static __device__ __align__(256) unsigned char g_diffusion_noalloc_scratch[kNoAllocBytes];

// Device address of the array per device; host code cannot use the symbol
// itself (in host code it names a host-side stand-in).
std::mutex g_noalloc_mutex;
void* g_noalloc_addr[64] = {};

int noalloc_scratch(void** out) {
    int dev = 0;
    EMBER_CUDA_TRY(cudaGetDevice(&dev));
    EMBER_CHECK_ARG(dev >= 0 && dev < 64, "device index %d out of range", dev);
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_diffusion_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            set_error("cudaGetSymbolAddress of the diffusion scratch failed: %s", cudaGetErrorString(e));
            return EMBER_ECUDA;
        }
        g_noalloc_addr[dev] = p;
    }
    *out = g_noalloc_addr[dev];
    return EMBER_OK;
}

// The per-system descriptors are built on the device from per-flame records
// passed by value as kernel parameters (copied with the launch), so the call
// needs neither a host buffer nor a host-to-device copy.
constexpr int kNoAllocFlamesPerLaunch = 256;

struct NoAllocFlame {
    int n, left_bc, right_bc, alpha;
    int64_t grid_off, val_off;
};

struct NoAllocFlames {
    int first, count, n_vars;
    NoAllocFlame f[kNoAllocFlamesPerLaunch];
};

__global__ void k_noalloc_info(const __grid_constant__ NoAllocFlames c, ember::DiffSysInfo* __restrict__ info) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= c.count * c.n_vars) return;
    const int fl = t / c.n_vars, v = t - fl * c.n_vars;
    const NoAllocFlame& g = c.f[fl];
    ember::DiffSysInfo s;
    s.n = g.n;
    s.left_bc = g.left_bc;
    s.right_bc = g.right_bc;
    s.alpha = g.alpha;
    s.grid_off = g.grid_off;
    s.off = g.val_off + int64_t(v) * g.n;
    info[int64_t(c.first + fl) * c.n_vars + v] = s;
}

}  // namespace

extern "C" int ember_diffusion_integrate_noalloc(int n_flames, const ember_diffusion_grid* grids, int n_vars,
                                                 const double* x, const double* B, const double* D,
                                                 const double* split_const, double* y,
                                                 const ember_diffusion_options* opts, int* status, void* stream) {
    EMBER_CHECK_ARG(n_flames > 0 && grids != nullptr, "need at least one flame");
    EMBER_CHECK_ARG(n_vars > 0, "n_vars must be positive");
    EMBER_CHECK_ARG(x && B && D && y && opts, "null array or options argument");
    const int64_t n_sys = int64_t(n_flames) * n_vars;
    EMBER_CHECK_ARG(n_sys <= EMBER_NOALLOC_MAX_SYSTEMS,
                    "ember_diffusion_integrate_noalloc: %lld systems exceed the maximum of %d "
                    "(use ember_diffusion_integrate)",
                    (long long)n_sys, EMBER_NOALLOC_MAX_SYSTEMS);
    int64_t n_pts = 0, n_vals = 0;
    int nmax = 0;
    for (int f = 0; f < n_flames; ++f) {
        const ember_diffusion_grid& g = grids[f];
        EMBER_CHECK_ARG(g.n_points >= 3, "flame %d: n_points must be >= 3 (got %d)", f, g.n_points);
        EMBER_CHECK_ARG(g.left_bc >= 0 && g.left_bc <= 4, "flame %d: bad left_bc %d", f, g.left_bc);
        EMBER_CHECK_ARG(g.right_bc == EMBER_BC_FIXED_VALUE || g.right_bc == EMBER_BC_ZERO_GRADIENT ||
                            g.right_bc == EMBER_BC_FLOATING,
                        "flame %d: bad right_bc %d", f, g.right_bc);
        EMBER_CHECK_ARG(g.alpha >= 0, "flame %d: bad alpha %d", f, g.alpha);
        n_pts += g.n_points;
        n_vals += int64_t(n_vars) * g.n_points;
        nmax = std::max(nmax, g.n_points);
    }
    EMBER_CHECK_ARG(n_vals <= EMBER_NOALLOC_MAX_VALUES,
                    "ember_diffusion_integrate_noalloc: %lld values (variables x points) exceed the maximum of %d "
                    "(use ember_diffusion_integrate)",
                    (long long)n_vals, EMBER_NOALLOC_MAX_VALUES);
    EMBER_CHECK_ARG(opts->h != nullptr || (opts->dt_multiplier > 0 && opts->global_timestep > 0),
                    "without explicit h, dt_multiplier and global_timestep must be positive");
    EMBER_CHECK_ARG(opts->t_end > opts->t_start, "t_end must exceed t_start");

    void* base = nullptr;
    EMBER_TRY(noalloc_scratch(&base));
    char* p = static_cast<char*>(base);
    double* work = reinterpret_cast<double*>(p);
    DiffSysInfo* d_info = reinterpret_cast<DiffSysInfo*>(p + kNoAllocWorkBytes);
    int* d_status = reinterpret_cast<int*>(p + kNoAllocWorkBytes + kNoAllocInfoBytes);
    cudaStream_t st = as_stream(stream);
    {
        NoAllocFlames c;
        int64_t pts = 0, vals = 0;
        for (int f0 = 0; f0 < n_flames; f0 += kNoAllocFlamesPerLaunch) {
            c.first = f0;
            c.count = std::min(kNoAllocFlamesPerLaunch, n_flames - f0);
            c.n_vars = n_vars;
            for (int i = 0; i < c.count; ++i) {
                const ember_diffusion_grid& g = grids[f0 + i];
                c.f[i] = NoAllocFlame{g.n_points, g.left_bc, g.right_bc, g.alpha, pts, vals};
                pts += g.n_points;
                vals += int64_t(n_vars) * g.n_points;
            }
            k_noalloc_info<<<blocks_for(int64_t(c.count) * n_vars, 128), 128, 0, st>>>(c, d_info);
            EMBER_CUDA_TRY(cudaGetLastError());
        }
    }

    DiffusionView dv;
    dv.n_systems = static_cast<int>(n_sys);
    dv.info = d_info;
    dv.x = x;
    dv.B = B;
    dv.D = D;
    dv.split_const = split_const;
    dv.h = opts->h;
    dv.wall_const = opts->wall_const;
    dv.y_inf = opts->y_inf;
    dv.status = status ? status : d_status;
    dv.a = work;
    dv.b = work + EMBER_NOALLOC_MAX_VALUES;
    dv.c = work + 2 * int64_t(EMBER_NOALLOC_MAX_VALUES);
    dv.k = work + 3 * int64_t(EMBER_NOALLOC_MAX_VALUES);
    dim3 grid_rows(std::min(blocks_for(nmax, 256), 32), std::min<int64_t>(n_sys, 65535));
    k_diffusion_rows<<<grid_rows, 256, 0, st>>>(dv);

    TriBatchView tb;
    tb.n_systems = static_cast<int>(n_sys);
    tb.off = nullptr;
    tb.info = d_info;
    tb.a = dv.a;
    tb.b = dv.b;
    tb.c = dv.c;
    tb.k = dv.k;
    tb.y = y;
    tb.yprev = work + 4 * int64_t(EMBER_NOALLOC_MAX_VALUES);
    tb.luc = work + 5 * int64_t(EMBER_NOALLOC_MAX_VALUES);
    tb.inv = work + 6 * int64_t(EMBER_NOALLOC_MAX_VALUES);
    StageTime tm;
    tm.t0 = opts->t_start;
    tm.t1 = opts->t_end;
    k_diffusion_integrate_serial<<<blocks_for(n_sys, 64), 64, 0, st>>>(dv, tb, tm, opts->dt_multiplier,
                                                                        opts->global_timestep);
    EMBER_CUDA_TRY(cudaGetLastError());
    return EMBER_OK;
}
