// Device-side building blocks of the tridiagonal integrator and the
// diffusion matrix (see tridiag.cu for the scheme and references).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../../include/ember_gpu.h"

namespace ember {

class Scratch;

// One (flame, variable) diffusion system.
struct DiffSysInfo {
    int64_t off;       // first element in the variable-major value arrays
    int64_t grid_off;  // first grid point of the flame in x
    int n;             // number of points
    int left_bc, right_bc, alpha;
};

// One system's arrays, already offset.
struct TriSys {
    int N;
    const double* a;
    const double* b;
    const double* c;
    const double* k;
    double* y;
    double* yprev;
    double* luc;
    double* inv;
};

// Arrays of a whole batch (CSR via off[], or via info[] for diffusion).
struct TriBatchView {
    int n_systems;
    const int64_t* off;
    const DiffSysInfo* info;
    const double* a;
    const double* b;
    const double* c;
    const double* k;
    double* y;
    double* yprev;
    double* luc;
    double* inv;
    double* t;
    double* h;
    double* lu_b0;
    int* step_count;
    int* status;

    __device__ TriSys system(int s) const {
        int64_t o;
        int n;
        if (off) {
            o = off[s];
            n = static_cast<int>(off[s + 1] - o);
        } else {
            o = info[s].off;
            n = info[s].n;
        }
        TriSys r;
        r.N = n;
        r.a = a + o;
        r.b = b + o;
        r.c = c + o;
        r.k = k + o;
        r.y = y + o;
        r.yprev = yprev + o;
        r.luc = luc + o;
        r.inv = inv + o;
        return r;
    }
};

struct DiffusionView {
    int n_systems;
    const DiffSysInfo* info;
    const double* x;
    const double* B;
    const double* D;
    const double* split_const;
    const double* h;
    const double* wall_const;
    const double* y_inf;
    double* a;
    double* b;
    double* c;
    double* k;
    int* status;
};

// Interval [t0, t1] of one diffusion stage: given on the host, or read from a
// device clock t (for graph replays, where launch parameters are fixed):
// t0 = t + f0*dt (t itself when f0 == 0) and t1 = t + f1*dt, the stage
// boundaries of SplitSolver::integrateSplitTerms (src/splitSolver.cpp:60-75).
struct StageTime {
    double t0 = 0.0, t1 = 0.0;
    const double* t_dev = nullptr;
    double f0 = 0.0, f1 = 0.0, dt = 0.0;

    __device__ void get(double& a, double& b) const {
        if (t_dev) {
            const double t = *t_dev;
            a = f0 == 0.0 ? t : t + f0 * dt;
            b = t + f1 * dt;
        } else {
            a = t0;
            b = t1;
        }
    }
};

// Status codes of one system.
enum : int {
    TRI_OK = 0,
    TRI_BAD_STEP = -1,    // h <= 0, not finite, or more than 2^31 steps requested
    TRI_NONFINITE = -2,   // the result contains a NaN or an infinity
};

// ---- Thomas factorisation of (A - shift*I): lu_c and 1/denominator ------
// Reference: src/integrator.cpp:147-152 (BDF1) and 176-181 (BDF2).
__device__ __forceinline__ void tri_factor_serial(const TriSys& s, double shift, double& lu_b0) {
    double lb0 = __dsub_rn(s.b[0], shift);
    double lc = __ddiv_rn(s.c[0], lb0);
    s.luc[0] = lc;
    for (int i = 1; i < s.N; ++i) {
        double den = __dsub_rn(__dsub_rn(s.b[i], shift), __dmul_rn(lc, s.a[i]));
        double iv = __ddiv_rn(1.0, den);
        s.inv[i] = iv;
        lc = __dmul_rn(s.c[i], iv);
        s.luc[i] = lc;
    }
    lu_b0 = lb0;
}

// Forward elimination and back substitution in place: y holds the right-hand
// side on entry and the solution on exit. Reference: src/integrator.cpp:158-168.
__device__ __forceinline__ void tri_solve_serial(const TriSys& s, double lu_b0) {
    double d = __ddiv_rn(s.y[0], lu_b0);
    s.y[0] = d;
    for (int i = 1; i < s.N; ++i) {
        d = __dmul_rn(__dsub_rn(s.y[i], __dmul_rn(d, s.a[i])), s.inv[i]);
        s.y[i] = d;
    }
    double yn = d;
    for (int i = s.N - 2; i >= 0; --i) {
        yn = __dsub_rn(s.y[i], __dmul_rn(s.luc[i], yn));
        s.y[i] = yn;
    }
}

// TridiagonalIntegrator::step (src/integrator.cpp:133-204).
__device__ __forceinline__ void tri_step_serial(const TriSys& s, double& t, double h, int& step_count,
                                                double& lu_b0) {
    if (step_count == 0) {
        for (int i = 0; i < s.N; ++i) s.yprev[i] = s.y[i];
        const double h8 = __ddiv_rn(h, 8.0);
        tri_factor_serial(s, __ddiv_rn(1.0, h8), lu_b0);
        for (int sub = 0; sub < 8; ++sub) {
            for (int i = 0; i < s.N; ++i) s.y[i] = __dsub_rn(__ddiv_rn(-s.y[i], h8), s.k[i]);
            tri_solve_serial(s, lu_b0);
        }
    } else {
        if (step_count == 1) tri_factor_serial(s, __ddiv_rn(3.0, __dmul_rn(2.0, h)), lu_b0);
        const double h2 = __dmul_rn(2.0, h);
        for (int i = 0; i < s.N; ++i) {
            double ynm1 = s.y[i];
            double r = __dsub_rn(__dadd_rn(__ddiv_rn(__dmul_rn(-2.0, ynm1), h), __ddiv_rn(s.yprev[i], h2)), s.k[i]);
            s.yprev[i] = ynm1;
            s.y[i] = r;
        }
        tri_solve_serial(s, lu_b0);
    }
    ++step_count;
    t = __dadd_rn(t, h);
}

// Integrator::integrateToTime (src/integrator.cpp:37-47). Returns a TRI_* code.
__device__ __forceinline__ int tri_integrate_serial(const TriSys& s, double& t, double& h, int& step_count,
                                                    double& lu_b0, double t_end) {
    double q = __dadd_rn(__ddiv_rn(__dsub_rn(t_end, t), h), 1e-5);
    if (!(h > 0.0) || !(q < 2147483647.0)) return TRI_BAD_STEP;
    int n_steps = q >= 1.0 ? static_cast<int>(q) : 1;
    h = __ddiv_rn(__dsub_rn(t_end, t), static_cast<double>(n_steps));
    for (int i = 0; i < n_steps; ++i) tri_step_serial(s, t, h, step_count, lu_b0);
    for (int i = 0; i < s.N; ++i)
        if (!isfinite(s.y[i])) return TRI_NONFINITE;
    return TRI_OK;
}

// ---- adjoint of a stage --------------------------------------------------
// The stage is linear in y: y_out = M y_in + (terms of k). The adjoint maps
// ybar = d phi / d y_out to d phi / d y_in = M^T ybar by running the sub-steps
// backwards with transposed solves; L^T of L = A - shift I has sub-diagonal
// c_{i-1}, diagonal b_i - shift and super-diagonal a_{i+1}.
__device__ __forceinline__ void tri_factor_transpose(const TriSys& s, double shift, double& lu_b0) {
    double lb0 = s.b[0] - shift;
    double lc = s.N > 1 ? s.a[1] / lb0 : 0.0;
    s.luc[0] = lc;
    for (int i = 1; i < s.N; ++i) {
        double den = (s.b[i] - shift) - lc * s.c[i - 1];
        double iv = 1.0 / den;
        s.inv[i] = iv;
        lc = i + 1 < s.N ? s.a[i + 1] * iv : 0.0;
        s.luc[i] = lc;
    }
    lu_b0 = lb0;
}

// Solve L^T x = r in place (r in v).
__device__ __forceinline__ void tri_solve_transpose(const TriSys& s, double lu_b0, double* v) {
    double d = v[0] / lu_b0;
    v[0] = d;
    for (int i = 1; i < s.N; ++i) {
        d = (v[i] - d * s.c[i - 1]) * s.inv[i];
        v[i] = d;
    }
    double yn = d;
    for (int i = s.N - 2; i >= 0; --i) {
        yn = v[i] - s.luc[i] * yn;
        v[i] = yn;
    }
}

// Adjoint of initialize(t, h) + integrateToTime(t_end) of one system: s.y
// holds ybar on entry and the adjoint of the start state on exit; s.yprev is
// workspace. Returns a TRI_* code (the forward's step rule).
__device__ __forceinline__ int tri_integrate_adjoint(const TriSys& s, double t, double h, double t_end) {
    double q = (t_end - t) / h + 1e-5;
    if (!(h > 0.0) || !(q < 2147483647.0)) return TRI_BAD_STEP;
    const int n_steps = q >= 1.0 ? static_cast<int>(q) : 1;
    h = (t_end - t) / static_cast<double>(n_steps);
    double lu_b0 = 0.0;
    double* g = s.y;       // adjoint of the newest state
    double* gp = s.yprev;  // adjoint of the state before it
    for (int i = 0; i < s.N; ++i) gp[i] = 0.0;
    if (n_steps > 1) {
        // BDF2 steps j = n-1..1: Y_{8+j} = L2^{-1} (-(2/h) Y_{8+j-1} + (1/(2h)) P_j - k),
        // P_1 = Y_0 (the state before the first step), P_j = Y_{8+j-2}.
        tri_factor_transpose(s, 3.0 / (2.0 * h), lu_b0);
        for (int j = n_steps - 1; j >= 1; --j) {
            tri_solve_transpose(s, lu_b0, g);
            for (int i = 0; i < s.N; ++i) {
                const double w = g[i];
                g[i] = gp[i] - (2.0 / h) * w;
                gp[i] = (1.0 / (2.0 * h)) * w;  // for j = 1: the term of Y_0, added at the end
            }
        }
    }
    // BDF1 sub-steps m = 7..0: Y_{m+1} = L1^{-1} (-Y_m / h8 - k)
    const double h8 = h / 8.0;
    tri_factor_transpose(s, 1.0 / h8, lu_b0);
    for (int m = 7; m >= 0; --m) {
        tri_solve_transpose(s, lu_b0, g);
        for (int i = 0; i < s.N; ++i) g[i] = -g[i] / h8;
    }
    for (int i = 0; i < s.N; ++i) {
        g[i] += gp[i];
        if (!isfinite(g[i])) return TRI_NONFINITE;
    }
    return TRI_OK;
}

// ---- DiffusionSystem::get_A (src/diffusionSystem.cpp:10-66) -------------
struct DiffRow {
    double a, b, c;
};

__device__ __forceinline__ double grid_pow(double v, int alpha) {
    if (alpha == 0) return 1.0;
    if (alpha == 1) return v;
    return pow(v, static_cast<double>(alpha));
}

// c1_j = 0.5 B_j / (dlj_j r_j) and c2_j = rphalf_j (D_j + D_{j+1}) / hh_j for
// 1 <= j <= N-2; both are zero elsewhere (they are never assigned there).
__device__ __forceinline__ double diff_c1(int j, int N, const double* x, int alpha, const double* B) {
    if (j < 1 || j > N - 2) return 0.0;
    double dlj = __dmul_rn(0.5, __dsub_rn(x[j + 1], x[j - 1]));
    return __ddiv_rn(__dmul_rn(0.5, B[j]), __dmul_rn(dlj, grid_pow(x[j], alpha)));
}

__device__ __forceinline__ double diff_c2(int j, int N, const double* x, int alpha, const double* D) {
    if (j < 1 || j > N - 2) return 0.0;
    double hh = __dsub_rn(x[j + 1], x[j]);
    double rph = grid_pow(__dmul_rn(0.5, __dadd_rn(x[j], x[j + 1])), alpha);
    return __ddiv_rn(__dmul_rn(rph, __dadd_rn(D[j], D[j + 1])), hh);
}

// Row j of the diffusion matrix: the final contents left by the reference's
// writes in order (left boundary, right boundary, interior loop).
__device__ __forceinline__ DiffRow diffusion_row(int j, int N, const double* x, int alpha, int left_bc,
                                                 int right_bc, const double* B, const double* D,
                                                 double wall_const) {
    DiffRow r{0.0, 0.0, 0.0};
    int j_start = 1;
    if (left_bc == EMBER_BC_FIXED_VALUE) {
        j_start = 1;
    } else if (left_bc == EMBER_BC_CONTROL_VOLUME) {
        j_start = 1;
        if (j == 0) {
            double hh0 = __dsub_rn(x[1], x[0]);
            double c0 = __ddiv_rn(__dmul_rn(__dmul_rn(B[0], static_cast<double>(alpha + 1)), __dadd_rn(D[0], D[1])),
                                  __dmul_rn(__dmul_rn(2.0, hh0), hh0));
            r.b = -c0;
            r.c = c0;
        }
    } else if (left_bc == EMBER_BC_WALL_FLUX) {
        j_start = 1;
        if (j == 0) {
            double hh0 = __dsub_rn(x[1], x[0]);
            double c0 = __ddiv_rn(__dmul_rn(B[0], static_cast<double>(alpha + 1)), hh0);
            double d = __dmul_rn(0.5, __dadd_rn(D[0], D[1]));
            r.b = __dmul_rn(-c0, __dadd_rn(__ddiv_rn(d, hh0), wall_const));
            r.c = __ddiv_rn(__dmul_rn(d, c0), hh0);
        }
    } else {  // ZeroGradient (and any other value)
        j_start = 2;
        if (j == 1) {
            double c11 = diff_c1(1, N, x, alpha, B);
            double c21 = diff_c2(1, N, x, alpha, D);
            r.b = __dmul_rn(-c11, c21);
            r.c = __dmul_rn(c11, c21);
        }
    }
    int j_stop;
    if (right_bc == EMBER_BC_FIXED_VALUE) {
        j_stop = N - 1;
    } else {
        j_stop = N - 2;
        if (j == N - 2) {
            double c1 = diff_c1(N - 2, N, x, alpha, B);
            double c2m = diff_c2(N - 3, N, x, alpha, D);
            r.a = __dmul_rn(c1, c2m);
            r.b = __dmul_rn(-c1, c2m);
        }
    }
    if (j >= j_start && j < j_stop) {
        double c1 = diff_c1(j, N, x, alpha, B);
        double c2m = diff_c2(j - 1, N, x, alpha, D);
        double c2 = diff_c2(j, N, x, alpha, D);
        r.a = __dmul_rn(c1, c2m);
        r.b = __dmul_rn(-c1, __dadd_rn(c2m, c2));
        r.c = __dmul_rn(c1, c2);
    }
    return r;
}

// h = min(mult * min_{1<=j<=N-2} dlj_j^2 / (B_j D_j), gdt)
// (FlameSolver::setDiffusionSolverState, src/flameSolver.cpp:707-709).
__device__ __forceinline__ double diffusion_step_size(int N, const double* x, const double* B, const double* D,
                                                      double mult, double gdt) {
    double m = 0.0;
    for (int j = 1; j <= N - 2; ++j) {
        double dlj = __dmul_rn(0.5, __dsub_rn(x[j + 1], x[j - 1]));
        double v = __ddiv_rn(__dmul_rn(dlj, dlj), __dmul_rn(B[j], D[j]));
        if (j == 1 || v < m) m = v;
    }
    double h = __dmul_rn(mult, m);
    return gdt < h ? gdt : h;  // std::min(h, gdt)
}

// Warp-parallel diffusion stage (diffusion_warp.cu). A plan holds the
// per-system workspace, the geometric factors of every grid point, the
// largest-first task list (systems packed onto the warps of a CTA) and the
// work counter of one batch of flames.
struct DiffusionWarpPlan {
    int n_sys = 0, n_flames = 0, n_vars = 0, nmax = 0;
    int64_t n_pts = 0;
    int n_tasks = 0, blocks = 0;
    double* ws = nullptr;
    double2* geo = nullptr;
    int64_t* ws_off = nullptr;
    int* tasks = nullptr;
    unsigned int* counter = nullptr;
};

// Allocate the plan's buffers from `sc` and upload its tables (host copies of
// the system descriptors in `info`).
int diffusion_warp_plan_init(DiffusionWarpPlan* p, const std::vector<DiffSysInfo>& info, int n_flames, int n_vars,
                             int64_t n_pts, Scratch& sc, cudaStream_t st);
// Bytes diffusion_warp_plan_init takes from its Scratch.
size_t diffusion_warp_plan_bytes(const std::vector<DiffSysInfo>& info, int64_t n_pts);
// Geometric factors of every grid point (x: all flames' coordinates).
int diffusion_warp_geometry(const DiffusionWarpPlan& p, const DiffSysInfo* d_info, const double* x, cudaStream_t st);
// One stage: rows, step size and integration of every system of `dv`, with
// one to eight warps per system; `y` (device, variable-major per flame) in place.
int diffusion_warp_run(const DiffusionWarpPlan& p, const DiffusionView& dv, double* y, const StageTime& tm,
                       double mult, double gdt, cudaStream_t st);

// Adjoint of a stage (B, D, split constants fixed): y holds d phi / d y_out
// on entry and d phi / d y_in on exit; work: 7 * n_vals doubles.
int diffusion_adjoint_run(const DiffusionView& dv, double* y, double* work, int64_t n_vals, int nmax,
                          const StageTime& tm, double mult, double gdt, cudaStream_t st);

// Serial (bitwise reference order) stage on a device workspace of
// 7 * n_vals doubles: rows, then one thread per system (tridiag.cu).
int diffusion_serial_run(const DiffusionView& dv, double* y, double* work, int64_t n_vals, int nmax,
                         const StageTime& tm, double mult, double gdt, cudaStream_t st);

}  // namespace ember
