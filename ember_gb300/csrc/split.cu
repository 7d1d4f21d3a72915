// Device split step for a batch of flames (the orchestration of
// SplitSolver::step / integrateSplitTerms, src/splitSolver.cpp:34-121, with
// the stage hooks of FlameSolver, src/flameSolver.cpp:702-854, and
// FlameSolver::finishStep's mass-fraction correction, src/flameSolver.cpp:
// 219-224, 942-949).
//
// One step on the device, with every array resident in HBM:
//   split constants from the previous step's time derivatives;
//   diffusion [t, t+dt/4] and [t+dt/4, t+dt/2];
//   source term [t, t+dt] (QSS or BDF, every grid point of every flame);
//   diffusion [t+dt/2, t+3dt/4] and [t+3dt/4, t+dt];
//   time derivatives (delta / dt - split constant), mass-fraction
//   correction, t += dt.
// The convection stages of the reference are not integrated here (the
// convection system is not part of this library); a caller that has them
// supplies their effect through ddt_cross. Stage times are read from a device
// clock, so a captured step replays as a CUDA graph.
//
// Layouts: the flame state is point-major [point][n_vars] (U, T, Y_0..), as
// FlameSolver::state; the diffusion stages work on a variable-major copy
// [flame][variable][point] (the rows DiffusionSystem integrates), produced
// and consumed by transpose kernels around each pair of diffusion stages.
//
// Compiled with --fmad=false: every multiply and add is rounded as written,
// so with the serial diffusion algorithm the step reproduces the CPU
// restatement bit for bit.
#include "common.cuh"
#include "convection.cuh"
#include "source.cuh"
#include "transport.cuh"
#include "tridiag.cuh"

#include <algorithm>
#include <vector>

namespace ember {
namespace {

struct SplitTables {
    int64_t n_pts;
    int n;                     // variables per point
    const int64_t* vm_base;    // per point: variable-major index of variable 0
    const int* npt;            // per point: points of its flame (variable stride)
};

__device__ __forceinline__ int64_t vm_index(const SplitTables& t, int64_t p, int v) {
    return t.vm_base[p] + int64_t(v) * t.npt[p];
}

// Point-major state -> variable-major copy (and the stage-start snapshot).
__global__ void k_to_varmajor(SplitTables tb, const double* __restrict__ state, double* __restrict__ yv,
                              double* __restrict__ ystart) {
    const int64_t total = tb.n_pts * tb.n;
    for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < total; e += int64_t(gridDim.x) * blockDim.x) {
        const int64_t p = e / tb.n;
        const int v = static_cast<int>(e - p * tb.n);
        const int64_t q = vm_index(tb, p, v);
        const double val = state[e];
        yv[q] = val;
        ystart[q] = val;
    }
}

// Variable-major copy -> point-major state (and, when given, a snapshot).
__global__ void k_to_pointmajor(SplitTables tb, const double* __restrict__ yv, double* __restrict__ state,
                                double* __restrict__ snap) {
    const int64_t total = tb.n_pts * tb.n;
    for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < total; e += int64_t(gridDim.x) * blockDim.x) {
        const int64_t p = e / tb.n;
        const int v = static_cast<int>(e - p * tb.n);
        const double val = yv[vm_index(tb, p, v)];
        state[e] = val;
        if (snap) snap[e] = val;
    }
}

// deltaDiff += state - startState after a diffusion stage (variable-major),
// and the next stage's start snapshot.
__global__ void k_diff_accumulate(int64_t n_vals, const double* __restrict__ yv, double* __restrict__ ystart,
                                  double* __restrict__ delta) {
    for (int64_t q = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; q < n_vals; q += int64_t(gridDim.x) * blockDim.x) {
        const double y = yv[q];
        delta[q] = delta[q] + (y - ystart[q]);
        ystart[q] = y;
    }
}

// Start of a step (SplitSolver::step, src/splitSolver.cpp:38-46): split
// constants from the previous step's time derivatives, deltaDiff = 0.
// Without convection, balanced splitting of the two integrated operators
// gives each half of the total rate: c_D = (f_S + f_X - f_D) / 2,
// c_S = (f_D + f_X - f_S) / 2. With convection (ddt_conv set) the reference's
// three-operator constants: c_D = (f_S + f_C + f_X - 3 f_D) / 4,
// c_C = (f_S + f_D + f_X - 3 f_C) / 4, c_S = (f_C + f_D + f_X - f_S) / 2.
// The plain Strang variant uses c_D = f_X and zero for the others.
__global__ void k_split_begin(SplitTables tb, int balanced, const double* __restrict__ ddt_diff,
                              const double* __restrict__ ddt_prod, const double* __restrict__ ddt_cross,
                              double* __restrict__ sc_diff, double* __restrict__ sc_diff_vm,
                              double* __restrict__ sc_prod, double* __restrict__ delta_diff_vm,
                              const double* __restrict__ ddt_conv, double* __restrict__ sc_conv,
                              double* __restrict__ sc_conv_vm, double* __restrict__ delta_conv_vm) {
    const int64_t total = tb.n_pts * tb.n;
    for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < total; e += int64_t(gridDim.x) * blockDim.x) {
        const int64_t p = e / tb.n;
        const int v = static_cast<int>(e - p * tb.n);
        const double fx = ddt_cross ? ddt_cross[e] : 0.0;
        double cd, cs, cc = 0.0;
        if (ddt_conv) {
            const double fd = ddt_diff[e], fs = ddt_prod[e], fc = ddt_conv[e];
            if (balanced) {
                cd = 0.25 * (((fs + fc) + fx) - 3.0 * fd);
                cc = 0.25 * (((fs + fd) + fx) - 3.0 * fc);
                cs = 0.5 * (((fc + fd) + fx) - fs);
            } else {
                cd = fx;
                cs = 0.0;
            }
        } else if (balanced) {
            cd = 0.5 * ((ddt_prod[e] + fx) - ddt_diff[e]);
            cs = 0.5 * ((ddt_diff[e] + fx) - ddt_prod[e]);
        } else {
            cd = fx;
            cs = 0.0;
        }
        const int64_t q = vm_index(tb, p, v);
        sc_diff[e] = cd;
        sc_diff_vm[q] = cd;
        sc_prod[e] = cs;
        delta_diff_vm[q] = 0.0;
        if (ddt_conv) {
            sc_conv[e] = cc;
            sc_conv_vm[q] = cc;
            delta_conv_vm[q] = 0.0;
        }
    }
}

// FlameSolver::prepareIntegrators' density derivative for the convection
// stage (src/flameSolver.cpp:208-212): ddt = ddtConv + ddtDiff + ddtProd
// (+ ddtCross when balanced), drho/dt = -rho (ddt_T / T + W sum_k ddt_Yk / W_k),
// with rho and the mean molecular weight W of the step-start state (mass
// fractions clipped at zero and normalised, sums in species order).
__global__ void k_density_derivative(int64_t n_pts, int n, int balanced, double pressure,
                                     const double* __restrict__ W, const double* __restrict__ state,
                                     const double* __restrict__ ddt_conv, const double* __restrict__ ddt_diff,
                                     const double* __restrict__ ddt_prod, const double* __restrict__ ddt_cross,
                                     double* __restrict__ drhodt) {
    const double R = 6.02214076e26 * 1.380649e-23;
    for (int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; p < n_pts; p += int64_t(gridDim.x) * blockDim.x) {
        const double* s = state + p * n;
        const int64_t e0 = p * n;
        double ysum = 0.0;
        for (int k = 2; k < n; ++k) ysum = ysum + (s[k] < 0.0 ? 0.0 : s[k]);
        const double rnorm = 1.0 / ysum;
        double acc = 0.0;
        for (int k = 2; k < n; ++k) acc = acc + ((s[k] < 0.0 ? 0.0 : s[k]) * rnorm) / W[k - 2];
        const double wmx = 1.0 / acc;
        const double T = s[1];
        const double rho = (pressure * wmx) / (R * T);
        auto ddt = [&](int64_t e) {
            double d = (ddt_conv[e] + ddt_diff[e]) + ddt_prod[e];
            if (balanced && ddt_cross) d = d + ddt_cross[e];
            return d;
        };
        double tmp = 0.0;
        for (int k = 2; k < n; ++k) tmp = tmp + ddt(e0 + k) / W[k - 2];
        drhodt[p] = -rho * (ddt(e0 + 1) / T + tmp * wmx);
    }
}

// Local duration of the source stage, (t + dt) - t, and its start time.
__global__ void k_stage_dt(int64_t n_pts, const double* __restrict__ t_dev, double dt, double* __restrict__ dtp) {
    const double t = *t_dev;
    const double d = (t + dt) - t;
    for (int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; p < n_pts; p += int64_t(gridDim.x) * blockDim.x)
        dtp[p] = d;
}

// End of a step: SplitSolver::calculateTimeDerivatives (src/splitSolver.cpp:
// 27-32) with deltaProd = state(after S) - state(before S).
__global__ void k_split_end(SplitTables tb, double dt, const double* __restrict__ xS, const double* __restrict__ xD2,
                            const double* __restrict__ delta_diff_vm, const double* __restrict__ sc_diff,
                            const double* __restrict__ sc_prod, double* __restrict__ ddt_diff,
                            double* __restrict__ ddt_prod, const double* __restrict__ delta_conv_vm,
                            const double* __restrict__ sc_conv, double* __restrict__ ddt_conv) {
    const int64_t total = tb.n_pts * tb.n;
    for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < total; e += int64_t(gridDim.x) * blockDim.x) {
        const int64_t p = e / tb.n;
        const int v = static_cast<int>(e - p * tb.n);
        const double delta_prod = xS[e] - xD2[e];
        ddt_diff[e] = delta_diff_vm[vm_index(tb, p, v)] / dt - sc_diff[e];
        ddt_prod[e] = delta_prod / dt - sc_prod[e];
        if (ddt_conv) ddt_conv[e] = delta_conv_vm[vm_index(tb, p, v)] / dt - sc_conv[e];
    }
}

// FlameSolver::correctMassFractions (src/flameSolver.cpp:942-949): Cantera's
// setState_TPY followed by getMassFractions, i.e. negative mass fractions
// set to zero and the rest scaled by 1 / (their sequential sum). One thread
// per point.
__global__ void k_correct_mass_fractions(int64_t n_pts, int n, double* __restrict__ state) {
    for (int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; p < n_pts; p += int64_t(gridDim.x) * blockDim.x) {
        double* Y = state + p * n + 2;
        double sum = 0.0;
        for (int k = 0; k < n - 2; ++k) sum = sum + (Y[k] < 0.0 ? 0.0 : Y[k]);  // std::max(y, 0.0)
        const double r = 1.0 / sum;
        for (int k = 0; k < n - 2; ++k) Y[k] = (Y[k] < 0.0 ? 0.0 : Y[k]) * r;
    }
}

__global__ void k_advance_clock(double* t_dev, double dt) {
    if (threadIdx.x == 0 && blockIdx.x == 0) *t_dev = *t_dev + dt;
}

// Running count of failed systems / points (status != 0) over the steps.
__global__ void k_count_failures(int n, const int* __restrict__ status, unsigned long long* count) {
    unsigned long long local = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) local += status[i] != 0;
    if (local) atomicAdd(count, local);
}

// ---- objectives ------------------------------------------------------------

__global__ void k_gather_TY(int64_t n_pts, int n, const double* __restrict__ state, double* __restrict__ T,
                            double* __restrict__ Y) {
    const int S = n - 2;
    const int64_t total = n_pts * S;
    for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < total; e += int64_t(gridDim.x) * blockDim.x) {
        const int64_t p = e / S;
        const int k = static_cast<int>(e - p * S);
        Y[e] = state[p * n + 2 + k];
        if (k == 0) T[p] = state[p * n + 1];
    }
}

// FlameSolver::calculateQdot (src/flameSolver.cpp:926-940): q_j = -sum_k
// wdot_k h_k (sequential sum), and q_j / cp_j.
__global__ void k_qdot(int64_t n_pts, int S, const double* __restrict__ net, const double* __restrict__ hk,
                       const double* __restrict__ cp, double* __restrict__ qdot, double* __restrict__ qcp) {
    for (int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; p < n_pts; p += int64_t(gridDim.x) * blockDim.x) {
        double s = 0.0;
        for (int k = 0; k < S; ++k) s = s + net[p * S + k] * hk[p * S + k];
        const double q = -s;
        qdot[p] = q;
        qcp[p] = q / cp[p];
    }
}

// mathUtils::integrate (src/mathUtils.h:338-358) of a natural cubic spline
// through (x, y) (computeSplines, src/mathUtils.h:189-237), one thread per
// flame; work: 3 doubles per point.
__device__ double spline_integral(int n, const double* x, const double* y, double* u, double* v, double* z) {
    // h_i and b_i are recomputed where used (same expressions, same rounding).
    auto hh = [&](int i) { return x[i + 1] - x[i]; };
    auto bb = [&](int i) { return (y[i + 1] - y[i]) / hh(i); };
    u[0] = 0;
    v[0] = 0;
    u[1] = 2 * (hh(0) + hh(1));
    v[1] = 6 * (bb(1) - bb(0));
    for (int i = 2; i < n - 1; i++) {
        u[i] = 2 * (hh(i - 1) + hh(i)) - hh(i - 1) * hh(i - 1) / u[i - 1];
        v[i] = 6 * (bb(i) - bb(i - 1)) - hh(i - 1) * v[i - 1] / u[i - 1];
    }
    z[n - 1] = 0;
    for (int i = n - 2; i > 0; i--) z[i] = (v[i] - hh(i) * z[i + 1]) / u[i];
    z[0] = 0;
    double I = 0;
    for (int i = 0; i < n - 1; i++) {
        const double h = hh(i);
        const double c0 = y[i];
        const double c1 = -h / 6 * z[i + 1] - h / 3 * z[i] + (y[i + 1] - y[i]) / h;
        const double c2 = 0.5 * z[i];
        const double c3 = (z[i + 1] - z[i]) / (6 * h);
        const double dx = x[i + 1] - x[i];
        I += dx * (c0 + dx * (c1 / 2 + dx * (c2 / 3 + dx * c3 / 4)));
    }
    return I;
}

// FlameSolver::getHeatReleaseRate / getConsumptionSpeed (src/flameSolver.cpp:
// 951-961): Q = integral of q dx, S_c = integral of q/cp dx / (rho_u (T_b - T_u)).
__global__ void k_flame_objectives(int n_flames, const int* __restrict__ npts, const int64_t* __restrict__ goff,
                                   const double* __restrict__ x, const double* __restrict__ qdot,
                                   const double* __restrict__ qcp, const double* __restrict__ T,
                                   const double* __restrict__ rho_u, const int* __restrict__ ju,
                                   const int* __restrict__ jb, double* __restrict__ work,
                                   double* __restrict__ heat_release, double* __restrict__ cons_speed) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_flames) return;
    const int n = npts[f];
    const int64_t o = goff[f];
    double* u = work + 3 * o;
    double* v = u + n;
    double* z = v + n;
    const double Q = spline_integral(n, x + o, qdot + o, u, v, z);
    if (heat_release) heat_release[f] = Q;
    if (cons_speed) {
        const double QoverCp = spline_integral(n, x + o, qcp + o, u, v, z);
        const double rhouDeltaT = rho_u[f] * (T[o + jb[f]] - T[o + ju[f]]);
        cons_speed[f] = QoverCp / rhouDeltaT;
    }
}

// ---- adjoint of the objectives and of the mass-fraction correction ------

// d I / d y_i of the spline integral I(y) = mathUtils::integrate(x, y): the
// integral is linear in y, so these weights are the reverse pass of
// spline_integral (one thread per flame; work: 4 doubles per point).
__global__ void k_spline_weights(int n_flames, const int* __restrict__ npts, const int64_t* __restrict__ goff,
                                 const double* __restrict__ x, double* __restrict__ work, double* __restrict__ w) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_flames) return;
    const int n = npts[f];
    const int64_t o = goff[f];
    const double* xf = x + o;
    double* wf = w + o;
    double* u = work + 4 * o;
    double* vb = u + n;
    double* zb = vb + n;
    double* bb = zb + n;
    auto hh = [&](int i) { return xf[i + 1] - xf[i]; };
    u[1] = 2 * (hh(0) + hh(1));
    for (int i = 2; i < n - 1; i++) u[i] = 2 * (hh(i - 1) + hh(i)) - hh(i - 1) * hh(i - 1) / u[i - 1];
    for (int i = 0; i < n; ++i) {
        wf[i] = 0.0;
        zb[i] = 0.0;
        vb[i] = 0.0;
        bb[i] = 0.0;
    }
    // I = sum_i h_i y_i + h_i^2 c1_i / 2 + h_i^3 c2_i / 3 + h_i^4 c3_i / 4
    for (int i = 0; i < n - 1; i++) {
        const double h = hh(i);
        wf[i] += h - 0.5 * h;
        wf[i + 1] += 0.5 * h;
        const double h3 = h * h * h;
        zb[i] += -h3 / 24.0;
        zb[i + 1] += -h3 / 24.0;
    }
    // z_i = (v_i - h_i z_{i+1}) / u_i, computed for i = n-2..1 (z_0 = z_{n-1} = 0)
    for (int i = 1; i <= n - 2; i++) {
        const double t = zb[i] / u[i];
        vb[i] += t;
        zb[i + 1] -= hh(i) * t;
    }
    // v_i = 6 (b_i - b_{i-1}) - h_{i-1} v_{i-1} / u_{i-1} (i >= 2), v_1 = 6 (b_1 - b_0)
    for (int i = n - 2; i >= 2; i--) {
        bb[i] += 6 * vb[i];
        bb[i - 1] -= 6 * vb[i];
        vb[i - 1] -= hh(i - 1) / u[i - 1] * vb[i];
    }
    if (n >= 3) {
        bb[1] += 6 * vb[1];
        bb[0] -= 6 * vb[1];
    }
    // b_i = (y_{i+1} - y_i) / h_i
    for (int i = 0; i < n - 1; i++) {
        const double t = bb[i] / hh(i);
        wf[i + 1] += t;
        wf[i] -= t;
    }
}

// Per point: gq = d J / d qdot, gcp = d J / d cp, gT = d J / d T for
// J = sum_f wq_f Q_f + ws_f S_c,f (one thread per flame).
__global__ void k_objective_weights(int n_flames, const int* __restrict__ npts, const int64_t* __restrict__ goff,
                                    const double* __restrict__ omega, const double* __restrict__ qdot,
                                    const double* __restrict__ cp, const double* __restrict__ T,
                                    const double* __restrict__ wq, const double* __restrict__ ws,
                                    const double* __restrict__ rho_u, const int* __restrict__ ju,
                                    const int* __restrict__ jb, const double* __restrict__ sc_val,
                                    double* __restrict__ gq, double* __restrict__ gcp, double* __restrict__ gT) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_flames) return;
    const int n = npts[f];
    const int64_t o = goff[f];
    const double a = wq ? wq[f] : 0.0;
    const double b = ws ? ws[f] : 0.0;
    double D = 1.0, dT = 1.0;
    if (b != 0.0) {
        dT = T[o + jb[f]] - T[o + ju[f]];
        D = rho_u[f] * dT;
    }
    for (int i = 0; i < n; ++i) {
        const int64_t p = o + i;
        const double c = cp[p];
        gq[p] = omega[p] * (a + (b != 0.0 ? b / (c * D) : 0.0));
        gcp[p] = b != 0.0 ? -b * omega[p] * qdot[p] / (c * c * D) : 0.0;
        gT[p] = 0.0;
    }
    if (b != 0.0) {
        const double s = sc_val[f];
        gT[o + jb[f]] += -b * s / dT;
        gT[o + ju[f]] += b * s / dT;
    }
}

// Adjoint of k_correct_mass_fractions: Y' = max(Y, 0) / sum max(Y, 0).
__global__ void k_correct_mass_fractions_adjoint(int64_t n_pts, int n, const double* __restrict__ xF,
                                                 double* __restrict__ ybar) {
    for (int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; p < n_pts; p += int64_t(gridDim.x) * blockDim.x) {
        const double* Y = xF + p * n + 2;
        double* g = ybar + p * n + 2;
        double sum = 0.0;
        for (int k = 0; k < n - 2; ++k) sum = sum + (Y[k] < 0.0 ? 0.0 : Y[k]);
        const double r = 1.0 / sum;
        double dot = 0.0;
        for (int k = 0; k < n - 2; ++k) dot = fma((Y[k] < 0.0 ? 0.0 : Y[k]) * r, g[k], dot);
        for (int k = 0; k < n - 2; ++k) g[k] = Y[k] < 0.0 ? 0.0 : (g[k] - dot) * r;
    }
}

// Sum of per-point rows [n_pts][R] (two arrays) over points, in point order.
__global__ void k_sum_rows2(int64_t n_pts, int R, const double* __restrict__ a, const double* __restrict__ b,
                            double* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < R; i += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int64_t j = 0; j < n_pts; ++j) s += a[j * R + i] + b[j * R + i];
        out[i] = s;
    }
}

// ---- properties of the step start (FlameSolver::step) ------------------------

// prepareIntegrators (src/flameSolver.cpp:156-172), not quasi-2D: B and D of
// every (point, variable) in the variable-major layout of the diffusion stages.
__global__ void k_bd_from_props(SplitTables tb, int S, const double* __restrict__ rho, const double* __restrict__ cp,
                                const double* __restrict__ lam, const double* __restrict__ mu,
                                const double* __restrict__ rhoD, double* __restrict__ B, double* __restrict__ D) {
    const int64_t total = tb.n_pts * tb.n;
    for (int64_t e = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; e < total; e += int64_t(gridDim.x) * blockDim.x) {
        const int64_t p = e / tb.n;
        const int v = static_cast<int>(e - p * tb.n);
        const int64_t q = vm_index(tb, p, v);
        if (v == 0) {
            B[q] = 1.0 / rho[p];
            D[q] = mu[p];
        } else if (v == 1) {
            B[q] = 1.0 / (rho[p] * cp[p]);
            D[q] = lam[p];
        } else {
            B[q] = 1.0 / rho[p];
            D[q] = rhoD[p * S + (v - 2)];
        }
    }
}

// Point p's Fick flux of species k to the right, jFick(k, j) of
// updateCrossTerms (src/flameSolver.cpp:555-556).
__device__ __forceinline__ double fick_flux(const double* st, const double* rhoD, int n, int S, int64_t p, int k,
                                            double hh) {
    return (-0.5 * (rhoD[p * S + k] + rhoD[(p + 1) * S + k])) * ((st[(p + 1) * n + 2 + k] - st[p * n + 2 + k]) / hh);
}

// jCorr = -sum_k jFick (no thermal diffusion: jSoret = 0), jCorr[jj] = 0
// (src/flameSolver.cpp:551-565), and the smoothing system's B = lambda/(rho cp)
// (573-577). One thread per point.
__global__ void k_jcorr_fick(int64_t n_pts, int n, int S, const int* __restrict__ pt_local,
                             const int* __restrict__ pt_flame, const int* __restrict__ flame_npts,
                             const double* __restrict__ x, const double* __restrict__ st,
                             const double* __restrict__ rhoD, const double* __restrict__ lam,
                             const double* __restrict__ rho, const double* __restrict__ cp, double* __restrict__ jcorr,
                             double* __restrict__ jB) {
    for (int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; p < n_pts; p += int64_t(gridDim.x) * blockDim.x) {
        const int i = pt_local[p];
        const int N = flame_npts[pt_flame[p]];
        double jc = 0.0;
        if (i < N - 1) {
            const double hh = x[p + 1] - x[p];
            for (int k = 0; k < S; ++k) jc = jc - fick_flux(st, rhoD, n, S, p, k, hh);
        }
        jcorr[p] = jc;
        jB[p] = lam[p] / (rho[p] * cp[p]);
    }
}

// Step size of the jCorr smoothing (src/flameSolver.cpp:579-582), one warp
// per flame. Every lane starts from dt and keeps the smaller candidate (a NaN
// candidate is never taken, as in the reference's std::min(dt, cand)), so the
// warp minimum equals the sequential one exactly.
__global__ void k_jcorr_h(int n_flames, const int64_t* __restrict__ goff, const int* __restrict__ npts,
                          const double* __restrict__ x, const double* __restrict__ jB, double mult, double gdt,
                          double* __restrict__ h) {
    const int f = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (f >= n_flames) return;
    const double* xf = x + goff[f];
    const double* bf = jB + goff[f];
    double dt = gdt;
    for (int j = 1 + lane; j < npts[f] - 1; j += 32) {
        const double dlj = 0.5 * (xf[j + 1] - xf[j - 1]);
        const double cand = ((mult * dlj) * dlj) / bf[j];
        dt = (cand < dt) ? cand : dt;
    }
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const double o = __shfl_xor_sync(0xffffffffu, dt, off);
        dt = (o < dt) ? o : dt;
    }
    if (lane == 0) h[f] = dt;
}

__device__ __forceinline__ double grid_pow(double v, int alpha) { return alpha == 0 ? 1.0 : (alpha == 1 ? v : pow(v, alpha)); }

// Species cross terms dYdtCross and the heat-capacity flux sums sumcpj
// (src/flameSolver.cpp:591-609, jSoret = 0); zero at the boundary points.
__global__ void k_cross_species(int64_t n_pts, int n, int S, const int* __restrict__ pt_local,
                                const int* __restrict__ pt_flame, const int* __restrict__ flame_npts,
                                const ember_diffusion_grid* __restrict__ grids, const double* __restrict__ x,
                                const double* __restrict__ st, const double* __restrict__ rhoD,
                                const double* __restrict__ cpS, const double* __restrict__ W,
                                const double* __restrict__ rho, const double* __restrict__ jcorr,
                                double* __restrict__ sumcpj, double* __restrict__ cross) {
    for (int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; p < n_pts; p += int64_t(gridDim.x) * blockDim.x) {
        const int i = pt_local[p];
        const int f = pt_flame[p];
        const int N = flame_npts[f];
        if (i == 0 || i == N - 1) {
            for (int k = 0; k < S; ++k) cross[p * n + 2 + k] = 0.0;
            sumcpj[p] = 0.0;
            continue;
        }
        const int alpha = grids[f].alpha;
        const double r = grid_pow(x[p], alpha);
        const double rph = grid_pow(0.5 * (x[p] + x[p + 1]), alpha);
        const double rphm = grid_pow(0.5 * (x[p - 1] + x[p]), alpha);
        const double dlj = 0.5 * (x[p + 1] - x[p - 1]);
        const double hh = x[p + 1] - x[p];
        const double c = -0.5 / ((r * rho[p]) * dlj);
        const double jc = jcorr[p], jcm = jcorr[p - 1];
        double s = 0.0;
        for (int k = 0; k < S; ++k) {
            const double yk = st[p * n + 2 + k], yk1 = st[(p + 1) * n + 2 + k], ykm = st[(p - 1) * n + 2 + k];
            cross[p * n + 2 + k] = c * ((rph * (yk + yk1)) * jc - (rphm * (ykm + yk)) * jcm);
            const double F = fick_flux(st, rhoD, n, S, p, k, hh);
            s = s + ((0.5 * (cpS[p * S + k] + cpS[(p + 1) * S + k])) / W[k]) * (F + ((0.5 * (yk + yk1)) * jc));
        }
        sumcpj[p] = s;
    }
}

// Temperature cross term dTdtCross (src/flameSolver.cpp:610-612) with the
// grid's centred first-derivative weights (src/grid.cpp:61-65); the U row
// and the boundary points are zero.
__global__ void k_cross_temperature(int64_t n_pts, int n, const int* __restrict__ pt_local,
                                    const int* __restrict__ pt_flame, const int* __restrict__ flame_npts,
                                    const double* __restrict__ x, const double* __restrict__ st,
                                    const double* __restrict__ rho, const double* __restrict__ cp,
                                    const double* __restrict__ sumcpj, double* __restrict__ cross) {
    for (int64_t p = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; p < n_pts; p += int64_t(gridDim.x) * blockDim.x) {
        const int i = pt_local[p];
        const int N = flame_npts[pt_flame[p]];
        cross[p * n] = 0.0;
        double dT = 0.0;
        if (i > 0 && i < N - 1) {
            const double hh = x[p + 1] - x[p], hm = x[p] - x[p - 1];
            const double cfp = hm / (hh * (hh + hm));
            const double cf = (hh - hm) / (hh * hm);
            const double cfm = -hh / (hm * (hh + hm));
            const double dTdx = (cfm * st[(p - 1) * n + 1] + cf * st[p * n + 1]) + cfp * st[(p + 1) * n + 1];
            dT = ((-0.5 * (sumcpj[p] + sumcpj[p - 1])) * dTdx) / (cp[p] * rho[p]);
        }
        cross[p * n + 1] = dT;
    }
}

int grid_for(int64_t n, int threads = 256) {
    return static_cast<int>(std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, 4096)));
}

}  // namespace
}  // namespace ember

using namespace ember;

struct ember_split_s {
    ember_mech mech = nullptr;
    ember_split_options opt{};
    int bdf_layout = 0;  // the BDF matrix layout the source arena was sized for (1 + mode)
    int n_flames = 0, n_vars = 0, nmax = 0;
    int64_t n_pts = 0, n_vals = 0;
    std::vector<ember_diffusion_grid> grids;
    std::vector<DiffSysInfo> info;
    std::vector<int64_t> h_goff;
    // one device allocation for every fixed-size array
    void* blob = nullptr;
    DiffSysInfo* d_info = nullptr;
    double* x = nullptr;
    int64_t* vm_base = nullptr;
    int* npt = nullptr;
    int* flame_npts = nullptr;
    int64_t* flame_goff = nullptr;
    double *state = nullptr, *xD2 = nullptr, *xS = nullptr;
    double *sc_diff = nullptr, *sc_diff_vm = nullptr, *sc_prod = nullptr;
    double *ddt_diff = nullptr, *ddt_prod = nullptr, *ddt_cross = nullptr;
    double *yv = nullptr, *ystart = nullptr, *delta_vm = nullptr;
    double *B = nullptr, *D = nullptr;
    double *dtp = nullptr, *t_dev = nullptr;
    int *diff_status = nullptr, *src_status = nullptr, *src_stats = nullptr, *src_counter = nullptr;
    unsigned long long* fails = nullptr;  // [0] source points, [1] diffusion systems
    double* serial_work = nullptr;
    void* diff_arena = nullptr;
    size_t diff_arena_bytes = 0;
    void* src_arena = nullptr;
    size_t src_arena_bytes = 0;
    DiffusionWarpPlan plan;
    // transport model (ember_split_set_transport_model): properties of the step start
    ember_transport tr = nullptr;
    double tr_threshold = 0.0;
    int tr_cross = 0;
    void* pblob = nullptr;
    double *p_rho = nullptr, *p_cp = nullptr, *p_lam = nullptr, *p_mu = nullptr, *p_rhoD = nullptr, *p_cpS = nullptr;
    // true once a step has run with the transport model attached: p_cp then holds the c_p of the
    // last step's property update, which the consumption speed divides by (as FlameSolver's cp)
    bool props_valid = false;
    double *jcorr = nullptr, *jB = nullptr, *jD = nullptr, *jsc = nullptr, *jh = nullptr, *sumcpj = nullptr;
    double* jwork = nullptr;
    DiffSysInfo* jinfo = nullptr;
    DiffusionWarpPlan jplan;  // jCorr systems (one per flame) with the warp-parallel algorithm
    ember_diffusion_grid* d_grids = nullptr;
    int *jstatus = nullptr, *pt_local = nullptr, *pt_flame = nullptr;
    // convection stage (ember_split_set_convection): D C D S D C D
    bool conv = false;
    ConvPlan cplan;
    void* cblob = nullptr;
    double *ddt_conv = nullptr, *sc_conv = nullptr, *sc_conv_vm = nullptr, *delta_conv_vm = nullptr;
    double *drhodt = nullptr, *y_left = nullptr;
    // the continuity point moved every step: a flag cleared at attach and set_state (the first step
    // keeps the caller's values), and for fixedQdot the start state's heat release rate
    int* conv_ready = nullptr;
    bool conv_qdot = false;
    double *cq_T = nullptr, *cq_Y = nullptr, *cq_net = nullptr, *cq_hk = nullptr, *cq_cp = nullptr,
           *cq_q = nullptr, *cq_qcp = nullptr, *cq_cache = nullptr;
    double* strain_stage = nullptr;  // [n_flames][2 + EMBER_CHEBYSHEV_MAX]: ember_split_set_strain's staging
    cudaStream_t capture_stream = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t graph_exec = nullptr;

    SplitTables tables() const { return SplitTables{n_pts, n_vars, vm_base, npt}; }

    SourceArgs source_args() const {
        // input from the snapshot taken before the stage (the adjoint's last step reads it)
        SourceArgs a = make_source_args(&opt.source, static_cast<int>(n_pts), xD2, sc_prod, dtp, 0.0, x, state,
                                        src_status, src_stats);
        a.t_start_dev = t_dev;
        a.bdf_layout = bdf_layout;
        return a;
    }

    DiffusionView diffusion_view(int* status) const {
        DiffusionView dv{};
        dv.n_systems = static_cast<int>(info.size());
        dv.info = d_info;
        dv.x = x;
        dv.B = B;
        dv.D = D;
        dv.split_const = sc_diff_vm;
        dv.h = nullptr;
        dv.wall_const = nullptr;
        dv.y_inf = nullptr;
        dv.status = status;
        return dv;
    }
};

namespace {

int check_split(ember_split h) {
    EMBER_CHECK_ARG(h != nullptr, "null ember_split handle");
    return EMBER_OK;
}

int copy_to_device(double* dst, const double* src, size_t n, int mem, cudaStream_t st) {
    EMBER_CHECK_ARG(mem == EMBER_MEM_HOST || mem == EMBER_MEM_DEVICE, "bad mem flag %d", mem);
    EMBER_CUDA_TRY(cudaMemcpyAsync(dst, src, n * sizeof(double),
                                   mem == EMBER_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, st));
    return EMBER_OK;
}

// One diffusion stage on the variable-major copy, its change added to deltaDiff.
int enqueue_diffusion_stage(ember_split h, double f0, double f1, cudaStream_t st) {
    const DiffusionView dv = h->diffusion_view(h->diff_status);
    StageTime tm;
    tm.t_dev = h->t_dev;
    tm.f0 = f0;
    tm.f1 = f1;
    tm.dt = h->opt.dt;
    if (h->opt.diffusion_algorithm == EMBER_DIFFUSION_PARALLEL) {
        EMBER_TRY(diffusion_warp_run(h->plan, dv, h->yv, tm, h->opt.dt_multiplier, h->opt.dt, st));
    } else {
        EMBER_TRY(diffusion_serial_run(dv, h->yv, h->serial_work, h->n_vals, h->nmax, tm, h->opt.dt_multiplier,
                                       h->opt.dt, st));
    }
    k_count_failures<<<grid_for(dv.n_systems), 256, 0, st>>>(dv.n_systems, h->diff_status, h->fails + 1);
    k_diff_accumulate<<<grid_for(h->n_vals), 256, 0, st>>>(h->n_vals, h->yv, h->ystart, h->delta_vm);
    return EMBER_OK;
}

// One convection stage (SplitSolver::_integrateConvectionTerms,
// src/splitSolver.cpp:106-121) on the variable-major copy, from t + f0 dt to
// t + f1 dt of the device clock, its change added to deltaConv.
int enqueue_convection_stage(ember_split h, double f0, double f1, cudaStream_t st) {
    ConvArgs a = h->cplan.a;
    a.f0 = f0;
    a.f1 = f1;
    EMBER_TRY(conv_launch(h->cplan, a, st));
    const int ns = h->n_flames * (1 + h->cplan.S);
    k_count_failures<<<grid_for(ns), 256, 0, st>>>(ns, a.status, h->fails + 1);
    k_diff_accumulate<<<grid_for(h->n_vals), 256, 0, st>>>(h->n_vals, h->yv, h->ystart, h->delta_conv_vm);
    return EMBER_OK;
}

// Two diffusion stages back to back on the variable-major copy.
int enqueue_diffusion_pair(ember_split h, double f0, double f1, double f2, cudaStream_t st) {
    const SplitTables tb = h->tables();
    const int g = grid_for(h->n_vals);
    k_to_varmajor<<<g, 256, 0, st>>>(tb, h->state, h->yv, h->ystart);
    const DiffusionView dv = h->diffusion_view(h->diff_status);
    const double fr[3] = {f0, f1, f2};
    for (int k = 0; k < 2; ++k) {
        StageTime tm;
        tm.t_dev = h->t_dev;
        tm.f0 = fr[k];
        tm.f1 = fr[k + 1];
        tm.dt = h->opt.dt;
        if (h->opt.diffusion_algorithm == EMBER_DIFFUSION_PARALLEL) {
            EMBER_TRY(diffusion_warp_run(h->plan, dv, h->yv, tm, h->opt.dt_multiplier, h->opt.dt, st));
        } else {
            EMBER_TRY(diffusion_serial_run(dv, h->yv, h->serial_work, h->n_vals, h->nmax, tm, h->opt.dt_multiplier,
                                           h->opt.dt, st));
        }
        k_count_failures<<<grid_for(dv.n_systems), 256, 0, st>>>(dv.n_systems, h->diff_status, h->fails + 1);
        k_diff_accumulate<<<g, 256, 0, st>>>(h->n_vals, h->yv, h->ystart, h->delta_vm);
    }
    return EMBER_OK;
}

// Start of FlameSolver::step (src/flameSolver.cpp): updateChemicalProperties
// from the current state, prepareIntegrators' B and D and, with cross terms,
// updateCrossTerms into ddt_cross.
int enqueue_properties(ember_split h, cudaStream_t st) {
    const SplitTables tb = h->tables();
    const int n = h->n_vars, S = n - 2;
    ember_properties pr{};
    pr.density = h->p_rho;
    pr.cp_mass = h->p_cp;
    pr.conductivity = h->p_lam;
    pr.viscosity = h->p_mu;
    pr.rho_d = h->p_rhoD;
    pr.cp_species = h->tr_cross ? h->p_cpS : nullptr;
    EMBER_TRY(launch_transport(h->mech->view, h->tr->view, static_cast<int>(h->n_pts), h->opt.source.pressure,
                               h->tr_threshold, h->state + 1, n, h->state + 2, n, pr, st));
    k_bd_from_props<<<grid_for(h->n_vals), 256, 0, st>>>(tb, S, h->p_rho, h->p_cp, h->p_lam, h->p_mu, h->p_rhoD,
                                                          h->B, h->D);
    if (!h->tr_cross) return EMBER_OK;
    const int gp = grid_for(h->n_pts);
    k_jcorr_fick<<<gp, 256, 0, st>>>(h->n_pts, n, S, h->pt_local, h->pt_flame, h->flame_npts, h->x, h->state,
                                      h->p_rhoD, h->p_lam, h->p_rho, h->p_cp, h->jcorr, h->jB);
    k_jcorr_h<<<blocks_for(int64_t(h->n_flames) * 32, 128), 128, 0, st>>>(h->n_flames, h->flame_goff, h->flame_npts,
                                                                          h->x, h->jB, h->opt.dt_multiplier, h->opt.dt,
                                                                          h->jh);
    DiffusionView jv{};
    jv.n_systems = h->n_flames;
    jv.info = h->jinfo;
    jv.x = h->x;
    jv.B = h->jB;
    jv.D = h->jD;
    jv.split_const = h->jsc;
    jv.h = h->jh;
    jv.status = h->jstatus;
    StageTime tm;
    tm.t0 = 0.0;
    tm.t1 = h->opt.dt;
    if (h->opt.diffusion_algorithm == EMBER_DIFFUSION_SERIAL) {
        EMBER_TRY(diffusion_serial_run(jv, h->jcorr, h->jwork, h->n_pts, h->nmax, tm, h->opt.dt_multiplier, h->opt.dt,
                                       st));
    } else {
        EMBER_TRY(diffusion_warp_run(h->jplan, jv, h->jcorr, tm, h->opt.dt_multiplier, h->opt.dt, st));
    }
    k_count_failures<<<blocks_for(h->n_flames, 256), 256, 0, st>>>(h->n_flames, h->jstatus, h->fails + 1);
    k_cross_species<<<gp, 256, 0, st>>>(h->n_pts, n, S, h->pt_local, h->pt_flame, h->flame_npts, h->d_grids, h->x,
                                         h->state, h->p_rhoD, h->p_cpS, h->mech->view.W, h->p_rho, h->jcorr,
                                         h->sumcpj, h->ddt_cross);
    k_cross_temperature<<<gp, 256, 0, st>>>(h->n_pts, n, h->pt_local, h->pt_flame, h->flame_npts, h->x, h->state,
                                             h->p_rho, h->p_cp, h->sumcpj, h->ddt_cross);
    EMBER_CUDA_TRY(cudaGetLastError());
    return EMBER_OK;
}

// One split step, enqueued on `st` (kernel launches and device copies only).
// What a taped step (the forward pass of ember_split_adjoint) keeps.
struct StepTape {
    double* t_saved;  // device clock at the start of the step
    double* buf;      // BDF tape of the source stage
    int64_t stride;
    int cap;
    double* xF;       // state before the mass-fraction correction
};

int enqueue_step(ember_split h, cudaStream_t st, const StepTape* tape = nullptr) {
    const SplitTables tb = h->tables();
    const int g = grid_for(h->n_vals);
    if (tape) EMBER_CUDA_TRY(cudaMemcpyAsync(tape->t_saved, h->t_dev, sizeof(double), cudaMemcpyDeviceToDevice, st));
    if (h->tr) EMBER_TRY(enqueue_properties(h, st));
    if (h->conv) {
        k_density_derivative<<<grid_for(h->n_pts), 256, 0, st>>>(h->n_pts, h->n_vars, h->opt.balanced,
                                                                 h->opt.source.pressure, h->mech->view.W, h->state,
                                                                 h->ddt_conv, h->ddt_diff, h->ddt_prod, h->ddt_cross,
                                                                 h->drhodt);
        // updateContinuityBoundaryCondition (prepareIntegrators, src/flameSolver.cpp:215), with the start
        // state's qdot for fixedQdot (calculateQdot after the previous step)
        if (h->conv_qdot) {
            const int S = h->n_vars - 2;
            k_gather_TY<<<grid_for(h->n_pts * S), 256, 0, st>>>(h->n_pts, h->n_vars, h->state, h->cq_T, h->cq_Y);
            EMBER_TRY(launch_gas_eval(h->mech->view, static_cast<int>(h->n_pts), h->opt.source.pressure,
                                      h->opt.source.kinetics_model, EMBER_STATE_NORMALIZED, h->cq_T, h->cq_Y,
                                      h->cq_cache, h->cq_net, h->cq_hk, h->cq_cp, st));
            k_qdot<<<grid_for(h->n_pts, 128), 128, 0, st>>>(h->n_pts, S, h->cq_net, h->cq_hk, h->cq_cp, h->cq_q,
                                                            h->cq_qcp);
        }
        EMBER_TRY(conv_continuity_launch(h->cplan, h->cplan.a, h->conv_ready, h->state, h->n_vars,
                                         h->conv_qdot ? h->cq_q : nullptr, st));
    }
    k_split_begin<<<g, 256, 0, st>>>(tb, h->opt.balanced, h->ddt_diff, h->ddt_prod, h->ddt_cross, h->sc_diff,
                                     h->sc_diff_vm, h->sc_prod, h->delta_vm, h->conv ? h->ddt_conv : nullptr,
                                     h->sc_conv, h->sc_conv_vm, h->delta_conv_vm);
    if (h->conv) {
        // diffusion 1/4, convection 1/2, diffusion 2/4 (src/splitSolver.cpp:68-70)
        k_to_varmajor<<<g, 256, 0, st>>>(tb, h->state, h->yv, h->ystart);
        EMBER_TRY(enqueue_diffusion_stage(h, 0.0, 0.25, st));
        EMBER_TRY(enqueue_convection_stage(h, 0.0, 0.5, st));
        EMBER_TRY(enqueue_diffusion_stage(h, 0.25, 0.5, st));
    } else {
        // diffusion 1/4 and 2/4
        EMBER_TRY(enqueue_diffusion_pair(h, 0.0, 0.25, 0.5, st));
    }
    k_to_pointmajor<<<g, 256, 0, st>>>(tb, h->yv, h->state, h->xD2);
    // source term over the whole step
    k_stage_dt<<<grid_for(h->n_pts), 256, 0, st>>>(h->n_pts, h->t_dev, h->opt.dt, h->dtp);
    {
        Scratch sc(st, h->src_arena, h->src_arena_bytes);
        EMBER_CUDA_TRY(cudaMemsetAsync(h->src_counter, 0, sizeof(int), st));
        SourceArgs a = h->source_args();
        if (tape) {
            a.tape = tape->buf;
            a.tape_stride = tape->stride;
            a.tape_cap = tape->cap;
        }
        if (h->opt.method == EMBER_SOURCE_QSS) {
            EMBER_TRY(launch_source_qss(h->mech->view, a, h->src_counter, sc, st));
        } else {
            EMBER_TRY(launch_source_bdf(h->mech->view, a, h->src_counter, sc, st));
        }
    }
    k_count_failures<<<grid_for(h->n_pts), 256, 0, st>>>(static_cast<int>(h->n_pts), h->src_status, h->fails);
    EMBER_CUDA_TRY(cudaMemcpyAsync(h->xS, h->state, sizeof(double) * h->n_vals, cudaMemcpyDeviceToDevice, st));
    if (h->conv) {
        // diffusion 3/4, convection 2/2, diffusion 4/4 (src/splitSolver.cpp:72-74)
        k_to_varmajor<<<g, 256, 0, st>>>(tb, h->state, h->yv, h->ystart);
        EMBER_TRY(enqueue_diffusion_stage(h, 0.5, 0.75, st));
        EMBER_TRY(enqueue_convection_stage(h, 0.5, 1.0, st));
        EMBER_TRY(enqueue_diffusion_stage(h, 0.75, 1.0, st));
    } else {
        // diffusion 3/4 and 4/4
        EMBER_TRY(enqueue_diffusion_pair(h, 0.5, 0.75, 1.0, st));
    }
    k_to_pointmajor<<<g, 256, 0, st>>>(tb, h->yv, h->state, nullptr);
    k_split_end<<<g, 256, 0, st>>>(tb, h->opt.dt, h->xS, h->xD2, h->delta_vm, h->sc_diff, h->sc_prod, h->ddt_diff,
                                   h->ddt_prod, h->delta_conv_vm, h->sc_conv, h->conv ? h->ddt_conv : nullptr);
    if (tape) EMBER_CUDA_TRY(cudaMemcpyAsync(tape->xF, h->state, sizeof(double) * h->n_vals, cudaMemcpyDeviceToDevice, st));
    k_correct_mass_fractions<<<grid_for(h->n_pts, 128), 128, 0, st>>>(h->n_pts, h->n_vars, h->state);
    k_advance_clock<<<1, 32, 0, st>>>(h->t_dev, h->opt.dt);
    EMBER_CUDA_TRY(cudaGetLastError());
    return EMBER_OK;
}

void free_split(ember_split h) {
    if (!h) return;
    if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
    if (h->graph) cudaGraphDestroy(h->graph);
    if (h->capture_stream) cudaStreamDestroy(h->capture_stream);
    cudaFree(h->blob);
    cudaFree(h->pblob);
    cudaFree(h->cblob);
    delete h;
}

}  // namespace

extern "C" int ember_split_create(ember_mech mech, int n_flames, const ember_diffusion_grid* grids, const double* x,
                                  const ember_split_options* opts, ember_split* out) {
    EMBER_CHECK_ARG(out != nullptr, "null output handle pointer");
    *out = nullptr;
    EMBER_CHECK_ARG(mech != nullptr, "null mechanism");
    EMBER_CHECK_ARG(n_flames > 0 && grids != nullptr && x != nullptr, "need at least one flame and its grid");
    EMBER_CHECK_ARG(opts != nullptr, "null options");
    EMBER_CHECK_ARG(opts->method == EMBER_SOURCE_QSS || opts->method == EMBER_SOURCE_BDF, "bad method %d",
                    opts->method);
    EMBER_CHECK_ARG(opts->diffusion_algorithm == EMBER_DIFFUSION_PARALLEL ||
                        opts->diffusion_algorithm == EMBER_DIFFUSION_SERIAL,
                    "bad diffusion algorithm %d", opts->diffusion_algorithm);
    EMBER_CHECK_ARG(opts->dt > 0 && opts->dt_multiplier > 0, "dt and dt_multiplier must be positive");
    EMBER_TRY(source_check_options(&opts->source));
    const int n_vars = mech->S + 2;

    // System table (flame-major, then variable) and the transpose tables.
    std::vector<DiffSysInfo> info;
    std::vector<int64_t> vm_base, goff(n_flames);
    std::vector<int> npt, fnpts(n_flames);
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
            DiffSysInfo s{};
            s.off = n_vals + int64_t(v) * g.n_points;
            s.grid_off = n_pts;
            s.n = g.n_points;
            s.left_bc = g.left_bc;
            s.right_bc = g.right_bc;
            s.alpha = g.alpha;
            info.push_back(s);
        }
        for (int i = 0; i < g.n_points; ++i) {
            vm_base.push_back(n_vals + i);
            npt.push_back(g.n_points);
        }
        goff[f] = n_pts;
        fnpts[f] = g.n_points;
        n_pts += g.n_points;
        n_vals += int64_t(n_vars) * g.n_points;
        nmax = std::max(nmax, g.n_points);
    }
    EMBER_CHECK_ARG(n_pts < (int64_t(1) << 31) && info.size() < (size_t(1) << 31), "batch too large");
    EMBER_TRY(ensure_device());

    // Sizes of everything the step touches, one allocation.
    const int n_sys = static_cast<int>(info.size());
    const bool serial = opts->diffusion_algorithm == EMBER_DIFFUSION_SERIAL;
    const size_t plan_bytes = serial ? 0 : diffusion_warp_plan_bytes(info, n_pts);
    SourceArgs probe = make_source_args(&opts->source, static_cast<int>(n_pts), nullptr, nullptr, nullptr, 0.0,
                                        nullptr, nullptr, nullptr, nullptr);
    size_t src_bytes = 0;
    if (opts->method == EMBER_SOURCE_QSS) {
        EMBER_TRY(source_qss_scratch_bytes(mech->view, probe, &src_bytes));
    } else {
        EMBER_TRY(source_bdf_scratch_bytes(mech->view, probe, &src_bytes));
    }
    const size_t R = Scratch::rounded(1);
    auto bd = [&](size_t n) { return Scratch::rounded(n * sizeof(double)); };
    const size_t total = Scratch::rounded(sizeof(DiffSysInfo) * n_sys) + bd(n_pts) +
                         Scratch::rounded(sizeof(int64_t) * n_pts) + Scratch::rounded(sizeof(int) * n_pts) +
                         Scratch::rounded(sizeof(int) * n_flames) + Scratch::rounded(sizeof(int64_t) * n_flames) +
                         14 * bd(n_vals) + bd(n_pts) + bd(1) + Scratch::rounded(sizeof(int) * n_sys) +
                         Scratch::rounded(sizeof(int) * n_pts) + Scratch::rounded(sizeof(int) * 4 * n_pts) + R +
                         Scratch::rounded(2 * sizeof(unsigned long long)) + (serial ? bd(7 * n_vals) : 0) +
                         plan_bytes + src_bytes;

    auto* h = new ember_split_s;
    h->mech = mech;
    h->opt = *opts;
    // the handle keeps the QSS width its scratch arena was sized for, even if
    // the mechanism is tuned again later
    if (opts->method == EMBER_SOURCE_QSS) {
        h->opt.source.threads_per_point = source_qss_threads(mech->view, probe);
        int tail_steps = 0, tail_threads = 0;
        source_qss_tail(mech->view, probe, &tail_steps, &tail_threads);
        h->opt.source.qss_tail_steps = tail_steps ? tail_steps : -1;
        h->opt.source.qss_tail_threads = tail_steps ? tail_threads : 0;
    } else {
        h->opt.source.threads_per_point = source_bdf_threads(mech->view, probe);
        h->bdf_layout = source_bdf_layout(mech->view, probe);
    }
    h->n_flames = n_flames;
    h->n_vars = n_vars;
    h->nmax = nmax;
    h->n_pts = n_pts;
    h->n_vals = n_vals;
    h->grids.assign(grids, grids + n_flames);
    h->info = info;
    h->h_goff = goff;
    cudaError_t e = cudaMalloc(&h->blob, total);
    if (e == cudaSuccess) e = cudaMemset(h->blob, 0, total);  // before anything is uploaded into it
    if (e != cudaSuccess) {
        set_error("ember_split_create: cudaMalloc(%zu bytes) failed: %s", total, cudaGetErrorString(e));
        free_split(h);
        return e == cudaErrorMemoryAllocation ? EMBER_ENOMEM : EMBER_ECUDA;
    }
    int rc = EMBER_OK;
    {
        Scratch a(nullptr, h->blob, total);
        auto carve = [&](auto** p, size_t n) {
            if (rc == EMBER_OK) rc = a.alloc(p, n);
        };
        carve(&h->d_info, n_sys);
        carve(&h->x, n_pts);
        carve(&h->vm_base, n_pts);
        carve(&h->npt, n_pts);
        carve(&h->flame_npts, n_flames);
        carve(&h->flame_goff, n_flames);
        double** big[14] = {&h->state, &h->xD2,      &h->xS,       &h->sc_diff, &h->sc_diff_vm,
                            &h->sc_prod, &h->ddt_diff, &h->ddt_prod, &h->ddt_cross, &h->yv,
                            &h->ystart,  &h->delta_vm, &h->B,        &h->D};
        for (double** q : big) carve(q, n_vals);
        carve(&h->dtp, n_pts);
        carve(&h->t_dev, 1);
        carve(&h->diff_status, n_sys);
        carve(&h->src_status, n_pts);
        carve(&h->src_stats, 4 * n_pts);
        carve(&h->src_counter, 1);
        carve(&h->fails, 2);
        if (serial) carve(&h->serial_work, 7 * n_vals);
        if (rc == EMBER_OK && !serial) {
            rc = diffusion_warp_plan_init(&h->plan, info, n_flames, n_vars, n_pts, a, nullptr);
        }
        if (rc == EMBER_OK) rc = a.alloc(reinterpret_cast<char**>(&h->src_arena), src_bytes);
        h->src_arena_bytes = src_bytes;
    }
    if (rc != EMBER_OK) {
        free_split(h);
        return rc;
    }
    e = cudaMemcpy(h->d_info, info.data(), sizeof(DiffSysInfo) * n_sys, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->x, x, sizeof(double) * n_pts, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->vm_base, vm_base.data(), sizeof(int64_t) * n_pts, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->npt, npt.data(), sizeof(int) * n_pts, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->flame_npts, fnpts.data(), sizeof(int) * n_flames, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->flame_goff, goff.data(), sizeof(int64_t) * n_flames, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->capture_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        set_error("ember_split_create: %s", cudaGetErrorString(e));
        free_split(h);
        return EMBER_ECUDA;
    }
    if (!serial) {
        // the plan's tables were queued on the legacy stream; wait for them
        rc = diffusion_warp_geometry(h->plan, h->d_info, h->x, nullptr);
        if (rc == EMBER_OK && cudaDeviceSynchronize() != cudaSuccess) {
            set_error("ember_split_create: %s", cudaGetErrorString(cudaGetLastError()));
            rc = EMBER_ECUDA;
        }
        if (rc != EMBER_OK) {
            free_split(h);
            return rc;
        }
    }
    *out = h;
    return EMBER_OK;
}

extern "C" int ember_split_destroy(ember_split h) {
    free_split(h);
    return EMBER_OK;
}

extern "C" int ember_split_set_state(ember_split h, double t, const double* state, int mem, void* stream) {
    EMBER_TRY(check_split(h));
    EMBER_CHECK_ARG(state != nullptr, "null state");
    cudaStream_t st = as_stream(stream);
    EMBER_TRY(copy_to_device(h->state, state, size_t(h->n_vals), mem, st));
    EMBER_CUDA_TRY(cudaMemcpyAsync(h->t_dev, &t, sizeof(double), cudaMemcpyHostToDevice, st));
    EMBER_CUDA_TRY(cudaMemsetAsync(h->ddt_diff, 0, sizeof(double) * h->n_vals, st));
    EMBER_CUDA_TRY(cudaMemsetAsync(h->ddt_prod, 0, sizeof(double) * h->n_vals, st));
    if (h->conv) {
        EMBER_CUDA_TRY(cudaMemsetAsync(h->ddt_conv, 0, sizeof(double) * h->n_vals, st));
        EMBER_CUDA_TRY(cudaMemsetAsync(h->conv_ready, 0, sizeof(int), st));
    }
    EMBER_CUDA_TRY(cudaMemsetAsync(h->fails, 0, 2 * sizeof(unsigned long long), st));
    h->props_valid = false;
    // the host value of t must outlive the copy
    EMBER_CUDA_TRY(cudaStreamSynchronize(st));
    return EMBER_OK;
}

extern "C" int ember_split_load_state(ember_split h, const double* state, int mem, void* stream) {
    EMBER_TRY(check_split(h));
    EMBER_CHECK_ARG(state != nullptr, "null state");
    cudaStream_t st = as_stream(stream);
    EMBER_TRY(copy_to_device(h->state, state, size_t(h->n_vals), mem, st));
    return finish_call(mem, st);
}

extern "C" int ember_split_set_transport(ember_split h, const double* B, const double* D, const double* ddt_cross,
                                         int mem, void* stream) {
    EMBER_TRY(check_split(h));
    EMBER_CHECK_ARG(B != nullptr && D != nullptr, "null B or D");
    cudaStream_t st = as_stream(stream);
    EMBER_TRY(copy_to_device(h->B, B, size_t(h->n_vals), mem, st));
    EMBER_TRY(copy_to_device(h->D, D, size_t(h->n_vals), mem, st));
    if (ddt_cross) {
        EMBER_TRY(copy_to_device(h->ddt_cross, ddt_cross, size_t(h->n_vals), mem, st));
    } else {
        EMBER_CUDA_TRY(cudaMemsetAsync(h->ddt_cross, 0, sizeof(double) * h->n_vals, st));
    }
    return finish_call(mem, st);
}

extern "C" int ember_split_set_convection(ember_split h, const ember_convection_flame* flames,
                                         const double* y_left, const ember_convection_options* opts) {
    EMBER_TRY(check_split(h));
    EMBER_TRY(ensure_device());
    // the captured graph (if any) has the old stage list
    if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
    if (h->graph) cudaGraphDestroy(h->graph);
    h->graph_exec = nullptr;
    h->graph = nullptr;
    EMBER_CUDA_TRY(cudaDeviceSynchronize());
    cudaFree(h->cblob);
    h->cblob = nullptr;
    h->conv = false;
    if (!flames) return EMBER_OK;
    EMBER_CHECK_ARG(y_left != nullptr && opts != nullptr, "null y_left or options");
    const int S = h->n_vars - 2;
    for (int f = 0; f < h->n_flames; ++f) {
        EMBER_CHECK_ARG(flames[f].n_points == h->grids[f].n_points, "flame %d: n_points %d differs from the grid's %d",
                        f, flames[f].n_points, h->grids[f].n_points);
        EMBER_CHECK_ARG(flames[f].alpha == h->grids[f].alpha, "flame %d: alpha differs from the grid's", f);
        // one gas pressure for the whole step, as the reference's single CanteraGas: the density
        // derivative and the transport model use the source options' pressure
        EMBER_CHECK_ARG(flames[f].pressure == h->opt.source.pressure,
                        "flame %d: pressure %g differs from the split options' %g", f, flames[f].pressure,
                        h->opt.source.pressure);
    }
    ConvPlan p;
    EMBER_TRY(conv_plan_layout(p, h->n_flames, flames, S, opts));
    const size_t nv = size_t(h->n_vals);
    bool any_qdot = false;
    for (int f = 0; f < h->n_flames; ++f) any_qdot = any_qdot || flames[f].continuity_bc == EMBER_CONTINUITY_QDOT;
    const size_t np = size_t(h->n_pts);
    const size_t cache = gas_eval_cache_doubles(h->mech->view, static_cast<int>(h->n_pts));
    // fixedQdot: T, cp, qdot, qdot/cp per point; Y, net rates, hk per point and species; the rate cache
    const size_t qdot_bytes = any_qdot ? 3 * Scratch::rounded(np * S * sizeof(double)) +
                                             4 * Scratch::rounded(np * sizeof(double)) +
                                             Scratch::rounded(cache * sizeof(double))
                                       : 0;
    const size_t bytes = conv_plan_bytes(p, false) + 4 * Scratch::rounded(nv * sizeof(double)) +
                         Scratch::rounded(size_t(h->n_pts) * sizeof(double)) +
                         Scratch::rounded(size_t(h->n_flames) * S * sizeof(double)) + Scratch::rounded(sizeof(int)) +
                         qdot_bytes + Scratch::rounded(size_t(h->n_flames) * (2 + EMBER_CHEBYSHEV_MAX) * sizeof(double));
    cudaError_t e = cudaMalloc(&h->cblob, bytes);
    if (e != cudaSuccess) {
        h->cblob = nullptr;
        set_error("ember_split_set_convection: cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? EMBER_ENOMEM : EMBER_ECUDA;
    }
    Scratch a(nullptr, h->cblob, bytes);
    EMBER_TRY(a.alloc(&h->ddt_conv, nv));
    EMBER_TRY(a.alloc(&h->sc_conv, nv));
    EMBER_TRY(a.alloc(&h->sc_conv_vm, nv));
    EMBER_TRY(a.alloc(&h->delta_conv_vm, nv));
    EMBER_TRY(a.alloc(&h->drhodt, size_t(h->n_pts)));
    EMBER_TRY(a.alloc(&h->y_left, size_t(h->n_flames) * S));
    EMBER_TRY(a.alloc(&h->conv_ready, 1));
    EMBER_TRY(a.alloc(&h->strain_stage, size_t(h->n_flames) * (2 + EMBER_CHEBYSHEV_MAX)));
    h->conv_qdot = any_qdot;
    if (any_qdot) {
        EMBER_TRY(a.alloc(&h->cq_T, np));
        EMBER_TRY(a.alloc(&h->cq_Y, np * S));
        EMBER_TRY(a.alloc(&h->cq_net, np * S));
        EMBER_TRY(a.alloc(&h->cq_hk, np * S));
        EMBER_TRY(a.alloc(&h->cq_cp, np));
        EMBER_TRY(a.alloc(&h->cq_q, np));
        EMBER_TRY(a.alloc(&h->cq_qcp, np));
        EMBER_TRY(a.alloc(&h->cq_cache, cache));
    }
    EMBER_CUDA_TRY(cudaMemset(h->conv_ready, 0, sizeof(int)));
    EMBER_TRY(conv_plan_alloc(p, a, false, nullptr));
    EMBER_CUDA_TRY(cudaMemcpy(h->y_left, y_left, sizeof(double) * h->n_flames * S, cudaMemcpyHostToDevice));
    EMBER_CUDA_TRY(cudaMemset(h->ddt_conv, 0, sizeof(double) * nv));
    EMBER_CUDA_TRY(cudaDeviceSynchronize());
    ConvArgs& c = p.a;
    c.W = h->mech->view.W;
    c.x = h->x;
    c.y_left = h->y_left;
    c.drhodt = h->drhodt;
    c.split = h->sc_conv_vm;
    c.state = h->yv;
    c.t_dev = h->t_dev;
    c.dt = h->opt.dt;
    h->cplan = std::move(p);
    h->conv = true;
    return EMBER_OK;
}


namespace ember {
namespace {
// The strain function of every flame becomes the Chebyshev series staged in
// stage[f][0..1] (t0, t1) and stage[f][2..2+n) (coefficients).
__global__ void k_set_strain(ConvFlame* flames, int n_flames, int n, const double* __restrict__ stage) {
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= n_flames) return;
    ember_convection_flame& fl = flames[f].f;
    const double* c = stage + size_t(f) * (2 + EMBER_CHEBYSHEV_MAX);
    fl.strain_type = EMBER_STRAIN_CHEBYSHEV;
    fl.n_cheb = n;
    fl.cheb_t0 = c[0];
    fl.cheb_t1 = c[1];
    for (int i = 0; i < EMBER_CHEBYSHEV_MAX; ++i) fl.cheb[i] = i < n ? c[2 + i] : 0.0;
}
}  // namespace
}  // namespace ember

extern "C" int ember_split_set_strain(ember_split h, int n_coeffs, const double* coeffs, void* stream) {
    EMBER_TRY(check_split(h));
    EMBER_CHECK_ARG(h->conv, "no convection stage attached (ember_split_set_convection)");
    EMBER_CHECK_ARG(n_coeffs >= 0 && n_coeffs <= EMBER_CHEBYSHEV_MAX, "n_coeffs must be 0..%d", EMBER_CHEBYSHEV_MAX);
    EMBER_CHECK_ARG(coeffs != nullptr, "null coefficients");
    const int w = 2 + n_coeffs, ws = 2 + EMBER_CHEBYSHEV_MAX;
    std::vector<double> stage(size_t(h->n_flames) * ws, 0.0);
    for (int f = 0; f < h->n_flames; ++f) {
        const double* c = coeffs + size_t(f) * w;
        EMBER_CHECK_ARG(c[1] != c[0], "flame %d: t1 equals t0", f);
        for (int i = 0; i < w; ++i) stage[size_t(f) * ws + i] = c[i];
    }
    cudaStream_t st = as_stream(stream);
    EMBER_CUDA_TRY(cudaMemcpyAsync(h->strain_stage, stage.data(), sizeof(double) * stage.size(),
                                   cudaMemcpyHostToDevice, st));
    k_set_strain<<<blocks_for(h->n_flames, 64), 64, 0, st>>>(const_cast<ConvFlame*>(h->cplan.a.flames), h->n_flames,
                                                             n_coeffs, h->strain_stage);
    EMBER_CUDA_TRY(cudaGetLastError());
    // the staging vector is a host buffer: the copy must be done before it goes away
    EMBER_CUDA_TRY(cudaStreamSynchronize(st));
    return EMBER_OK;
}

extern "C" int ember_split_set_transport_model(ember_split h, ember_transport tr, double threshold,
                                               int cross_terms) {
    EMBER_TRY(check_split(h));
    EMBER_CHECK_ARG(!tr || tr->mech == h->mech, "the transport model belongs to another mechanism");
    EMBER_CHECK_ARG(threshold >= 0 && threshold < 1, "threshold must be in [0, 1)");
    EMBER_TRY(ensure_device());
    // the captured graph (if any) has the old stage list
    if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
    if (h->graph) cudaGraphDestroy(h->graph);
    h->graph_exec = nullptr;
    h->graph = nullptr;
    EMBER_CUDA_TRY(cudaDeviceSynchronize());
    cudaFree(h->pblob);
    h->pblob = nullptr;
    h->tr = nullptr;
    h->props_valid = false;
    if (!tr) return EMBER_OK;
    const int64_t np = h->n_pts;
    const int S = h->n_vars - 2, nf = h->n_flames;
    std::vector<DiffSysInfo> ji(nf);
    std::vector<int> loc(np), fl(np);
    for (int f = 0; f < nf; ++f) {
        const ember_diffusion_grid& g = h->grids[f];
        ji[f].off = h->h_goff[f];
        ji[f].grid_off = h->h_goff[f];
        ji[f].n = g.n_points;
        ji[f].left_bc = g.left_bc;
        ji[f].right_bc = g.right_bc;
        ji[f].alpha = g.alpha;
        for (int i = 0; i < g.n_points; ++i) {
            loc[h->h_goff[f] + i] = i;
            fl[h->h_goff[f] + i] = f;
        }
    }
    const bool serial = h->opt.diffusion_algorithm == EMBER_DIFFUSION_SERIAL;
    auto bd = [](size_t c) { return Scratch::rounded(c * sizeof(double)); };
    const size_t total = 4 * bd(np) + 2 * bd(size_t(np) * S) + 6 * bd(np) + (serial ? bd(7 * size_t(np)) : 0) +
                         (serial ? 0 : diffusion_warp_plan_bytes(ji, np)) + Scratch::rounded(sizeof(DiffSysInfo) * nf) +
                         Scratch::rounded(sizeof(ember_diffusion_grid) * nf) + Scratch::rounded(sizeof(int) * nf) +
                         2 * Scratch::rounded(sizeof(int) * np);
    EMBER_CUDA_TRY(cudaMalloc(&h->pblob, total));
    int rc = EMBER_OK;
    {
        Scratch a(nullptr, h->pblob, total);
        auto carve = [&](auto** p, size_t c) {
            if (rc == EMBER_OK) rc = a.alloc(p, c);
        };
        carve(&h->p_rho, np);
        carve(&h->p_cp, np);
        carve(&h->p_lam, np);
        carve(&h->p_mu, np);
        carve(&h->p_rhoD, size_t(np) * S);
        carve(&h->p_cpS, size_t(np) * S);
        carve(&h->jcorr, np);
        carve(&h->jB, np);
        carve(&h->jD, np);
        carve(&h->jsc, np);
        carve(&h->jh, np);
        carve(&h->sumcpj, np);
        if (serial) carve(&h->jwork, 7 * size_t(np));
        carve(&h->jinfo, nf);
        carve(&h->d_grids, nf);
        carve(&h->jstatus, nf);
        carve(&h->pt_local, np);
        carve(&h->pt_flame, np);
        if (rc == EMBER_OK && !serial) rc = diffusion_warp_plan_init(&h->jplan, ji, nf, 1, np, a, nullptr);
    }
    if (rc != EMBER_OK) return rc;
    std::vector<double> ones(np, 1.0);
    cudaError_t e = cudaMemcpy(h->jinfo, ji.data(), sizeof(DiffSysInfo) * nf, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->d_grids, h->grids.data(), sizeof(ember_diffusion_grid) * nf,
                                         cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->pt_local, loc.data(), sizeof(int) * np, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->pt_flame, fl.data(), sizeof(int) * np, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->jD, ones.data(), sizeof(double) * np, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(h->jsc, 0, sizeof(double) * np);
    if (e == cudaSuccess && !serial) {
        rc = diffusion_warp_geometry(h->jplan, h->jinfo, h->x, nullptr);
        if (rc != EMBER_OK) return rc;
        e = cudaDeviceSynchronize();
    }
    if (e != cudaSuccess) {
        set_error("ember_split_set_transport_model: %s", cudaGetErrorString(e));
        return EMBER_ECUDA;
    }
    h->tr = tr;
    h->tr_threshold = threshold;
    h->tr_cross = cross_terms != 0;
    return EMBER_OK;
}

extern "C" int ember_split_step(ember_split h, int n_steps, int use_graph, void* stream) {
    EMBER_TRY(check_split(h));
    EMBER_CHECK_ARG(n_steps >= 0, "n_steps must be >= 0");
    cudaStream_t st = as_stream(stream);
    if (h->tr && n_steps > 0) h->props_valid = true;
    if (!use_graph) {
        for (int k = 0; k < n_steps; ++k) EMBER_TRY(enqueue_step(h, st));
        return EMBER_OK;
    }
    if (!h->graph_exec) {
        EMBER_CUDA_TRY(cudaStreamBeginCapture(h->capture_stream, cudaStreamCaptureModeRelaxed));
        const int rc = enqueue_step(h, h->capture_stream);
        cudaGraph_t g = nullptr;
        const cudaError_t e = cudaStreamEndCapture(h->capture_stream, &g);
        if (rc != EMBER_OK) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        EMBER_CUDA_TRY(e);
        h->graph = g;
        EMBER_CUDA_TRY(cudaGraphInstantiate(&h->graph_exec, h->graph, 0));
    }
    for (int k = 0; k < n_steps; ++k) EMBER_CUDA_TRY(cudaGraphLaunch(h->graph_exec, st));
    return EMBER_OK;
}

extern "C" int ember_split_get_state(ember_split h, double* state, double* t, int mem, void* stream) {
    EMBER_TRY(check_split(h));
    EMBER_CHECK_ARG(mem == EMBER_MEM_HOST || mem == EMBER_MEM_DEVICE, "bad mem flag %d", mem);
    cudaStream_t st = as_stream(stream);
    const cudaMemcpyKind kind = mem == EMBER_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (state) EMBER_CUDA_TRY(cudaMemcpyAsync(state, h->state, sizeof(double) * h->n_vals, kind, st));
    if (t) EMBER_CUDA_TRY(cudaMemcpyAsync(t, h->t_dev, sizeof(double), kind, st));
    return finish_call(mem, st);
}

extern "C" int ember_split_get_derivatives(ember_split h, double* ddt_diff, double* ddt_prod, int mem, void* stream) {
    EMBER_TRY(check_split(h));
    EMBER_CHECK_ARG(mem == EMBER_MEM_HOST || mem == EMBER_MEM_DEVICE, "bad mem flag %d", mem);
    cudaStream_t st = as_stream(stream);
    const cudaMemcpyKind kind = mem == EMBER_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (ddt_diff) EMBER_CUDA_TRY(cudaMemcpyAsync(ddt_diff, h->ddt_diff, sizeof(double) * h->n_vals, kind, st));
    if (ddt_prod) EMBER_CUDA_TRY(cudaMemcpyAsync(ddt_prod, h->ddt_prod, sizeof(double) * h->n_vals, kind, st));
    return finish_call(mem, st);
}

extern "C" int ember_split_get_convection_derivative(ember_split h, double* ddt_conv, int mem, void* stream) {
    EMBER_TRY(check_split(h));
    EMBER_CHECK_ARG(mem == EMBER_MEM_HOST || mem == EMBER_MEM_DEVICE, "bad mem flag %d", mem);
    EMBER_CHECK_ARG(h->conv, "no convection stage attached");
    EMBER_CHECK_ARG(ddt_conv != nullptr, "null ddt_conv");
    cudaStream_t st = as_stream(stream);
    const cudaMemcpyKind kind = mem == EMBER_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    EMBER_CUDA_TRY(cudaMemcpyAsync(ddt_conv, h->ddt_conv, sizeof(double) * h->n_vals, kind, st));
    return finish_call(mem, st);
}

extern "C" int ember_split_get_velocity(ember_split h, double* V, int mem, void* stream) {
    EMBER_TRY(check_split(h));
    EMBER_CHECK_ARG(mem == EMBER_MEM_HOST || mem == EMBER_MEM_DEVICE, "bad mem flag %d", mem);
    EMBER_CHECK_ARG(h->conv, "no convection stage attached");
    EMBER_CHECK_ARG(V != nullptr, "null V");
    cudaStream_t st = as_stream(stream);
    Scratch sc(st);
    double* dv = V;
    if (mem == EMBER_MEM_HOST) EMBER_TRY(sc.alloc(&dv, size_t(h->n_pts)));
    EMBER_TRY(conv_velocity_launch(h->cplan, h->cplan.a, dv, st));
    if (mem == EMBER_MEM_HOST)
        EMBER_CUDA_TRY(cudaMemcpyAsync(V, dv, sizeof(double) * h->n_pts, cudaMemcpyDeviceToHost, st));
    sc.release();
    return finish_call(mem, st);
}

extern "C" int ember_split_set_derivatives(ember_split h, const double* ddt_diff, const double* ddt_prod,
                                           const double* ddt_conv, int mem, void* stream) {
    EMBER_TRY(check_split(h));
    EMBER_CHECK_ARG(ddt_diff && ddt_prod, "null ddt_diff or ddt_prod");
    EMBER_CHECK_ARG(!ddt_conv || h->conv, "ddt_conv given but no convection stage is attached");
    cudaStream_t st = as_stream(stream);
    EMBER_TRY(copy_to_device(h->ddt_diff, ddt_diff, size_t(h->n_vals), mem, st));
    EMBER_TRY(copy_to_device(h->ddt_prod, ddt_prod, size_t(h->n_vals), mem, st));
    if (h->conv) {
        if (ddt_conv) EMBER_TRY(copy_to_device(h->ddt_conv, ddt_conv, size_t(h->n_vals), mem, st));
        else EMBER_CUDA_TRY(cudaMemsetAsync(h->ddt_conv, 0, sizeof(double) * h->n_vals, st));
    }
    return finish_call(mem, st);
}

extern "C" int ember_split_source_status(ember_split h, int* status, int* stats, int mem, void* stream) {
    EMBER_TRY(check_split(h));
    EMBER_CHECK_ARG(mem == EMBER_MEM_HOST || mem == EMBER_MEM_DEVICE, "bad mem flag %d", mem);
    cudaStream_t st = as_stream(stream);
    const cudaMemcpyKind kind = mem == EMBER_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (status) EMBER_CUDA_TRY(cudaMemcpyAsync(status, h->src_status, sizeof(int) * h->n_pts, kind, st));
    if (stats) EMBER_CUDA_TRY(cudaMemcpyAsync(stats, h->src_stats, sizeof(int) * 4 * h->n_pts, kind, st));
    return finish_call(mem, st);
}

extern "C" int ember_split_failures(ember_split h, int64_t* source_points, int64_t* diffusion_systems,
                                    void* stream) {
    EMBER_TRY(check_split(h));
    cudaStream_t st = as_stream(stream);
    unsigned long long f[2] = {0, 0};
    EMBER_CUDA_TRY(cudaMemcpyAsync(f, h->fails, sizeof(f), cudaMemcpyDeviceToHost, st));
    EMBER_CUDA_TRY(cudaStreamSynchronize(st));
    if (source_points) *source_points = static_cast<int64_t>(f[0]);
    if (diffusion_systems) *diffusion_systems = static_cast<int64_t>(f[1]);
    return EMBER_OK;
}

extern "C" int ember_split_objectives(ember_split h, const double* rho_u, const int* ju, const int* jb,
                                      double* qdot, double* heat_release, double* consumption_speed, int mem,
                                      void* stream) {
    EMBER_TRY(check_split(h));
    EMBER_CHECK_ARG(mem == EMBER_MEM_HOST || mem == EMBER_MEM_DEVICE, "bad mem flag %d", mem);
    EMBER_CHECK_ARG(!consumption_speed || (rho_u && ju && jb), "consumption speed needs rho_u, ju and jb");
    if (consumption_speed && mem == EMBER_MEM_HOST) {
        for (int f = 0; f < h->n_flames; ++f)
            EMBER_CHECK_ARG(ju[f] >= 0 && ju[f] < h->grids[f].n_points && jb[f] >= 0 && jb[f] < h->grids[f].n_points,
                            "flame %d: ju/jb out of range", f);
    }
    cudaStream_t st = as_stream(stream);
    Scratch sc(st);
    const int S = h->mech->S;
    double *T, *Y, *net, *hk, *cp, *q, *qcp, *work;
    EMBER_TRY(sc.alloc(&T, h->n_pts));
    EMBER_TRY(sc.alloc(&Y, size_t(h->n_pts) * S));
    EMBER_TRY(sc.alloc(&net, size_t(h->n_pts) * S));
    EMBER_TRY(sc.alloc(&hk, size_t(h->n_pts) * S));
    EMBER_TRY(sc.alloc(&cp, h->n_pts));
    EMBER_TRY(sc.alloc(&qcp, h->n_pts));
    EMBER_TRY(sc.alloc(&work, 3 * h->n_pts));
    EMBER_TRY(stage_buffer(sc, qdot, size_t(h->n_pts), mem, &q));
    if (!q) EMBER_TRY(sc.alloc(&q, h->n_pts));
    double *hr = nullptr, *cs = nullptr;
    EMBER_TRY(stage_buffer(sc, heat_release, size_t(h->n_flames), mem, &hr));
    EMBER_TRY(stage_buffer(sc, consumption_speed, size_t(h->n_flames), mem, &cs));
    const double* d_rho = nullptr;
    const int *d_ju = nullptr, *d_jb = nullptr;
    if (consumption_speed) {
        EMBER_TRY(stage_in(sc, rho_u, size_t(h->n_flames), mem, st, &d_rho));
        EMBER_TRY(stage_in(sc, ju, size_t(h->n_flames), mem, st, &d_ju));
        EMBER_TRY(stage_in(sc, jb, size_t(h->n_flames), mem, st, &d_jb));
    }
    k_gather_TY<<<grid_for(h->n_pts * S), 256, 0, st>>>(h->n_pts, h->n_vars, h->state, T, Y);
    EMBER_TRY(ember_gas_eval(h->mech, static_cast<int>(h->n_pts), h->opt.source.pressure,
                             h->opt.source.kinetics_model, EMBER_STATE_NORMALIZED, T, Y, nullptr, nullptr, net, hk,
                             cp, nullptr, EMBER_MEM_DEVICE, stream));
    // qdot of the current state; q/cp with the c_p of the last property update when the transport
    // model ran one (FlameSolver::getConsumptionSpeed divides by the cp of updateChemicalProperties,
    // src/flameSolver.cpp:956-961), else with the current state's
    const double* cp_sc = (h->tr && h->props_valid) ? h->p_cp : cp;
    k_qdot<<<grid_for(h->n_pts, 128), 128, 0, st>>>(h->n_pts, S, net, hk, cp_sc, q, qcp);
    if (hr || cs)
        k_flame_objectives<<<blocks_for(h->n_flames, 64), 64, 0, st>>>(h->n_flames, h->flame_npts, h->flame_goff, h->x,
                                                                        q, qcp, T, d_rho, d_ju, d_jb, work, hr, cs);
    EMBER_CUDA_TRY(cudaGetLastError());
    EMBER_TRY(stage_out(qdot, q, size_t(h->n_pts), mem, st));
    EMBER_TRY(stage_out(heat_release, hr, size_t(h->n_flames), mem, st));
    EMBER_TRY(stage_out(consumption_speed, cs, size_t(h->n_flames), mem, st));
    sc.release();
    return finish_call(mem, st);
}

extern "C" int ember_split_adjoint(ember_split h, const double* w_heat_release, const double* w_consumption_speed,
                                   const double* rho_u, const int* ju, const int* jb, int tape_cap,
                                   double* heat_release, double* consumption_speed, double* state_bar,
                                   double* lnk_bar, int mem, void* stream) {
    EMBER_TRY(check_split(h));
    const bool qss = h->opt.method == EMBER_SOURCE_QSS;
    EMBER_CHECK_ARG(!qss || h->opt.source.qss_stability_check == 0,
                    "the split-step adjoint with the QSS source needs qss_stability_check = 0");
    EMBER_CHECK_ARG(h->tr == nullptr, "the split-step adjoint holds B and D fixed: detach the transport model");
    EMBER_CHECK_ARG(!h->conv, "the split-step adjoint covers D-S-D: detach the convection stage");
    EMBER_CHECK_ARG(mem == EMBER_MEM_HOST || mem == EMBER_MEM_DEVICE, "bad mem flag %d", mem);
    EMBER_CHECK_ARG(w_heat_release || w_consumption_speed, "no objective weights");
    EMBER_CHECK_ARG(!w_consumption_speed || (rho_u && ju && jb), "consumption speed needs rho_u, ju and jb");
    EMBER_CHECK_ARG(tape_cap >= 0 && tape_cap <= (1 << 20), "bad tape_cap %d", tape_cap);
    if (tape_cap == 0) tape_cap = qss ? 4096 : 1024;
    cudaStream_t st = as_stream(stream);
    Scratch sc(st);
    const MechView& m = h->mech->view;
    const int n = h->n_vars, S = m.S, R = std::max(m.R, 1);
    const int64_t np = h->n_pts, nv = h->n_vals;
    const int nf = h->n_flames;
    // ---- forward: one taped step, then the objectives (the QSS adjoint
    // replays each step of the source stage from the recorded step starts;
    // its input stays in xD2)
    StepTape tape{};
    tape.cap = tape_cap;
    EMBER_TRY(sc.alloc(&tape.t_saved, 1));
    if (!qss) {
        tape.stride = bdf_tape_doubles(n, tape_cap);
        EMBER_TRY(sc.alloc(&tape.buf, size_t(np) * tape.stride));
    } else if (qss_tape_doubles(m, static_cast<int>(np), tape_cap) * sizeof(double) <= kQssTapeBudgetBytes) {
        // the forward step's QSS launch records every step start; beyond the
        // budget the adjoint integrates the stage again from its input
        tape.stride = int64_t(kQssTapeHeader) + int64_t(tape_cap) * (n + 2);
        EMBER_TRY(sc.alloc(&tape.buf, qss_tape_doubles(m, static_cast<int>(np), tape_cap)));
    }
    EMBER_TRY(sc.alloc(&tape.xF, size_t(nv)));
    EMBER_TRY(enqueue_step(h, st, &tape));
    double *T, *Y, *net, *hk, *cp, *q, *qcp, *work, *hr, *cs;
    EMBER_TRY(sc.alloc(&T, np));
    EMBER_TRY(sc.alloc(&Y, size_t(np) * S));
    EMBER_TRY(sc.alloc(&net, size_t(np) * S));
    EMBER_TRY(sc.alloc(&hk, size_t(np) * S));
    EMBER_TRY(sc.alloc(&cp, np));
    EMBER_TRY(sc.alloc(&q, np));
    EMBER_TRY(sc.alloc(&qcp, np));
    EMBER_TRY(sc.alloc(&work, 4 * np));
    EMBER_TRY(sc.alloc(&hr, nf));
    EMBER_TRY(sc.alloc(&cs, nf));
    const double *d_wq = nullptr, *d_ws = nullptr, *d_rho = nullptr;
    const int *d_ju = nullptr, *d_jb = nullptr;
    EMBER_TRY(stage_in(sc, w_heat_release, size_t(nf), mem, st, &d_wq));
    EMBER_TRY(stage_in(sc, w_consumption_speed, size_t(nf), mem, st, &d_ws));
    if (w_consumption_speed) {
        EMBER_TRY(stage_in(sc, rho_u, size_t(nf), mem, st, &d_rho));
        EMBER_TRY(stage_in(sc, ju, size_t(nf), mem, st, &d_ju));
        EMBER_TRY(stage_in(sc, jb, size_t(nf), mem, st, &d_jb));
    }
    k_gather_TY<<<grid_for(np * S), 256, 0, st>>>(np, n, h->state, T, Y);
    EMBER_TRY(ember_gas_eval(h->mech, static_cast<int>(np), h->opt.source.pressure, h->opt.source.kinetics_model,
                             EMBER_STATE_NORMALIZED, T, Y, nullptr, nullptr, net, hk, cp, nullptr, EMBER_MEM_DEVICE,
                             stream));
    k_qdot<<<grid_for(np, 128), 128, 0, st>>>(np, S, net, hk, cp, q, qcp);
    k_flame_objectives<<<blocks_for(nf, 64), 64, 0, st>>>(nf, h->flame_npts, h->flame_goff, h->x, q, qcp, T, d_rho,
                                                          d_ju, d_jb, work, hr, d_ws ? cs : nullptr);
    // ---- backward: objectives -> end state
    double *omega, *gq, *gcp, *gT, *ybar, *prow_obj, *prow_src, *ybar2;
    int* adj_status;
    EMBER_TRY(sc.alloc(&omega, np));
    EMBER_TRY(sc.alloc(&gq, np));
    EMBER_TRY(sc.alloc(&gcp, np));
    EMBER_TRY(sc.alloc(&gT, np));
    EMBER_TRY(sc.alloc(&ybar, nv));
    EMBER_TRY(sc.alloc(&ybar2, nv));
    EMBER_TRY(sc.alloc(&prow_obj, size_t(np) * R));
    EMBER_TRY(sc.alloc(&prow_src, size_t(np) * R));
    EMBER_TRY(sc.alloc(&adj_status, np));
    k_spline_weights<<<blocks_for(nf, 64), 64, 0, st>>>(nf, h->flame_npts, h->flame_goff, h->x, work, omega);
    k_objective_weights<<<blocks_for(nf, 64), 64, 0, st>>>(nf, h->flame_npts, h->flame_goff, omega, q, cp, T, d_wq,
                                                           d_ws, d_rho, d_ju, d_jb, cs, gq, gcp, gT);
    SourceArgs oa = make_source_args(&h->opt.source, static_cast<int>(np), nullptr, nullptr, nullptr, 0.0, nullptr,
                                     nullptr, nullptr, nullptr);
    oa.ign_energy = 0.0;  // calculateQdot has no igniter term
    EMBER_TRY(launch_objective_vjp(m, oa, static_cast<int>(np), h->state, gq, gcp, gT, ybar, prow_obj, sc, st));
    // mass-fraction correction
    k_correct_mass_fractions_adjoint<<<grid_for(np, 128), 128, 0, st>>>(np, n, tape.xF, ybar);
    // diffusion 4/4 and 3/4 (transposed), in the variable-major layout
    const SplitTables tb = h->tables();
    const int g = grid_for(nv);
    double* dwork;
    EMBER_TRY(sc.alloc(&dwork, size_t(7) * nv));
    auto diffusion_pair_adjoint = [&](double fa, double fb, double fc) -> int {
        k_to_varmajor<<<g, 256, 0, st>>>(tb, ybar, ybar2, h->ystart);
        const DiffusionView dv = h->diffusion_view(h->diff_status);
        const double fr[3] = {fa, fb, fc};
        for (int k = 1; k >= 0; --k) {
            StageTime tm;
            tm.t_dev = tape.t_saved;
            tm.f0 = fr[k];
            tm.f1 = fr[k + 1];
            tm.dt = h->opt.dt;
            EMBER_TRY(diffusion_adjoint_run(dv, ybar2, dwork, nv, h->nmax, tm, h->opt.dt_multiplier, h->opt.dt, st));
        }
        k_to_pointmajor<<<g, 256, 0, st>>>(tb, ybar2, ybar, nullptr);
        return EMBER_OK;
    };
    EMBER_TRY(diffusion_pair_adjoint(0.5, 0.75, 1.0));
    // source stage
    {
        SourceArgs a = h->source_args();
        a.t_start_dev = tape.t_saved;
        a.tape = tape.buf;
        a.tape_stride = tape.stride;
        a.tape_cap = tape.cap;
        int* counter = nullptr;
        EMBER_TRY(sc.alloc(&counter, 1));
        EMBER_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(int), st));
        if (qss) {
            // the replayed forward writes its end states into scratch, not into the step's state
            EMBER_TRY(sc.alloc(&a.state_out, size_t(nv)));
            a.status = nullptr;
            a.stats = nullptr;
            EMBER_TRY(launch_source_qss_adjoint(m, a, tape_cap, counter, h->src_status, ybar, ybar2, prow_src,
                                                adj_status, sc, st));
        } else {
            EMBER_TRY(launch_source_bdf_adjoint(m, a, counter, ybar, ybar2, prow_src, adj_status, sc, st));
        }
        EMBER_CUDA_TRY(cudaMemcpyAsync(ybar, ybar2, sizeof(double) * nv, cudaMemcpyDeviceToDevice, st));
        k_count_failures<<<grid_for(np), 256, 0, st>>>(static_cast<int>(np), adj_status, h->fails);
    }
    // diffusion 2/4 and 1/4
    EMBER_TRY(diffusion_pair_adjoint(0.0, 0.25, 0.5));
    // ---- outputs
    double* d_lnk = nullptr;
    EMBER_TRY(stage_buffer(sc, lnk_bar, size_t(R), mem, &d_lnk));
    if (d_lnk) k_sum_rows2<<<blocks_for(R, 128), 128, 0, st>>>(np, R, prow_obj, prow_src, d_lnk);
    EMBER_CUDA_TRY(cudaGetLastError());
    const cudaMemcpyKind kind = mem == EMBER_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (state_bar) EMBER_CUDA_TRY(cudaMemcpyAsync(state_bar, ybar, sizeof(double) * nv, kind, st));
    if (heat_release) EMBER_CUDA_TRY(cudaMemcpyAsync(heat_release, hr, sizeof(double) * nf, kind, st));
    if (consumption_speed && d_ws)
        EMBER_CUDA_TRY(cudaMemcpyAsync(consumption_speed, cs, sizeof(double) * nf, kind, st));
    if (lnk_bar) EMBER_TRY(stage_out(lnk_bar, d_lnk, size_t(m.R), mem, st));
    sc.release();
    return finish_call(mem, st);
}
