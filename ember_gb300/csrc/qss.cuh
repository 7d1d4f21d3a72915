// CTA-per-point QSS integrator: the CHEMEQ2-style predictor-corrector of
// QssIntegrator (src/qssintegrator.cpp:58-265), with the state vectors of one
// point in shared memory (element i on thread i mod kChemThreads) and every
// scalar of the step control replicated across the CTA. Generic over the
// right-hand side (QssOde::odefun, src/qssintegrator.h:6-21): `Ode` provides
//     __device__ void eval(double t, const double* y, double* q, double* d, bool corrector)
// called by all threads with y, q, d in shared memory; it must end with a
// barrier.
#pragma once

#include "chem.cuh"

namespace ember {

struct QssParams {
    double epsmin, epsmax, dtmin, dtmax, abstol;
    int itermax, stability_check;
    int max_steps;
};

// Shared-memory vectors of one point (n entries each).
struct QssSmem {
    double *y, *q, *d, *rtau, *rtaus, *y1, *ys, *qs, *ym1, *ym2, *scratch, *ymin;
    static __host__ __device__ size_t doubles(int n) { return size_t(12) * n; }
    __device__ void carve(double* base, int n) {
        y = base;
        q = y + n;
        d = q + n;
        rtau = d + n;
        rtaus = rtau + n;
        y1 = rtaus + n;
        ys = y1 + n;
        qs = ys + n;
        ym1 = qs + n;
        ym2 = ym1 + n;
        scratch = ym2 + n;
        ymin = scratch + n;
    }
};

struct QssStats {
    int steps, gcount, rcount;
};

__device__ __forceinline__ double rsign(double x) { return (x > 0) ? 1.0 : (x < 0) ? -1.0 : 0.0; }

// enforce(i): whether component i is limited to ymin (QssIntegrator::enforce_ymin).
// red: block reduction scratch (kChemThreads + 2 doubles).
template <class Ode, class Enforce>
__device__ __forceinline__ int qss_integrate_block(Ode& ode, QssSmem& v, int n, const QssParams& P, Enforce enforce, double tf,
                                   double tstart, double* red, QssStats& st) {
    const int t0 = threadIdx.x;
    constexpr int NT = kChemThreads;
    const double tfd = 1.000008;
    // setState: y limited to ymin where enforced; q, d zeroed (initialize()).
    for (int i = t0; i < n; i += NT) {
        v.y[i] = enforce(i) ? dmaxr(v.y[i], v.ymin[i]) : v.y[i];
        v.q[i] = 0.0;
        v.d[i] = 0.0;
        v.ym1[i] = 0.0;
        v.ym2[i] = 0.0;
    }
    __syncthreads();
    double tn = 0.0, ts = 0.0, dt = 0.0;
    bool first = true;
    int gcount = 0, rcount = 0, steps = 0;
    int ret = 0;
    const bool stab_on = P.stability_check != 0;
    while (tfd * tn < tf) {
        if (steps >= P.max_steps) {
            ret = -20;
            break;
        }
        ++steps;
        // ---- integrateOneStep --------------------------------------------
        ode.eval(tn + tstart, v.y, v.q, v.d, false);
        gcount += 1;
        if (first) {
            first = false;
            double scrtch = 1.0e-25;
            for (int i = t0; i < n; i += NT) {
                if (fabs(v.y[i]) > P.abstol) {
                    const double absq = fabs(v.q[i]);
                    const double scr2 = fabs(1 / v.y[i]) * rsign(0.1 * P.epsmin * absq - v.d[i]);
                    const double scr1 = scr2 * v.d[i];
                    scrtch = dmaxr(dmaxr(scr1, -fabs(absq - v.d[i]) * scr2), scrtch);
                }
            }
            scrtch = block_max(red, scrtch);
            const double sqreps = 0.5;
            dt = dminr(sqreps / scrtch, tf);
            dt = dminr(dt, P.dtmax);
        }
        ts = tn;
        for (int i = t0; i < n; i += NT) {
            const double r = enforce(i) ? dt * v.d[i] / v.y[i] : 0.0;
            v.rtau[i] = r;
            v.rtaus[i] = r;
            v.qs[i] = v.q[i];
            v.ys[i] = v.y[i];
        }
        int step_ret = 1;  // 1: keep looping
        while (step_ret == 1) {
            for (int i = t0; i < n; i += NT) {
                const double r = v.rtau[i];
                v.scratch[i] = (v.q[i] - v.d[i]) /
                               (1.0 + r * (180 + r * (60 + r * (11 + r))) / (360 + r * (60 + r * (12 + r))));
            }
            double eps = 1e-10;
            for (int iter = 0; iter < P.itermax; ++iter) {
                for (int i = t0; i < n; i += NT) {
                    if (stab_on) {
                        v.ym2[i] = v.ym1[i];
                        v.ym1[i] = v.y[i];
                    }
                    const double yi = dmaxr(v.ymin[i], v.ys[i] + dt * v.scratch[i]);
                    v.y[i] = yi;
                    if (iter == 0) v.y1[i] = yi;
                }
                if (iter == 0) tn = ts + dt;
                __syncthreads();
                ode.eval(tn + tstart, v.y, v.q, v.d, true);
                gcount += 1;
                eps = 1.0e-10;
                for (int i = t0; i < n; i += NT) {
                    const double rb = enforce(i) ? 0.5 * (v.rtaus[i] + dt * v.d[i] / v.y[i]) : 0.0;
                    const double alpha = (180. + rb * (60. + rb * (11. + rb))) / (360. + rb * (60. + rb * (12. + rb)));
                    v.scratch[i] = (v.qs[i] * (1.0 - alpha) + v.q[i] * alpha - v.ys[i] * rb / dt) / (1.0 + alpha * rb);
                }
            }
            double epsl = eps;
            for (int i = t0; i < n; i += NT) {
                double scr2 = v.ys[i] + dt * v.scratch[i];
                if (enforce(i)) scr2 = dmaxr(scr2, v.ymin[i]);
                double scr1 = fabs(scr2 - v.y1[i]);
                const double yi = dmaxr(scr2, v.ymin[i]);
                v.y[i] = yi;
                if (fabs(yi) > P.abstol && 0.25 * (v.ys[i] + yi) > v.ymin[i]) {
                    scr1 = scr1 / yi;
                    epsl = dmaxr(.5 * (scr1 + dminr(fabs(v.q[i] - v.d[i]) / (v.q[i] + v.d[i] + 1e-30), scr1)), epsl);
                }
                if (stab_on) {
                    v.ym2[i] = v.ym1[i];
                    v.ym1[i] = yi;
                }
            }
            eps = block_max(red, epsl);  // includes a barrier: y is complete
            eps /= P.epsmin;
            if (dt <= P.dtmin + 1e-16 * tn) {
                step_ret = -1;
                break;
            }
            double stab = 0;
            if (stab_on && P.itermax >= 3) {
                // ym1 == y here, so the reference's ratio compares y with itself
                double sl = 0.01;
                for (int i = t0; i < n; i += NT)
                    if (fabs(v.y[i]) > P.abstol)
                        sl = dmaxr(sl, fabs(v.y[i] - v.ym1[i]) / (fabs(v.ym1[i] - v.ym2[i]) + 1e-20 * v.y[i]));
                stab = block_max(red, sl);
            }
            if (eps <= P.epsmax && stab <= 1.0) {
                if (tf <= tn * tfd) {
                    step_ret = 0;
                    break;
                }
            } else {
                tn = ts;
            }
            double rteps = 0.5 * (eps + 1.0);
            rteps = 0.5 * (rteps + eps / rteps);
            rteps = 0.5 * (rteps + eps / rteps);
            const double dto = dt;
            dt = dminr(dt * (1.0 / rteps + 0.005), tfd * (tf - tn));
            dt = dminr(dt, P.dtmax);
            if (stab_on) dt = dminr(dt, dto / (stab + .001));
            if (eps > P.epsmax || stab > 1) {
                rcount += 1;
                for (int i = t0; i < n; i += NT) v.rtaus[i] *= dt / dto;
            } else {
                step_ret = 0;
            }
        }
        if (step_ret != 0) {
            ret = step_ret;
            break;
        }
    }
    __syncthreads();
    st.steps = steps;
    st.gcount = gcount;
    st.rcount = rcount;
    return ret;
}

}  // namespace ember
