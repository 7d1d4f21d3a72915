// CTA-per-point QSS integrator: the CHEMEQ2-style predictor-corrector of
// QssIntegrator (src/qssintegrator.cpp:58-265), with the state vectors of one
// point in shared memory (element i on thread i mod NT) and every scalar of
// the step control replicated across the CTA. Generic over the right-hand
// side (QssOde::odefun, src/qssintegrator.h:6-21): `Ode` provides
//     __device__ void eval(double t, const double* y, double* q, double* d, bool corrector)
// called by all threads with y, q, d in shared memory; it must end with a
// barrier.
//
// Arithmetic forms (identical in the CPU oracle): the Pade factors are
// evaluated in Horner form with fma, and the predictor and corrector updates
// are each written over a single division,
//     predictor:  (q - d) den / (den + num),  num/den = r(180+r(60+r(11+r))) / (360+r(60+r(12+r)))
//     corrector:  (qs (ad - an) + q an - ys rb ad / dt) / (ad + an rb),  alpha = an/ad
// which are the reference's expressions multiplied through by den (resp. ad).
#pragma once

#include "chem.cuh"

namespace ember {

struct QssParams {
    double epsmin, epsmax, dtmin, dtmax, abstol;
    int itermax, stability_check;
    int max_steps;
};

// Shared-memory vectors of one point (n entries each; ym1/ym2 only with the
// stability check).
struct QssSmem {
    double *y, *q, *d, *rtau, *rtaus, *y1, *ys, *qs, *scratch, *ym1, *ym2;
    static __host__ __device__ size_t doubles(int n, bool stab) { return size_t(stab ? 11 : 9) * n; }
    __device__ void carve(double* base, int n, bool stab) {
        y = base;
        q = y + n;
        d = q + n;
        rtau = d + n;
        rtaus = rtau + n;
        y1 = rtaus + n;
        ys = y1 + n;
        qs = ys + n;
        scratch = qs + n;
        ym1 = stab ? scratch + n : nullptr;
        ym2 = stab ? ym1 + n : nullptr;
    }
};

struct QssStats {
    int steps, gcount, rcount;
};

// Integrator state between two steps, for suspending a point after a number
// of steps and resuming it later (in another launch, with another CTA width):
// everything the step loop carries from one step to the next.
struct QssResume {
    double tn, dt;
    int steps, gcount, rcount, started;
};
constexpr int kQssSuspended = -31;
// QSS tape of a point (SourceArgs::tape with a QSS launch): a header of
// kQssTapeHeader doubles (steps taken, overflow flag), then one record of
// n + 2 doubles per step start (see qss_integrate_block).
constexpr int kQssTapeHeader = 2;

__device__ __forceinline__ double rsign(double x) { return (x > 0) ? 1.0 : (x < 0) ? -1.0 : 0.0; }

// Pade numerator / denominator of the QSS predictor and corrector.
__device__ __forceinline__ double pade_num(double r) { return r * fma(r, fma(r, 11.0 + r, 60.0), 180.0); }
__device__ __forceinline__ double pade_den(double r) { return fma(r, fma(r, 12.0 + r, 60.0), 360.0); }
__device__ __forceinline__ double pade_an(double r) { return fma(r, fma(r, 11.0 + r, 60.0), 180.0); }

// enforce(i): whether component i is limited to ymin(i) (QssIntegrator::enforce_ymin / ymin).
// red: block reduction scratch (kMaxChemThreads + 2 doubles).
// step_cap > 0: stop before step step_cap + 1 (counted from the first step
// of the point, across resumptions), save the loop state in *rs and return
// kQssSuspended. rs with started set: continue from that state.
// tape (or null): the start of every step k < tape_cap is recorded at
// tape + k (n + 2): time, step size carried into the step (0 before the
// first), state (for the adjoint, qss_adjoint.cu).
template <int NT, class Ode, class Enforce, class Ymin>
__device__ __forceinline__ int qss_integrate_block(Ode& ode, QssSmem& v, int n, const QssParams& P, Enforce enforce,
                                                   Ymin ymin, double tf, double tstart, double* red, QssStats& st,
                                                   int step_cap = 0, QssResume* rs = nullptr, double* tape = nullptr,
                                                   int tape_cap = 0) {
    const int t0 = threadIdx.x;
    const double tfd = 1.000008;
    const bool stab_on = P.stability_check != 0;
    // setState: y limited to ymin where enforced; q, d zeroed (initialize()).
    for (int i = t0; i < n; i += NT) {
        v.y[i] = enforce(i) ? dmaxr(v.y[i], ymin(i)) : v.y[i];
        v.q[i] = 0.0;
        v.d[i] = 0.0;
        if (stab_on) {
            v.ym1[i] = 0.0;
            v.ym2[i] = 0.0;
        }
    }
    __syncthreads();
    double tn = 0.0, ts = 0.0, dt = 0.0;
    bool first = true;
    int gcount = 0, rcount = 0, steps = 0;
    if (rs && rs->started) {
        tn = rs->tn;
        dt = rs->dt;
        first = false;
        steps = rs->steps;
        gcount = rs->gcount;
        rcount = rs->rcount;
    }
    int ret = 0;
    while (tfd * tn < tf) {
        if (steps >= P.max_steps) {
            ret = -20;
            break;
        }
        if (step_cap > 0 && steps >= step_cap) {
            ret = kQssSuspended;
            if (rs && t0 == 0) *rs = QssResume{tn, dt, steps, gcount, rcount, 1};
            break;
        }
        ++steps;
        if (tape && steps <= tape_cap) {
            double* rec = tape + size_t(steps - 1) * (n + 2);
            if (t0 == 0) {
                rec[0] = tn;
                rec[1] = dt;
            }
            for (int i = t0; i < n; i += NT) rec[2 + i] = v.y[i];
        }
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
            scrtch = block_max<NT>(red, scrtch);
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
            const double rdt = 1.0 / dt;
            for (int i = t0; i < n; i += NT) {
                const double r = v.rtau[i];
                const double den = pade_den(r);
                v.scratch[i] = ((v.q[i] - v.d[i]) * den) / (den + pade_num(r));
            }
            double eps = 1e-10;
            for (int iter = 0; iter < P.itermax; ++iter) {
                for (int i = t0; i < n; i += NT) {
                    if (stab_on) {
                        v.ym2[i] = v.ym1[i];
                        v.ym1[i] = v.y[i];
                    }
                    const double yi = dmaxr(ymin(i), fma(dt, v.scratch[i], v.ys[i]));
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
                    const double an = pade_an(rb);
                    const double ad = pade_den(rb);
                    const double num = fma(v.qs[i], ad - an, v.q[i] * an) - ((v.ys[i] * rb) * ad) * rdt;
                    v.scratch[i] = num / fma(an, rb, ad);
                }
            }
            double epsl = eps;
            for (int i = t0; i < n; i += NT) {
                const double ym = ymin(i);
                double scr2 = fma(dt, v.scratch[i], v.ys[i]);
                if (enforce(i)) scr2 = dmaxr(scr2, ym);
                double scr1 = fabs(scr2 - v.y1[i]);
                const double yi = dmaxr(scr2, ym);
                v.y[i] = yi;
                if (fabs(yi) > P.abstol && 0.25 * (v.ys[i] + yi) > ym) {
                    scr1 = scr1 / yi;
                    epsl = dmaxr(.5 * (scr1 + dminr(fabs(v.q[i] - v.d[i]) / (v.q[i] + v.d[i] + 1e-30), scr1)), epsl);
                }
                if (stab_on) {
                    v.ym2[i] = v.ym1[i];
                    v.ym1[i] = yi;
                }
            }
            eps = block_max<NT>(red, epsl);  // includes a barrier: y is complete
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
                stab = block_max<NT>(red, sl);
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
                const double ratio = dt / dto;
                for (int i = t0; i < n; i += NT) v.rtaus[i] *= ratio;
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
