// Discrete adjoint of the QSS source-term integration on the GPU
// (SourceSystemQSS + QssIntegrator: src/sourceSystem.cpp:403-531,
// src/qssintegrator.cpp:58-265; the reference integrates forward only).
//
// One CTA per point, persistent grid with an atomic work counter. For each
// point the kernel runs the integration forward (the operations of
// qss_integrate_block, so the end state is the forward kernel's, bit for
// bit), keeping every step's start state, time and initial step size in a
// per-CTA tape; then it walks the steps backwards. Each step is replayed from
// its start state with every intermediate kept (the attempts' predictor and
// corrector states and rates, the error estimates, the branches taken), and
// the replay is differentiated in reverse:
//   every attempt of the step, because a retried attempt's predictor uses
//   the rates of the rejected attempt's last corrector evaluation;
//   the step sizes as functions of the state: getInitialStepSize's
//   max over components, each new step size from the error estimate eps
//   (dt (1/sqrt(eps) + 0.005), the square root by the integrator's two
//   Newton iterations), or the clip tfd (tf - t), or dtmax, whichever the
//   forward pass took; rtaus = rtau dt_a / dt_0 after rejections;
//   each right-hand side evaluation: the mass fractions analytically (rates
//   of progress, third-body concentrations, falloff blending, the clip and
//   normalisation of setState_TPY), the temperature by a forward
//   difference of step sqrt(eps) |T| (rate constants, 1/Kc, thermo); a
//   corrector evaluation uses the predictor's T, rho and cp, so its
//   adjoint flows back to the step's start state through them.
// The accept / reject decisions and the components that take each max stay
// fixed. d ropf_i / d ln(multiplier_i) = ropf_i and likewise ropr_i give the
// gradient with respect to every reaction's ln(multiplier), per point.
// The CPU restatement of the same adjoint is oracle/oracle_qss_adjoint.c.
//
// Compiled with --fmad=false: the forward replay must reproduce the forward
// kernel's bits (only explicit fma() calls are fused).

#include <algorithm>

#include "common.cuh"
#include "source.cuh"

namespace ember {
namespace {

constexpr int kQaMaxAttempts = 32;
constexpr int kQaMaxIter = 4;

__device__ __forceinline__ double pade_num_d(double r) { return fma(r, fma(r, fma(4.0, r, 33.0), 120.0), 180.0); }
__device__ __forceinline__ double pade_den_d(double r) { return fma(r, fma(3.0, r, 24.0), 60.0); }
__device__ __forceinline__ double pade_an_d(double r) { return fma(r, fma(3.0, r, 22.0), 60.0); }

// Sum of one value per thread (fixed tree for a given width).
template <int NT>
__device__ __forceinline__ double block_add(double* red, double v) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = red[0];
#pragma unroll
    for (int w = 1; w < NT / 32; ++w) r += red[w];
    __syncthreads();
    return r;
}

// The largest value over the CTA and, among equal values, the largest
// index: the element a sequential scan "if (!(v < best)) take v" keeps.
template <int NT>
__device__ __forceinline__ void block_argmax(double* red, int* ired, double& v, int& idx) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, v, off);
        const int oi = __shfl_xor_sync(0xffffffffu, idx, off);
        if (ov > v || (ov == v && oi > idx)) {
            v = ov;
            idx = oi;
        }
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
        red[threadIdx.x >> 5] = v;
        ired[threadIdx.x >> 5] = idx;
    }
    __syncthreads();
    v = red[0];
    idx = ired[0];
#pragma unroll
    for (int w = 1; w < NT / 32; ++w)
        if (red[w] > v || (red[w] == v && ired[w] > idx)) {
            v = red[w];
            idx = ired[w];
        }
    __syncthreads();
}

// What a step's replay keeps besides the vectors (uniform over the CTA;
// thread 0 writes).
struct QaScalars {
    int A;                                  // attempts (the last one accepted)
    double dt[kQaMaxAttempts + 1];          // step size of each attempt; dt[A]: the next step's
    double eps[kQaMaxAttempts], rteps[kQaMaxAttempts];
    int imax[kQaMaxAttempts], ebr[kQaMaxAttempts];  // eps's component; 0: el = scr1, 1: el = (scr1 + g)/2
    int dtbr[kQaMaxAttempts + 1];           // 0: dt (1/rteps + .005), 1: tfd (tf - t), 2: dtmax
    int dt0_br, dt0_imax, dt0_side;         // initial step: 0 scrtch, 1 tf, 2 dtmax; argmax; 0 scr1, 1 other
    double scrtch;
    double T, rrho, rrc, rho, cp;           // the predictor call's
};

template <int NT>
struct QaPoint {
    const MechView& m;
    __device__ explicit QaPoint(const MechView& mv) : m(mv) {}
    ChemSmem w;
    const SourceArgs* a = nullptr;
    const double* split = nullptr;
    double x = 0.0;
    int n = 0, S = 0, I = 1;
    double T = 0.0, rrho = 1.0, rrc = 1.0, rho_p = 1.0, cp_p = 1.0, qdot = 0.0, rho_c = 1.0;
    double cachedT = 0.0;
    double tf = 0.0, tstart = 0.0;
    // shared memory: adjoints of the creation / destruction rates and concentrations
    double *wqb = nullptr, *wdb = nullptr, *cb = nullptr;
    int* ired = nullptr;
    // per-CTA global work area
    double *ys = nullptr, *q0 = nullptr, *d0 = nullptr, *rtau = nullptr;
    double *q2 = nullptr, *d2 = nullptr, *ycp = nullptr;
    double *ysb = nullptr, *q0b = nullptr, *d0b = nullptr, *rtaub = nullptr, *qnb = nullptr, *dnb = nullptr;
    double *rtsb = nullptr, *rtsbc = nullptr, *scrb = nullptr, *yfb = nullptr, *qjb = nullptr, *djb = nullptr;
    double *yjb = nullptr, *att = nullptr, *fdb = nullptr, *sav = nullptr;

    // One saved evaluation: what the adjoint of an evaluation reads that
    // depends on the composition (the temperature-only values stay in the
    // rate-constant cache, since every evaluation of a step but the
    // temperature differences runs at the predictor's T).
    static __host__ __device__ size_t save_doubles(const MechView& mv) {
        return size_t(4) * mv.S + mv.n_tb + size_t(2) * mv.R + size_t(4) * mv.n_fo + 4;
    }
    static __host__ __device__ size_t work_doubles(const MechView& mv, int I) {
        const int n = mv.S + 2;
        return size_t(21 + I) * n + size_t(kQaMaxAttempts) * size_t(4 + 4 * I) * n +
               size_t(kQaMaxAttempts) * I * 2 * n + (1 + size_t(kQaMaxAttempts) * I) * save_doubles(mv);
    }
    __device__ void carve_work(double* g) {
        ys = g;
        q0 = ys + n;
        d0 = q0 + n;
        rtau = d0 + n;
        q2 = rtau + n;
        d2 = q2 + n;
        ycp = d2 + n;
        ysb = ycp + n;
        q0b = ysb + n;
        d0b = q0b + n;
        rtaub = d0b + n;
        qnb = rtaub + n;
        dnb = qnb + n;
        rtsb = dnb + n;
        rtsbc = rtsb + n;
        scrb = rtsbc + n;
        yfb = scrb + n;
        qjb = yfb + n;
        djb = qjb + n;
        // then two vectors the kernel carves after djb (19 n + 2 n in all), then yjb
        yjb = djb + n + 2 * size_t(n);
        att = yjb + size_t(I) * n;
        fdb = att + size_t(kQaMaxAttempts) * (4 + 4 * I) * n;
        sav = fdb + size_t(kQaMaxAttempts) * I * 2 * n;
    }
    // saved evaluations: slot 0 the predictor, 1 + a I + j corrector j of attempt a
    __device__ double* sv_slot(int slot) const { return sav + size_t(slot) * save_doubles(m); }
    __device__ double* at_rtaus(int a) const { return att + size_t(a) * (4 + 4 * I) * n; }
    __device__ double* at_scrp(int a) const { return at_rtaus(a) + n; }
    __device__ double* at_y(int a, int j) const { return at_rtaus(a) + size_t(2 + 4 * j) * n; }
    __device__ double* at_q(int a, int j) const { return at_y(a, j) + n; }
    __device__ double* at_d(int a, int j) const { return at_y(a, j) + 2 * n; }
    __device__ double* at_scr(int a, int j) const { return at_y(a, j) + 3 * n; }
    __device__ double* at_raw(int a) const { return at_rtaus(a) + size_t(2 + 4 * I) * n; }
    __device__ double* at_yf(int a) const { return at_raw(a) + n; }
    __device__ double* fd_q(int a, int j) const { return fdb + (size_t(a) * I + j) * 2 * n; }
    __device__ double* fd_d(int a, int j) const { return fd_q(a, j) + n; }

    __device__ bool en(int i) const { return i != 0; }
    __device__ double ymin(int i) const { return i == 0 ? -1e4 : a->qss_minval; }

    // SourceSystemQSS::odefun with the operations of the forward kernel's
    // right-hand side (source.cu, SourceQssOde::eval). Starts and ends with a barrier.
    __device__ void eval(double t, const double* y, double* q, double* d, bool corrector, double* save = nullptr) {
        const int tid = threadIdx.x;
        __syncthreads();
        if (!corrector) T = y[1];
        if (!(cachedT == T)) {
            chem_rate_constants<NT>(m, w, T, a->kinetics_model == KIN_INTERP);
            cachedT = T;
        }
        double rc, cpc;
        chem_rates<NT>(m, w, a->pressure, STATE_NORMALIZED, T, y + 2, rc, cpc, false);
        if (!corrector) {
            rrho = 1.0 / rc;
            rrc = 1.0 / (rc * cpc);
            rho_p = rc;
            cp_p = cpc;
        }
        rho_c = rc;
        const double *wq = w.wq, *wd = w.wd, *hk = w.hk;
        const double qd =
            -block_sum<NT>(w.red, S, [&](int k, double p) { return fma(wq[k] - wd[k], hk[k], p); }) + igniter(*a, t, x);
        qdot = qd;
        if (save) {
            const int S_ = S, R = m.R, ntb = m.n_tb, nfo = m.n_fo;
            double* p = save;
            for (int k = tid; k < S_; k += NT) {
                p[k] = w.c[k];
                p[S_ + k] = w.ym[k];
                p[2 * S_ + k] = w.wq[k];
                p[3 * S_ + k] = w.wd[k];
            }
            p += 4 * S_;
            for (int s2 = tid; s2 < ntb; s2 += NT) p[s2] = w.concm[s2];
            p += ntb;
            for (int i = tid; i < R; i += NT) {
                p[i] = w.ropf[i];
                p[R + i] = w.ropr[i];
            }
            p += 2 * R;
            for (int f = tid; f < nfo; f += NT) {
                p[f] = w.fo_F[f];
                p[nfo + f] = w.fo_pr[f];
                p[2 * nfo + f] = w.fo_dF[f];
                p[3 * nfo + f] = w.kfm[m.fo_rxn[f]];
            }
            p += 4 * nfo;
            if (tid == 0) {
                p[0] = w.mmw;
                p[1] = rc;
                p[2] = qd;
            }
        }
        for (int i = tid; i < n; i += NT) {
            const double sc = split ? split[i] : 0.0;
            if (i == 0) {
                q[0] = sc;
                d[0] = 0.0;
            } else if (i == 1) {
                q[1] = fma(qd, rrc, sc);
                d[1] = 0.0 * rrc;
            } else {
                const int k = i - 2;
                q[i] = fma(w.wq[k] * m.W[k], rrho, sc);
                d[i] = (w.wd[k] * m.W[k]) * rrho;
            }
        }
        __syncthreads();
    }

    // Adjoint of the evaluation whose intermediates are in w (eval just
    // called on y), at fixed T. qb, db: adjoints of q, d. Accumulates the
    // mass-fraction part into yb + 2 and the multiplier part into pb; a
    // corrector call adds the adjoints of the rrho / rrc it used to *rrho_b
    // and *rrc_b; a predictor call takes the correctors' adjoints of its
    // rrho, rrc (ext_*) and sends all of them to rho and cp.
    __device__ void vjp(const double* y, const double* sv, const double* qb, const double* db, bool predictor,
                        double ext_rrho_b, double ext_rrc_b, double* yb, double* pb, double* rrho_b, double* rrc_b) {
        const int tid = threadIdx.x;
        const double* Y = y + 2;
        const int nfo = m.n_fo;
        const double* c = sv;
        const double* ym = c + S;
        const double* wq = ym + S;
        const double* wd = wq + S;
        const double* concm = wd + S;
        const double* ropf = concm + m.n_tb;
        const double* ropr = ropf + m.R;
        const double* foF = ropr + m.R;
        const double* fopr = foF + nfo;
        const double* fodF = fopr + nfo;
        const double* fokfm = fodF + nfo;
        const double mmw = fokfm[nfo], rho = fokfm[nfo + 1], qdot_s = fokfm[nfo + 2];
        __syncthreads();
        const double qdb = qb[1] * rrc;
        double part = 0.0;
        for (int k = tid; k < S; k += NT) {
            wqb[k] = qb[2 + k] * m.W[k] * rrho - qdb * w.hk[k];
            wdb[k] = db[2 + k] * m.W[k] * rrho + qdb * w.hk[k];
            cb[k] = 0.0;
            part += qb[2 + k] * wq[k] * m.W[k] + db[2 + k] * wd[k] * m.W[k];
        }
        const double own_rrho_b = block_add<NT>(w.red, part);
        const double own_rrc_b = qb[1] * qdot_s;
        double rho_b_in = 0.0, cp_b_in = 0.0;
        if (predictor) {
            const double rr_b = own_rrho_b + ext_rrho_b, rc_b = own_rrc_b + ext_rrc_b;
            rho_b_in = -rr_b * rrho * rrho - rc_b * rrc * rrc * cp_p;
            cp_b_in = -rc_b * rrc * rrc * rho_p;
        } else {
            *rrho_b += own_rrho_b;
            *rrc_b += own_rrc_b;
        }
        // rates of progress -> concentrations, [M], multipliers
        double ctot_part = 0.0;
        for (int i = tid; i < m.R; i += NT) {
            const int info = m.rinfo[i];
            const int ty = rinfo_type(info);
            const bool rev = rinfo_rev(info);
            const int4 st = m.stoich[i];
            const int rc4[4] = {unpack_lo(st.x), unpack_hi(st.x), unpack_lo(st.y), unpack_hi(st.y)};
            const int pd4[4] = {unpack_lo(st.z), unpack_hi(st.z), unpack_lo(st.w), unpack_hi(st.w)};
            double fb = 0.0, rbb = 0.0, pf = 1.0, pp = 1.0;
#pragma unroll
            for (int o = 0; o < 4; ++o) {
                if (pd4[o] != 0xffff) {
                    fb += wqb[pd4[o]];
                    rbb += wdb[pd4[o]];
                    pp *= c[pd4[o]];
                }
                if (rc4[o] != 0xffff) {
                    fb += wdb[rc4[o]];
                    rbb += wqb[rc4[o]];
                    pf *= c[rc4[o]];
                }
            }
            pb[i] += fb * ropf[i] + rbb * ropr[i];
            int slot = -1, fo = -1;
            if (ty != RXN_ELEMENTARY) {
                slot = rinfo_tbslot(info);
                fo = m.tb_fo[slot];
            }
            const double kfm = fo >= 0 ? fokfm[fo] : w.kfm[i];
            const double rf = ty == RXN_THREE_BODY ? kfm * concm[slot] : kfm;
            const double kr = rev ? w.rkc[i] : 0.0;
#pragma unroll
            for (int o = 0; o < 4; ++o) {
                if (rc4[o] == 0xffff) continue;
                double dv = rf;
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (q != o && rc4[q] != 0xffff) dv *= c[rc4[q]];
                atomicAdd(&cb[rc4[o]], fb * dv);
            }
            if (rev) {
#pragma unroll
                for (int o = 0; o < 4; ++o) {
                    if (pd4[o] == 0xffff) continue;
                    double dv = rf * kr;
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        if (q != o && pd4[q] != 0xffff) dv *= c[pd4[q]];
                    atomicAdd(&cb[pd4[o]], rbb * dv);
                }
            }
            if (slot >= 0) {
                double Mb;
                if (ty == RXN_THREE_BODY) {
                    Mb = fb * (kfm * pf) + rbb * (kfm * kr * pp);
                } else {
                    const int f = fo;
                    const double prr = fopr[f], pr1 = 1.0 + prr;
                    const double dkdm = (foF[f] / (pr1 * pr1) + (prr / pr1) * fodF[f]) *
                                        (w.fo_k0[f] * w.fo_rkinf[f]) * w.fo_kinf[f] * m.mult[i];
                    Mb = (fb * pf + rbb * kr * pp) * dkdm;
                }
                ctot_part += Mb * m.tb_def[slot];
                const int e1 = m.tb_off[slot + 1];
                for (int e = m.tb_off[slot]; e < e1; ++e) atomicAdd(&cb[m.tb_sp[e]], Mb * m.tb_eff[e]);
            }
        }
        const double ctotb = block_add<NT>(w.red, ctot_part);  // also the barrier after the atomics
        // composition: c = ym rho, ctot = rho / mmw, rho = p mmw / (R T), mmw = 1 / sum ym,
        // ym = max(Y, 0) rnorm / W, rnorm = 1 / sum max(Y, 0); predictor: cp = R cpsum / mmw
        part = 0.0;
        double cps = 0.0, ycp_s = 0.0;
        for (int k = tid; k < S; k += NT) {
            part += cb[k] * ym[k];
            if (predictor) {
                cps += ym[k] * mmw * w.cpR[k];
                ycp_s += ym[k] * w.cpR[k];
            }
        }
        const double rhob = rho_b_in + ctotb / mmw + block_add<NT>(w.red, part);
        double mmwb = -ctotb * rho / (mmw * mmw);
        double cpsb = 0.0;
        if (predictor) {
            const double cpsum = block_add<NT>(w.red, cps);
            const double ycp_sum = block_add<NT>(w.red, ycp_s);
            cpsb = cp_b_in * kGasConstant / mmw;
            mmwb += -cp_b_in * kGasConstant * cpsum / (mmw * mmw) + cpsb * ycp_sum;
        }
        mmwb += rhob * a->pressure / (kGasConstant * T);
        double* ymb = wqb;  // reuse
        part = 0.0;
        double yps = 0.0;
        for (int k = tid; k < S; k += NT) {
            double v = cb[k] * rho + cpsb * mmw * w.cpR[k] - mmwb * mmw * mmw;
            ymb[k] = v;
            const double yp = dmaxr(Y[k], 0.0);
            part += v * yp * m.rW[k];
            yps += yp;
        }
        const double rnb = block_add<NT>(w.red, part);
        const double rnorm = 1.0 / block_add<NT>(w.red, yps);
        for (int k = tid; k < S; k += NT)
            if (Y[k] > 0.0) yb[2 + k] += ymb[k] * rnorm * m.rW[k] - rnb * rnorm * rnorm;
        __syncthreads();
    }

    // One integrateOneStep from ys_in at ts (first: the initial step size is
    // computed, else *dt is the step size), as qss_integrate_block, keeping
    // what the adjoint needs. y_out: the state after the step; *tn_out its
    // time; *dt the next step's size. Returns 0, -1 (dtmin) or -33 (more
    // than kQaMaxAttempts attempts).
    __device__ int step_run(const double* ys_in, double ts, bool first, double* dt, double* tn_out, double* y_out,
                            QaScalars& sc, bool keep) {
        const int tid = threadIdx.x;
        const double tfd = 1.000008;
        for (int i = tid; i < n; i += NT) ys[i] = ys_in[i];
        eval(ts + tstart, ys, q0, d0, false, keep ? sv_slot(0) : nullptr);
        if (tid == 0) {
            sc.T = T;
            sc.rrho = rrho;
            sc.rrc = rrc;
            sc.rho = rho_p;
            sc.cp = cp_p;
        }
        if (first) {
            double best = 1.0e-25;
            int bi = -1;
            for (int i = tid; i < n; i += NT) {
                if (fabs(ys[i]) > a->qss_abstol) {
                    const double absq = fabs(q0[i]);
                    const double scr2 = fabs(1 / ys[i]) * rsign(0.1 * a->qss_epsmin * absq - d0[i]);
                    const double scr1 = scr2 * d0[i];
                    const double mx = dmaxr(scr1, -fabs(absq - d0[i]) * scr2);
                    if (!(mx < best)) {
                        best = mx;
                        bi = i;
                    }
                }
            }
            block_argmax<NT>(w.red, ired, best, bi);
            const double d0v = dminr(0.5 / best, tf);
            int br = (tf < 0.5 / best) ? 1 : 0;
            if (a->qss_dtmax < d0v) br = 2;
            *dt = dminr(d0v, a->qss_dtmax);
            if (tid == 0) {
                sc.scrtch = best;
                sc.dt0_imax = bi;
                sc.dt0_br = br;
                int side = 0;
                if (bi >= 0) {
                    const double absq = fabs(q0[bi]);
                    const double scr2 = fabs(1 / ys[bi]) * rsign(0.1 * a->qss_epsmin * absq - d0[bi]);
                    side = (scr2 * d0[bi] < -fabs(absq - d0[bi]) * scr2) ? 1 : 0;
                }
                sc.dt0_side = side;
            }
        }
        for (int i = tid; i < n; i += NT) rtau[i] = en(i) ? *dt * d0[i] / ys[i] : 0.0;
        const double* qprev = q0;
        const double* dprev = d0;
        double tn = ts;
        for (int at = 0;; ++at) {
            if (at >= kQaMaxAttempts) return -33;
            const double dta = *dt;
            if (tid == 0) sc.dt[at] = dta;
            double* rtaus = at_rtaus(at);
            if (at == 0) {
                for (int i = tid; i < n; i += NT) rtaus[i] = rtau[i];
            } else {
                const double ratio = dta / sc.dt[at - 1];
                const double* prev = at_rtaus(at - 1);
                for (int i = tid; i < n; i += NT) rtaus[i] = prev[i] * ratio;
            }
            const double rdt = 1.0 / dta;
            double* scr = at_scrp(at);
            for (int i = tid; i < n; i += NT) {
                const double r = rtau[i];
                const double den = pade_den(r);
                scr[i] = ((qprev[i] - dprev[i]) * den) / (den + pade_num(r));
            }
            for (int j = 0; j < I; ++j) {
                double* yj = at_y(at, j);
                for (int i = tid; i < n; i += NT) yj[i] = dmaxr(ymin(i), fma(dta, scr[i], ys[i]));
                if (j == 0) tn = ts + dta;
                double *qj = at_q(at, j), *dj = at_d(at, j), *sj = at_scr(at, j);
                eval(tn + tstart, yj, qj, dj, true, keep ? sv_slot(1 + at * I + j) : nullptr);
                for (int i = tid; i < n; i += NT) {
                    const double rb = en(i) ? 0.5 * (rtaus[i] + dta * dj[i] / yj[i]) : 0.0;
                    const double an = pade_an(rb), ad = pade_den(rb);
                    const double num = fma(q0[i], ad - an, qj[i] * an) - ((ys[i] * rb) * ad) * rdt;
                    sj[i] = num / fma(an, rb, ad);
                }
                scr = sj;
            }
            const double* qL = at_q(at, I - 1);
            const double* dL = at_d(at, I - 1);
            const double* y1 = at_y(at, 0);
            double* raw = at_raw(at);
            double* yf = at_yf(at);
            double best = 1e-10;
            int bi = -1;
            for (int i = tid; i < n; i += NT) {
                double scr2 = fma(dta, scr[i], ys[i]);
                raw[i] = scr2;
                if (en(i)) scr2 = dmaxr(scr2, ymin(i));
                double scr1 = fabs(scr2 - y1[i]);
                const double yi = dmaxr(scr2, ymin(i));
                yf[i] = yi;
                if (fabs(yi) > a->qss_abstol && 0.25 * (ys[i] + yi) > ymin(i)) {
                    scr1 = scr1 / yi;
                    const double el =
                        .5 * (scr1 + dminr(fabs(qL[i] - dL[i]) / (qL[i] + dL[i] + 1e-30), scr1));
                    if (!(el < best)) {
                        best = el;
                        bi = i;
                    }
                }
            }
            block_argmax<NT>(w.red, ired, best, bi);
            const double eps = best / a->qss_epsmin;
            if (tid == 0) {
                sc.eps[at] = eps;
                sc.imax[at] = bi;
                int br = 0;
                if (bi >= 0) {
                    double scr2 = raw[bi];
                    if (en(bi)) scr2 = dmaxr(scr2, ymin(bi));
                    const double scr1 = fabs(scr2 - y1[bi]) / yf[bi];
                    const double g = fabs(qL[bi] - dL[bi]) / (qL[bi] + dL[bi] + 1e-30);
                    br = (scr1 < g) ? 0 : 1;
                }
                sc.ebr[at] = br;
            }
            if (dta <= a->qss_dtmin + 1e-16 * tn) return -1;
            const bool accepted = eps <= a->qss_epsmax;
            if (accepted && tf <= tn * tfd) {
                if (tid == 0) {
                    sc.A = at + 1;
                    sc.dt[at + 1] = 0.0;
                    sc.dtbr[at + 1] = -1;
                }
                for (int i = tid; i < n; i += NT) y_out[i] = yf[i];
                *tn_out = tn;
                __syncthreads();
                return 0;
            }
            if (!accepted) tn = ts;
            double rteps = 0.5 * (eps + 1.0);
            rteps = 0.5 * (rteps + eps / rteps);
            rteps = 0.5 * (rteps + eps / rteps);
            const double ca = dta * (1.0 / rteps + 0.005), cbv = tfd * (tf - tn);
            double nd = dminr(ca, cbv);
            int b = (cbv < ca) ? 1 : 0;
            if (a->qss_dtmax < nd) b = 2;
            nd = dminr(nd, a->qss_dtmax);
            *dt = nd;
            if (tid == 0) {
                sc.rteps[at] = rteps;
                sc.dtbr[at + 1] = b;
            }
            if (!accepted) {
                qprev = qL;
                dprev = dL;
                continue;
            }
            if (tid == 0) {
                sc.A = at + 1;
                sc.dt[at + 1] = nd;
            }
            for (int i = tid; i < n; i += NT) y_out[i] = yf[i];
            *tn_out = tn;
            __syncthreads();
            return 0;
        }
    }

    // Backward through the step just replayed by step_run from ys at ts.
    // yb: in, adjoint of the state after the step; out, of ys. *tsb: in, of
    // the time after the step; out, of ts. *dtb: in, of the step size handed
    // to the next step (unused for the last step); out, of the step size the
    // step started with (0 for the first step).
    __device__ void step_back(double ts, bool first, bool last, double* yb, double* tsb, double* dtb, double* pb,
                              const QaScalars& sc) {
        const int tid = threadIdx.x;
        const double tfd = 1.000008, epsmin = a->qss_epsmin;
        const int A = sc.A;
        double dtb_a[kQaMaxAttempts + 1];
        for (int at = 0; at <= A; ++at) dtb_a[at] = 0.0;
        __syncthreads();
        for (int i = tid; i < n; i += NT) {
            ysb[i] = 0.0;
            q0b[i] = 0.0;
            d0b[i] = 0.0;
            rtaub[i] = 0.0;
            qnb[i] = 0.0;
            dnb[i] = 0.0;
            rtsb[i] = 0.0;
        }
        double rrho_b = 0.0, rrc_b = 0.0, ts_b = *tsb;
        dtb_a[A - 1] += *tsb;
        if (!last) dtb_a[A] = *dtb;
        for (int at = A - 1; at >= 0; --at) {
            const double dta = sc.dt[at];
            const double* rtaus = at_rtaus(at);
            if (at < A - 1) {
                const double ratio = sc.dt[at + 1] / dta;
                double part = 0.0;
                for (int i = tid; i < n; i += NT) {
                    part += rtsb[i] * rtaus[i];
                    rtsbc[i] = rtsb[i] * ratio;
                }
                const double rb = block_add<NT>(w.red, part);
                dtb_a[at + 1] += rb / dta;
                dtb_a[at] += -rb * sc.dt[at + 1] / (dta * dta);
            } else {
                for (int i = tid; i < n; i += NT) rtsbc[i] = 0.0;
            }
            double rtepsb = 0.0;
            if (!(at == A - 1 && last)) {
                const double g = dtb_a[at + 1];
                const int b = sc.dtbr[at + 1];
                if (b == 0) {
                    const double rt = sc.rteps[at];
                    dtb_a[at] += g * (1.0 / rt + 0.005);
                    rtepsb = -g * dta / (rt * rt);
                } else if (b == 1) {
                    const double tnb = -tfd * g;
                    ts_b += tnb;
                    if (at == A - 1) dtb_a[at] += tnb;
                }
            }
            for (int j = 0; j < I; ++j)
                for (int i = tid; i < n; i += NT) yjb[size_t(j) * n + i] = 0.0;
            for (int i = tid; i < n; i += NT) {
                qjb[i] = qnb[i];
                djb[i] = dnb[i];
                yfb[i] = (at == A - 1) ? yb[i] : 0.0;
            }
            const double* qL = at_q(at, I - 1);
            const double* dL = at_d(at, I - 1);
            const double* y1 = at_y(at, 0);
            const double* raw = at_raw(at);
            const double* yf = at_yf(at);
            // eps: el of component ie -> scr1 (y1, scr2c, yf) and g (qL, dL)
            const int ie = (rtepsb != 0.0) ? sc.imax[at] : -1;
            double ub_e = 0.0;
            if (ie >= 0) {
                const double eps = sc.eps[at];
                const double r0 = 0.5 * (eps + 1.0);
                const double r1 = 0.5 * (r0 + eps / r0);
                const double r1b = 0.5 * rtepsb * (1.0 - eps / (r1 * r1));
                double epsb = 0.5 * rtepsb / r1;
                const double r0b = 0.5 * r1b * (1.0 - eps / (r0 * r0));
                epsb += 0.5 * r1b / r0 + 0.5 * r0b;
                const double elb = epsb / epsmin;
                double scr1b = elb, gb = 0.0;
                if (sc.ebr[at] != 0) {
                    scr1b = 0.5 * elb;
                    gb = 0.5 * elb;
                }
                const double scr2c = en(ie) ? dmaxr(raw[ie], ymin(ie)) : raw[ie];
                const double u = scr2c - y1[ie];
                ub_e = scr1b * rsign(u) / yf[ie];
                if ((ie % NT) == tid) {
                    yfb[ie] += -scr1b * fabs(u) / (yf[ie] * yf[ie]);
                    yjb[ie] -= ub_e;
                    const double v = qL[ie] - dL[ie], wv = qL[ie] + dL[ie] + 1e-30;
                    qjb[ie] += gb * (rsign(v) / wv - fabs(v) / (wv * wv));
                    djb[ie] += gb * (-rsign(v) / wv - fabs(v) / (wv * wv));
                }
            }
            // the state after the attempt: yf = max(scr2c, ymin), scr2c = en ? max(raw, ymin) : raw,
            // raw = ys + dt scr_last
            const double* scr_last = at_scr(at, I - 1);
            double part = 0.0;
            for (int i = tid; i < n; i += NT) {
                const double scr2c = en(i) ? dmaxr(raw[i], ymin(i)) : raw[i];
                double sb2 = (scr2c < ymin(i)) ? 0.0 : yfb[i];
                if (i == ie) sb2 += ub_e;
                const double rawb = (en(i) && raw[i] < ymin(i)) ? 0.0 : sb2;
                scrb[i] = rawb * dta;
                ysb[i] += rawb;
                part += rawb * scr_last[i];
            }
            dtb_a[at] += block_add<NT>(w.red, part);
            const double rdt = 1.0 / dta;
            for (int j = I - 1; j >= 0; --j) {
                const double* yj = at_y(at, j);
                const double* qj = at_q(at, j);
                const double* dj = at_d(at, j);
                const double* sj = at_scr(at, j);
                double* ybj = yjb + size_t(j) * n;
                double* fq = fd_q(at, j);
                double* fd = fd_d(at, j);
                part = 0.0;
                for (int i = tid; i < n; i += NT) {
                    const double rb = en(i) ? 0.5 * (rtaus[i] + dta * dj[i] / yj[i]) : 0.0;
                    const double an = pade_an(rb), ad = pade_den(rb);
                    const double den = fma(an, rb, ad);
                    const double sb = scrb[i];
                    const double nmb = sb / den;
                    const double denb = -sb * sj[i] / den;
                    const double qs = q0[i];
                    q0b[i] += nmb * (ad - an);
                    const double qjbi = qjb[i] + nmb * an;
                    ysb[i] += -nmb * rb * ad * rdt;
                    part += (-nmb * ys[i] * rb * ad) * (-rdt * rdt);
                    const double anb = nmb * (qj[i] - qs) + denb * rb;
                    const double adb = nmb * (qs - ys[i] * rb * rdt) + denb;
                    const double rbb = -nmb * ys[i] * ad * rdt + denb * an + anb * pade_an_d(rb) + adb * pade_den_d(rb);
                    double djbi = djb[i];
                    if (en(i)) {
                        rtsbc[i] += 0.5 * rbb;
                        part += 0.5 * rbb * dj[i] / yj[i];
                        djbi += 0.5 * rbb * dta / yj[i];
                        ybj[i] += -0.5 * rbb * dta * dj[i] / (yj[i] * yj[i]);
                    }
                    qjb[i] = qjbi;
                    djb[i] = djbi;
                    fq[i] = qjbi;  // kept for the temperature difference at the end of the step
                    fd[i] = djbi;
                }
                dtb_a[at] += block_add<NT>(w.red, part);
                // the corrector evaluation at yj (the predictor's T, rho, cp), from its saved values
                T = sc.T;
                rrho = sc.rrho;
                rrc = sc.rrc;
                vjp(yj, sv_slot(1 + at * I + j), qjb, djb, false, 0.0, 0.0, ybj, pb, &rrho_b, &rrc_b);
                // yj = max(ymin, ys + dt scr_{j-1})
                const double* sp = (j > 0) ? at_scr(at, j - 1) : at_scrp(at);
                part = 0.0;
                for (int i = tid; i < n; i += NT) {
                    const double rw = fma(dta, sp[i], ys[i]);
                    const double b = (ymin(i) < rw) ? ybj[i] : 0.0;
                    scrb[i] = b * dta;
                    ysb[i] += b;
                    part += b * sp[i];
                    qjb[i] = 0.0;
                    djb[i] = 0.0;
                }
                dtb_a[at] += block_add<NT>(w.red, part);
            }
            // predictor: scr_p = (qprev - dprev) den(r) / (den(r) + num(r)), r = rtau
            const double* qprev = (at == 0) ? q0 : at_q(at - 1, I - 1);
            const double* dprev = (at == 0) ? d0 : at_d(at - 1, I - 1);
            double* qpb = (at == 0) ? q0b : qnb;
            double* dpb = (at == 0) ? d0b : dnb;
            for (int i = tid; i < n; i += NT) {
                if (at > 0) {
                    qnb[i] = 0.0;
                    dnb[i] = 0.0;
                }
                const double r = rtau[i];
                const double den = pade_den(r), num = pade_num(r);
                const double P = den / (den + num);
                const double Pd = (pade_den_d(r) * num - den * pade_num_d(r)) / ((den + num) * (den + num));
                const double sb = scrb[i];
                qpb[i] += sb * P;
                dpb[i] -= sb * P;
                rtaub[i] += sb * (qprev[i] - dprev[i]) * Pd;
                if (at == 0) rtaub[i] += rtsbc[i];
                else rtsb[i] = rtsbc[i];
            }
        }
        // rtau = dt_0 d0 / ys
        const double dt0 = sc.dt[0];
        double part = 0.0;
        for (int i = tid; i < n; i += NT) {
            if (!en(i)) continue;
            d0b[i] += rtaub[i] * dt0 / ys[i];
            ysb[i] += -rtaub[i] * dt0 * d0[i] / (ys[i] * ys[i]);
            part += rtaub[i] * d0[i] / ys[i];
        }
        dtb_a[0] += block_add<NT>(w.red, part);
        if (first) {
            const int i = sc.dt0_imax;
            if (sc.dt0_br == 0 && i >= 0 && (i % NT) == tid) {
                const double scb = dtb_a[0] * (-0.5 / (sc.scrtch * sc.scrtch));
                const double sg = rsign(0.1 * epsmin * fabs(q0[i]) - d0[i]);
                const double ay = fabs(1 / ys[i]);
                const double day = -rsign(ys[i]) / (ys[i] * ys[i]);
                if (sc.dt0_side == 0) {
                    d0b[i] += scb * ay * sg;
                    ysb[i] += scb * d0[i] * sg * day;
                } else {
                    const double u = fabs(q0[i]) - d0[i];
                    const double ub = -scb * rsign(u) * ay * sg;
                    q0b[i] += ub * rsign(q0[i]);
                    d0b[i] -= ub;
                    ysb[i] += scb * (-fabs(u)) * sg * day;
                }
            }
            *dtb = 0.0;
        } else {
            *dtb = dtb_a[0];
        }
        // the predictor evaluation at ys, its rrho / rrc also used by the correctors
        T = sc.T;
        rrho = sc.rrho;
        rrc = sc.rrc;
        rho_p = sc.rho;
        cp_p = sc.cp;
        vjp(ys, sv_slot(0), q0b, d0b, true, rrho_b, rrc_b, ysb, pb, nullptr, nullptr);
        // temperature by a forward difference, every evaluation of the step at T + dT
        const double T0 = sc.T;
        const double dT = fabs(T0) * 1.4901161193847656e-08;
        double acc_part = 0.0;
        for (int at = 0; at < A; ++at)
            for (int j = 0; j < I; ++j) {
                T = T0 + dT;
                rrho = sc.rrho;
                rrc = sc.rrc;
                eval(ts + sc.dt[at] + tstart, at_y(at, j), q2, d2, true);
                const double *qj = at_q(at, j), *dj = at_d(at, j), *fq = fd_q(at, j), *fd = fd_d(at, j);
                for (int i = tid; i < n; i += NT) acc_part += fq[i] * (q2[i] - qj[i]) + fd[i] * (d2[i] - dj[i]);
            }
        for (int i = tid; i < n; i += NT) ycp[i] = (i == 1) ? T0 + dT : ys[i];
        eval(ts + tstart, ycp, q2, d2, false);
        for (int i = tid; i < n; i += NT) acc_part += q0b[i] * (q2[i] - q0[i]) + d0b[i] * (d2[i] - d0[i]);
        const double acc = block_add<NT>(w.red, acc_part) + rrho_b * (rrho - sc.rrho) + rrc_b * (rrc - sc.rrc);
        const double rdT = 1.0 / ((T0 + dT) - T0);
        for (int i = tid; i < n; i += NT) yb[i] = ysb[i] + (i == 1 ? acc * rdT : 0.0);
        *tsb = ts_b;
        __syncthreads();
    }
};

// Per point: the step starts from the forward kernel's tape (a.tape, when it
// holds the whole integration), or else from this kernel's own forward
// integration with a per-CTA tape; then the backward pass. fwd_status: the
// forward kernel's status per point (with a.tape). status: the integrator's
// (0, -1 dtmin, -20 max_steps), -30 (tape full), -33 (attempt cap).
template <int NT>
__global__ void __launch_bounds__(NT) k_source_qss_adjoint(const __grid_constant__ MechView m,
                                                            const __grid_constant__ SourceArgs a, int* counter,
                                                            double* kcache, double* work, size_t work_stride,
                                                            double* tape, int tape_cap, const int* fwd_status,
                                                            const double* ybar_out, double* ybar_in, double* pbar,
                                                            int* adj_status) {
    extern __shared__ double smem[];
    __shared__ int next_point;
    __shared__ int ired[kMaxChemThreads / 32];
    __shared__ QaScalars sc;
    const int tid = threadIdx.x;
    const int n = m.S + 2;
    QaPoint<NT> P(m);
    const size_t cd = ChemSmem::doubles(m.S, m.R, m.n_tb, m.n_fo, false);
    P.w.carve(smem, kcache + size_t(blockIdx.x) * ChemSmem::global_doubles(m), m, false);
    P.w.fo_F = smem + cd;
    P.w.fo_pr = P.w.fo_F + m.n_fo;
    P.w.fo_dF = P.w.fo_pr + m.n_fo;
    P.wqb = P.w.fo_dF + m.n_fo;
    P.wdb = P.wqb + m.S;
    P.cb = P.wdb + m.S;
    P.ired = ired;
    P.a = &a;
    P.n = n;
    P.S = m.S;
    P.I = a.qss_itermax;
    P.cachedT = __longlong_as_double(0x7ff8000000000000LL);
    double* wk = work + size_t(blockIdx.x) * work_stride;
    P.carve_work(wk);
    double* y = P.djb + n;       // the two vectors after the named ones
    double* yb = y + n;
    double* tp = tape + size_t(blockIdx.x) * size_t(tape_cap) * (n + 2);
    const double tfd = 1.000008;
    P.tstart = a.t_start_dev ? *a.t_start_dev : a.t_start;
    for (;;) {
        if (tid == 0) {
            const int slot = atomicAdd(counter, 1);
            next_point = slot < a.n ? slot : a.n;
        }
        __syncthreads();
        const int j = next_point;
        __syncthreads();
        if (j >= a.n) break;
        P.split = a.split ? a.split + size_t(j) * n : nullptr;
        P.x = a.x ? a.x[j] : 0.0;
        P.tf = a.dt[j];
        const double* yin = a.state_in + size_t(j) * n;
        int N = 0, status = 0;
        const double* recs = tp;  // step records: (time, step size, state) each
        bool have_tape = false;
        if (a.tape) {
            const double* hdr = a.tape + size_t(j) * a.tape_stride;
            status = fwd_status ? fwd_status[j] : 0;
            if (status == 0 && hdr[1] == 0.0) {
                have_tape = true;
                N = static_cast<int>(hdr[0]);
                recs = hdr + kQssTapeHeader;
            }
        }
        for (int i = tid; i < n; i += NT) y[i] = P.en(i) ? dmaxr(yin[i], P.ymin(i)) : yin[i];
        __syncthreads();
        // forward, keeping each step's start (state, time, step size)
        double tn = 0.0, dt = 0.0;
        while (!have_tape && status == 0 && tfd * tn < P.tf) {
            if (N >= a.max_steps) {
                status = -20;
                break;
            }
            if (N >= tape_cap) {
                status = -30;
                break;
            }
            double* rec = tp + size_t(N) * (n + 2);
            for (int i = tid; i < n; i += NT) rec[2 + i] = y[i];
            if (tid == 0) {
                rec[0] = tn;
                rec[1] = dt;
            }
            double tnew = tn;
            const int r = P.step_run(y, tn, N == 0, &dt, &tnew, yb, sc, false);
            ++N;
            if (r != 0) {
                status = r;
                break;
            }
            tn = tnew;
            for (int i = tid; i < n; i += NT) y[i] = yb[i];
            __syncthreads();
        }
        if (!have_tape) {
            int nonfinite = 0;
            double* yout = a.state_out + size_t(j) * n;
            for (int i = tid; i < n; i += NT) {
                nonfinite |= !isfinite(y[i]);
                yout[i] = y[i];
            }
            nonfinite = __syncthreads_or(nonfinite);
            if (status == 0 && nonfinite) status = -21;
        }
        double* pb = pbar + size_t(j) * m.R;
        for (int i = tid; i < m.R; i += NT) pb[i] = 0.0;
        if (status == 0) {
            for (int i = tid; i < n; i += NT) yb[i] = ybar_out[size_t(j) * n + i];
            double tsb = 0.0, dtb = 0.0;
            __syncthreads();
            for (int k = N - 1; k >= 0 && status == 0; --k) {
                const double* rec = recs + size_t(k) * (n + 2);
                double dtk = rec[1], tk = 0.0;
                const int r = P.step_run(rec + 2, rec[0], k == 0, &dtk, &tk, y, sc, true);
                if (r != 0) {
                    status = r;
                    break;
                }
                __syncthreads();
                P.step_back(rec[0], k == 0, k == N - 1, yb, &tsb, &dtb, pb, sc);
            }
        }
        for (int i = tid; i < n; i += NT)
            ybar_in[size_t(j) * n + i] = (status == 0 && !(P.en(i) && yin[i] < P.ymin(i))) ? yb[i] : 0.0;
        if (tid == 0) {
            adj_status[j] = status;
            if (a.status && !a.tape) a.status[j] = status;
            if (a.stats && !a.tape) {
                a.stats[4 * size_t(j) + 0] = N;
                a.stats[4 * size_t(j) + 1] = 0;
                a.stats[4 * size_t(j) + 2] = 0;
                a.stats[4 * size_t(j) + 3] = 0;
            }
        }
        __syncthreads();
    }
}

template <int NT>
int launch_qss_adjoint_nt(const MechView& m, const SourceArgs& a, int tape_cap, int* counter, const int* fwd_status,
                          const double* ybar_out, double* ybar_in, double* pbar, int* adj_status, Scratch& scr,
                          cudaStream_t st) {
    const int n = m.S + 2;
    const size_t per = sizeof(double) * (ChemSmem::doubles(m.S, m.R, m.n_tb, m.n_fo, false) + 3 * size_t(m.n_fo) +
                                         3 * size_t(m.S));
    EMBER_CHECK_ARG(per <= 200 * 1024, "mechanism too large for the QSS adjoint's shared-memory work area");
    EMBER_TRY(raise_dynamic_smem(reinterpret_cast<const void*>(k_source_qss_adjoint<NT>), per));
    int dev = 0, sms = 0, per_sm = 0;
    EMBER_CUDA_TRY(cudaGetDevice(&dev));
    EMBER_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    EMBER_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_source_qss_adjoint<NT>, NT, per));
    per_sm = std::max(1, std::min(per_sm, 4));
    const int blocks = std::max(1, std::min(a.n, sms * per_sm));
    const size_t wstride = QaPoint<NT>::work_doubles(m, a.qss_itermax);
    // the per-CTA tape of points integrated again here (no forward tape, or
    // one that overflowed): at least 4096 step starts
    const int cta_cap = std::max(tape_cap, 4096);
    double *kcache = nullptr, *work = nullptr, *tape = nullptr;
    EMBER_TRY(scr.alloc(&kcache, size_t(blocks) * ChemSmem::global_doubles(m)));
    EMBER_TRY(scr.alloc(&work, size_t(blocks) * wstride));
    EMBER_TRY(scr.alloc(&tape, size_t(blocks) * size_t(cta_cap) * (n + 2)));
    k_source_qss_adjoint<NT><<<blocks, NT, per, st>>>(m, a, counter, kcache, work, wstride, tape, cta_cap,
                                                      fwd_status, ybar_out, ybar_in, pbar, adj_status);
    EMBER_CUDA_TRY(cudaGetLastError());
    return EMBER_OK;
}

__global__ void k_sum_point_rows(int n, int R, const double* __restrict__ rows, double* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < R; i += gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int j = 0; j < n; ++j) s += rows[size_t(j) * R + i];
        out[i] = s;
    }
}

}  // namespace

int launch_source_qss_adjoint(const MechView& m, const SourceArgs& a, int tape_cap, int* counter,
                              const int* fwd_status, const double* ybar_out, double* ybar_in, double* pbar,
                              int* adj_status, Scratch& sc, cudaStream_t st) {
    EMBER_CHECK_ARG(a.qss_stability_check == 0, "the QSS adjoint needs qss_stability_check = 0");
    EMBER_CHECK_ARG(a.qss_itermax >= 1 && a.qss_itermax <= kQaMaxIter, "the QSS adjoint supports 1-%d iterations",
                    kQaMaxIter);
    EMBER_CHECK_ARG(tape_cap >= 1, "bad tape_cap %d", tape_cap);
    if (m.S + 2 <= 64)
        return launch_qss_adjoint_nt<64>(m, a, tape_cap, counter, fwd_status, ybar_out, ybar_in, pbar, adj_status,
                                         sc, st);
    return launch_qss_adjoint_nt<128>(m, a, tape_cap, counter, fwd_status, ybar_out, ybar_in, pbar, adj_status, sc,
                                      st);
}

size_t qss_tape_doubles(const MechView& m, int n_points, int tape_cap) {
    return size_t(n_points) * (kQssTapeHeader + size_t(tape_cap) * (m.S + 4));
}

int source_qss_adjoint_run(const MechView& m, const SourceArgs& a_in, int tape_cap, const double* ybar_out,
                           double* ybar_in, double* lnk_bar, double* lnk_bar_points, int* adj_status, Scratch& sc,
                           cudaStream_t st) {
    SourceArgs a = a_in;
    int* counter = nullptr;
    EMBER_TRY(sc.alloc(&counter, 1));
    EMBER_CUDA_TRY(cudaMemsetAsync(counter, 0, sizeof(int), st));
    double* rows = lnk_bar_points;
    if (!rows) EMBER_TRY(sc.alloc(&rows, size_t(a.n) * std::max(m.R, 1)));
    // With room for a whole tape, the forward kernel records every step start
    // and the adjoint does not integrate again.
    if (qss_tape_doubles(m, a.n, tape_cap) * sizeof(double) <= kQssTapeBudgetBytes) {
        a.tape_cap = tape_cap;
        a.tape_stride = int64_t(kQssTapeHeader) + int64_t(tape_cap) * (m.S + 4);
        EMBER_TRY(sc.alloc(&a.tape, qss_tape_doubles(m, a.n, tape_cap)));
        int* fcounter = nullptr;
        EMBER_TRY(sc.alloc(&fcounter, 1));
        EMBER_CUDA_TRY(cudaMemsetAsync(fcounter, 0, sizeof(int), st));
        EMBER_TRY(launch_source_qss(m, a, fcounter, sc, st));
        EMBER_TRY(launch_source_qss_adjoint(m, a, tape_cap, counter, a.status, ybar_out, ybar_in, rows, adj_status,
                                            sc, st));
    } else {
        a.tape = nullptr;
        EMBER_TRY(launch_source_qss_adjoint(m, a, tape_cap, counter, nullptr, ybar_out, ybar_in, rows, adj_status, sc,
                                            st));
    }
    if (lnk_bar && m.R > 0) k_sum_point_rows<<<blocks_for(m.R, 128), 128, 0, st>>>(a.n, m.R, rows, lnk_bar);
    EMBER_CUDA_TRY(cudaGetLastError());
    return EMBER_OK;
}

}  // namespace ember

using namespace ember;

extern "C" int ember_source_adjoint_qss(ember_mech m, int n, const double* state_in, const double* split_const,
                                        const double* dt, double t_start, const double* x,
                                        const ember_source_options* opts, const double* state_bar, int tape_cap,
                                        double* state_out, int* status, double* state_in_bar, double* lnk_bar,
                                        int mem, void* stream) {
    EMBER_CHECK_ARG(m != nullptr, "null mechanism");
    EMBER_CHECK_ARG(n > 0 && state_in && dt && state_bar && state_out && status && state_in_bar,
                    "need points, state_in, dt, state_bar, state_out, status and state_in_bar");
    EMBER_CHECK_ARG(mem == EMBER_MEM_HOST || mem == EMBER_MEM_DEVICE, "bad mem flag %d", mem);
    EMBER_CHECK_ARG(tape_cap >= 0 && tape_cap <= (1 << 22), "bad tape_cap %d", tape_cap);
    EMBER_TRY(source_check_options(opts));
    EMBER_CHECK_ARG(opts == nullptr || opts->qss_stability_check == 0, "the QSS adjoint needs qss_stability_check = 0");
    EMBER_TRY(ensure_device());
    if (tape_cap == 0) tape_cap = 4096;
    cudaStream_t st = as_stream(stream);
    Scratch sc(st);
    const int nv = m->S + 2;
    const double *d_in, *d_split, *d_dt, *d_x, *d_bar;
    EMBER_TRY(stage_in(sc, state_in, size_t(n) * nv, mem, st, &d_in));
    EMBER_TRY(stage_in(sc, split_const, size_t(n) * nv, mem, st, &d_split));
    EMBER_TRY(stage_in(sc, dt, n, mem, st, &d_dt));
    EMBER_TRY(stage_in(sc, x, n, mem, st, &d_x));
    EMBER_TRY(stage_in(sc, state_bar, size_t(n) * nv, mem, st, &d_bar));
    double *d_out, *d_inbar, *d_lnk = nullptr;
    int *d_status, *d_adj;
    EMBER_TRY(stage_buffer(sc, state_out, size_t(n) * nv, mem, &d_out));
    EMBER_TRY(stage_buffer(sc, status, n, mem, &d_status));
    EMBER_TRY(stage_buffer(sc, state_in_bar, size_t(n) * nv, mem, &d_inbar));
    EMBER_TRY(stage_buffer(sc, lnk_bar, size_t(std::max(m->R, 1)), mem, &d_lnk));
    EMBER_TRY(sc.alloc(&d_adj, n));
    SourceArgs a = make_source_args(opts, n, d_in, d_split, d_dt, t_start, d_x, d_out, d_status, nullptr);
    EMBER_TRY(source_qss_adjoint_run(m->view, a, tape_cap, d_bar, d_inbar, d_lnk, nullptr, d_adj, sc, st));
    // status: the forward's, or the adjoint's when the forward succeeded
    EMBER_CUDA_TRY(cudaMemcpyAsync(d_status, d_adj, sizeof(int) * n, cudaMemcpyDeviceToDevice, st));
    EMBER_TRY(stage_out(state_out, d_out, size_t(n) * nv, mem, st));
    EMBER_TRY(stage_out(status, d_status, n, mem, st));
    EMBER_TRY(stage_out(state_in_bar, d_inbar, size_t(n) * nv, mem, st));
    if (lnk_bar) EMBER_TRY(stage_out(lnk_bar, d_lnk, size_t(m->R), mem, st));
    sc.release();
    EMBER_TRY(finish_call(mem, st));
    if (mem == EMBER_MEM_HOST) {
        int bad = 0;
        for (int j = 0; j < n; ++j) bad += status[j] != 0;
        if (bad) {
            set_error("%d of %d points failed (see status)", bad, n);
            return EMBER_EFAIL;
        }
    }
    return EMBER_OK;
}
