/*
 * CPU ORACLE -- test infrastructure only (see oracle_tridiag.c).
 *
 * Discrete adjoint of the QSS source-term integration of one point
 * (SourceSystemQSS + QssIntegrator, src/sourceSystem.cpp:403-531,
 * src/qssintegrator.cpp:58-265), the CPU check of the device adjoint. The
 * reference runs the integrator forward only; this file differentiates the
 * forward map of oracle_chem.c exactly as it is computed:
 *
 *   every accepted and every rejected attempt of every step, because a
 *   retried attempt's predictor uses the q and d of the rejected attempt's
 *   last corrector evaluation;
 *   the step sizes, as functions of the state: the initial step size of
 *   getInitialStepSize, and each new step size from the error estimate eps
 *   (dt (1/sqrt(eps) + 0.005), with the two Newton iterations for the square
 *   root, or tfd (tf - t) or dtmax, whichever the forward pass took);
 *   rtaus = rtau dt_a / dt_0 after a rejection;
 *   every min / max / abs by the branch the forward pass took;
 *   the right-hand side's frozen quantities: a corrector evaluation uses the
 *   predictor's T (rate constants, h_k, the density's temperature), rho and
 *   cp, so its adjoint flows back to the predictor's state.
 * The accept / reject decisions, the number of steps and the set of
 * components in each max are held fixed (a finite-difference quotient that
 * straddles a change of one of them measures a jump, not a derivative).
 * The right-hand side's dependence on the mass fractions is differentiated
 * analytically (rates of progress, third-body concentrations, falloff
 * blending, the normalisation of setState_TPY); its dependence on T
 * (rate constants, reverse factors, thermo) by a forward difference with
 * the step sqrt(eps) |T|, as the BDF adjoint's temperature column.
 *
 * The gradient with respect to ln(multiplier_i) uses d ropf_i / d ln m_i =
 * ropf_i and d ropr_i / d ln m_i = ropr_i. The igniter term depends on time
 * only (piecewise constant in the step sizes). Requires qss_stability_check
 * = 0 (the reference's default); the reference's default iteration count 1
 * and any other count are covered.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

#define GAS_CONSTANT (6.02214076e26 * 1.380649e-23)
#define SMALL_NUMBER 1e-300
#define QA_MAX_ATTEMPTS 64
#define QA_MAX_ITER 8

static double dmax(double a, double b) { return (a < b) ? b : a; } /* std::max */
static double dmin(double a, double b) { return (b < a) ? b : a; } /* std::min */
static double rsign(double x) { return (x > 0) ? 1.0 : (x < 0) ? -1.0 : 0.0; }
static double pade_num(double r) { return r * fma(r, fma(r, 11.0 + r, 60.0), 180.0); }
static double pade_den(double r) { return fma(r, fma(r, 12.0 + r, 60.0), 360.0); }
static double pade_an(double r) { return fma(r, fma(r, 11.0 + r, 60.0), 180.0); }
/* derivatives of the three polynomials */
static double pade_num_d(double r) { return fma(r, fma(r, fma(4.0, r, 33.0), 120.0), 180.0); }
static double pade_den_d(double r) { return fma(r, fma(3.0, r, 24.0), 60.0); }
static double pade_an_d(double r) { return fma(r, fma(3.0, r, 22.0), 60.0); }

static double igniter(const oracle_source_options* o, double t, double x) {
    if (o->ignition_energy != 0.0 && t >= o->ignition_tstart && t < o->ignition_tstart + o->ignition_duration) {
        const double pi = 3.14159265358979323846;
        const double dx = x - o->ignition_center;
        return o->ignition_energy / (o->ignition_stddev * sqrt(2 * pi) * o->ignition_duration) *
               oracle_exp(-(dx * dx) / (2 * (o->ignition_stddev * o->ignition_stddev)));
    }
    return 0.0;
}

/* ---- the right-hand side and its adjoint ------------------------------- */

typedef struct {
    const oracle_mech* m;
    const oracle_source_options* o;
    oracle_ws* w;
    const double* split;
    double x;
    double T;               /* predictor's temperature (frozen in corrector calls) */
    double rrho, rrc;       /* predictor's 1/rho, 1/(rho cp) */
    double rho_p, cp_p;     /* predictor's rho, cp */
    double qdot;            /* of the last evaluation */
    double rho_c;           /* density of the last evaluation's composition */
} qa_ode;

/* SourceSystemQSS::odefun, the operations of oracle_chem.c's qss_odefun. */
static void qa_eval(qa_ode* e, double t, const double* y, double* q, double* d, int corrector) {
    const oracle_mech* m = e->m;
    oracle_ws* w = e->w;
    const int S = m->S;
    if (!corrector) e->T = y[1];
    double rho, cp;
    oracle_rates(m, w, e->o->pressure, e->o->kinetics_model, ORACLE_STATE_NORMALIZED, e->T, y + 2, &rho, &cp);
    if (!corrector) {
        e->rrho = 1.0 / rho;
        e->rrc = 1.0 / (rho * cp);
        e->rho_p = rho;
        e->cp_p = cp;
    }
    e->rho_c = rho;
    for (int k = 0; k < S; ++k) w->tmp[k] = w->wq[k] - w->wd[k];
    const double qdot =
        -oracle_block_sum(w->tmp, w->hk, S, oracle_reduction_width(S)) + igniter(e->o, t, e->x);
    e->qdot = qdot;
    const double* sc = e->split;
    q[0] = sc ? sc[0] : 0.0;
    d[0] = 0.0;
    q[1] = fma(qdot, e->rrc, sc ? sc[1] : 0.0);
    d[1] = 0.0 * e->rrc;
    for (int k = 0; k < S; ++k) {
        q[2 + k] = fma(w->wq[k] * m->W[k], e->rrho, sc ? sc[2 + k] : 0.0);
        d[2 + k] = (w->wd[k] * m->W[k]) * e->rrho;
    }
}

static double arrh(const double* p, double lnT, double rT) {
    return p[0] * oracle_exp(fma(p[1], lnT, -(p[2] * rT)));
}

/* Adjoint of an evaluation at fixed T, with w holding that evaluation's
 * intermediates (qa_eval just called on Y = y + 2). qb, db: adjoints of q, d.
 * Accumulates the mass-fraction adjoints into Yb[S] and the multiplier
 * adjoints into pb[R]; returns the adjoints of the rrho / rrc the
 * evaluation used (*rrho_b, *rrc_b, accumulated). For a predictor call,
 * rho_b_in / cp_b_in are adjoints of the evaluation's own rho and cp
 * (through the predictor's rrho, rrc), 0 for a corrector call. */
static void qa_vjp(qa_ode* e, const double* Y, const double* qb, const double* db, double rho_b_in, double cp_b_in,
                   double* Yb, double* pb, double* rrho_b, double* rrc_b, double* scratch) {
    const oracle_mech* m = e->m;
    oracle_ws* w = e->w;
    const int S = m->S, R = m->R;
    double* wqb = scratch;          /* S */
    double* wdb = wqb + S;          /* S */
    double* cb = wdb + S;           /* S */
    double* ymb = cb + S;           /* S */
    const double qdb = qb[1] * e->rrc;
    double rb = 0.0;
    for (int k = 0; k < S; ++k) {
        wqb[k] = qb[2 + k] * m->W[k] * e->rrho - qdb * w->hk[k];
        wdb[k] = db[2 + k] * m->W[k] * e->rrho + qdb * w->hk[k];
        rb += qb[2 + k] * w->wq[k] * m->W[k] + db[2 + k] * w->wd[k] * m->W[k];
        cb[k] = 0.0;
    }
    *rrho_b += rb;
    *rrc_b += qb[1] * e->qdot;
    double ctotb = 0.0;
    const double T = e->T, lnT = oracle_log(T), rT = 1.0 / T;
    for (int i = 0; i < R; ++i) {
        const int* rc = m->reac + i * ORACLE_MAX_STOICH;
        const int* pr = m->prod + i * ORACLE_MAX_STOICH;
        double fb = 0.0, rbb = 0.0;
        for (int o = 0; o < ORACLE_MAX_STOICH; ++o) {
            if (pr[o] >= 0) { fb += wqb[pr[o]]; rbb += wdb[pr[o]]; }
            if (rc[o] >= 0) { fb += wdb[rc[o]]; rbb += wqb[rc[o]]; }
        }
        pb[i] += fb * w->ropf[i] + rbb * w->ropr[i];
        const int ty = m->type[i];
        const double kfm = (ty == ORACLE_RXN_LINDEMANN || ty == ORACLE_RXN_TROE ? w->kf_fall[i] : w->kf[i]) * m->mult[i];
        double rf = kfm;
        if (ty == ORACLE_RXN_THREE_BODY) rf *= w->concm[i];
        const double kr = m->rev[i] ? w->rkc[i] : 0.0;
        double pf = 1.0, pp = 1.0;
        for (int o = 0; o < ORACLE_MAX_STOICH; ++o) {
            if (rc[o] >= 0) pf *= w->c[rc[o]];
            if (pr[o] >= 0) pp *= w->c[pr[o]];
        }
        for (int o = 0; o < ORACLE_MAX_STOICH; ++o) {
            if (rc[o] < 0) continue;
            double dv = rf;
            for (int q2 = 0; q2 < ORACLE_MAX_STOICH; ++q2)
                if (q2 != o && rc[q2] >= 0) dv *= w->c[rc[q2]];
            cb[rc[o]] += fb * dv;
        }
        if (m->rev[i]) {
            for (int o = 0; o < ORACLE_MAX_STOICH; ++o) {
                if (pr[o] < 0) continue;
                double dv = rf * kr;
                for (int q2 = 0; q2 < ORACLE_MAX_STOICH; ++q2)
                    if (q2 != o && pr[q2] >= 0) dv *= w->c[pr[q2]];
                cb[pr[o]] += rbb * dv;
            }
        }
        double Mb = 0.0;
        if (ty == ORACLE_RXN_THREE_BODY) {
            Mb = fb * (kfm * pf) + rbb * (kfm * kr * pp);
        } else if (ty == ORACLE_RXN_LINDEMANN || ty == ORACLE_RXN_TROE) {
            const double kinf = arrh(m->arr + 3 * i, lnT, rT);
            const double rkinf = 1.0 / (kinf + SMALL_NUMBER);
            const double prr = w->pr_fall[i], pr1 = 1.0 + prr;
            const double dkdm = (w->F_fall[i] / (pr1 * pr1) + (prr / pr1) * w->dF_fall[i]) *
                                (w->k0_fall[i] * rkinf) * kinf * m->mult[i];
            Mb = (fb * pf + rbb * kr * pp) * dkdm;
        }
        if (ty != ORACLE_RXN_ELEMENTARY) {
            const double de = m->def_eff[i];
            ctotb += Mb * de;
            for (int64_t q2 = m->eff_off[i]; q2 < m->eff_off[i + 1]; ++q2)
                cb[m->eff_sp[q2]] += Mb * (m->eff_val[q2] - de);
        }
    }
    /* c_k = ym_k rho, ctot = rho / mmw; predictor: rrho = 1/rho, rrc = 1/(rho cp),
     * cp = R cpsum / mmw, cpsum = sum ym_k mmw cpR_k; rho = p mmw / (R T);
     * mmw = 1 / sum ym; ym_k = max(Y_k, 0) rnorm / W_k, rnorm = 1 / sum max(Y, 0) */
    const double rho = e->rho_c, mmw = w->mmw;
    double rhob = rho_b_in + ctotb / mmw;
    double mmwb = -ctotb * rho / (mmw * mmw);
    for (int k = 0; k < S; ++k) {
        ymb[k] = cb[k] * rho;
        rhob += cb[k] * w->ym[k];
    }
    if (cp_b_in != 0.0) {
        double cpsum = 0.0, ycp = 0.0;
        for (int k = 0; k < S; ++k) {
            cpsum += w->ym[k] * mmw * w->cp_R[k];
            ycp += w->ym[k] * w->cp_R[k];
        }
        const double cpsb = cp_b_in * GAS_CONSTANT / mmw;
        mmwb += -cp_b_in * GAS_CONSTANT * cpsum / (mmw * mmw) + cpsb * ycp;
        for (int k = 0; k < S; ++k) ymb[k] += cpsb * mmw * w->cp_R[k];
    }
    mmwb += rhob * e->o->pressure / (GAS_CONSTANT * T);
    double yp_sum = 0.0;
    for (int k = 0; k < S; ++k) {
        ymb[k] += -mmwb * mmw * mmw;
        yp_sum += dmax(Y[k], 0.0);
    }
    const double rnorm = 1.0 / yp_sum;
    double rnb = 0.0;
    for (int k = 0; k < S; ++k) rnb += ymb[k] * dmax(Y[k], 0.0) * m->rW[k];
    for (int k = 0; k < S; ++k)
        if (Y[k] > 0.0) Yb[k] += ymb[k] * rnorm * m->rW[k] - rnb * rnorm * rnorm;
}

/* ---- one integrateOneStep, replayed ---------------------------------- */

typedef struct {
    int n, itermax, A;
    double dt[QA_MAX_ATTEMPTS + 1];    /* dt of each attempt; dt[A]: the next step's (if any) */
    double *q0, *d0, *rtau, *ys;       /* predictor call */
    double* buf;                       /* per attempt: rtaus, scr_p, then per iteration y, q, d, scr; then scr2, yfin */
    double eps[QA_MAX_ATTEMPTS], rteps[QA_MAX_ATTEMPTS];
    int imax[QA_MAX_ATTEMPTS], epsmin_branch[QA_MAX_ATTEMPTS];
    int dt_branch[QA_MAX_ATTEMPTS + 1];  /* 0: dt (1/rteps + .005), 1: tfd (tf - t), 2: dtmax */
    int dt0_branch, dt0_imax, dt0_side;  /* initial step: 0 scrtch, 1 tf, 2 dtmax; argmax; 0 scr1, 1 other */
    double scrtch;
    double rrho, rrc, rho, cp, T;
} qa_step;

static size_t qa_att_doubles(int n, int I) { return (size_t)n * (2 + 4 * I + 2); }
static double* att_rtaus(qa_step* s, int a) { return s->buf + qa_att_doubles(s->n, s->itermax) * a; }
static double* att_scrp(qa_step* s, int a) { return att_rtaus(s, a) + s->n; }
static double* att_y(qa_step* s, int a, int j) { return att_rtaus(s, a) + (size_t)s->n * (2 + 4 * j); }
static double* att_q(qa_step* s, int a, int j) { return att_y(s, a, j) + s->n; }
static double* att_d(qa_step* s, int a, int j) { return att_y(s, a, j) + 2 * s->n; }
static double* att_scr(qa_step* s, int a, int j) { return att_y(s, a, j) + 3 * s->n; }
static double* att_scr2(qa_step* s, int a) { return att_rtaus(s, a) + (size_t)s->n * (2 + 4 * s->itermax); }
static double* att_yfin(qa_step* s, int a) { return att_scr2(s, a) + s->n; }

typedef struct {
    int n;
    const double *ymin;
    const int* en;
    oracle_qss_params P;
    double tf, tstart, tfd;
} qa_ctx;

/* integrateOneStep from ys at ts with step *dt (first: the initial step is
 * computed), exactly as oracle_chem.c's qss_one_step, recording what the
 * adjoint needs into s. y: out, the state after the step. Returns 0 (done,
 * *tn, *dt updated) or -1 (dtmin), -33 (attempt cap). */
static int qa_step_run(qa_ode* e, const qa_ctx* c, qa_step* s, const double* ys, double ts, int first, double* dt,
                       double* tn_out, double* y) {
    const int n = c->n;
    const int* en = c->en;
    const double* ymin = c->ymin;
    const oracle_qss_params* o = &c->P;
    const double tf = c->tf;
    memcpy(s->ys, ys, sizeof(double) * n);
    qa_eval(e, ts + c->tstart, ys, s->q0, s->d0, 0);
    s->rrho = e->rrho; s->rrc = e->rrc; s->rho = e->rho_p; s->cp = e->cp_p; s->T = e->T;
    if (first) {
        double scrtch = 1.0e-25;
        int im = -1, side = 0;
        for (int i = 0; i < n; ++i) {
            if (fabs(ys[i]) > o->abstol) {
                const double absq = fabs(s->q0[i]);
                const double scr2 = fabs(1 / ys[i]) * rsign(0.1 * o->epsmin * absq - s->d0[i]);
                const double scr1 = scr2 * s->d0[i];
                const double other = -fabs(absq - s->d0[i]) * scr2;
                const double mx = dmax(scr1, other);
                if (!(mx < scrtch)) { /* dmax(mx, scrtch) takes mx */
                    scrtch = mx;
                    im = i;
                    side = (scr1 < other) ? 1 : 0;
                }
            }
        }
        s->scrtch = scrtch;
        s->dt0_imax = im;
        s->dt0_side = side;
        double d0 = dmin(0.5 / scrtch, tf);
        s->dt0_branch = (tf < 0.5 / scrtch) ? 1 : 0;
        if (o->dtmax < d0) s->dt0_branch = 2;
        *dt = dmin(d0, o->dtmax);
    }
    for (int i = 0; i < n; ++i) s->rtau[i] = en[i] ? *dt * s->d0[i] / ys[i] : 0.0;
    const double* qprev = s->q0;
    const double* dprev = s->d0;
    double tn = ts;
    int a = 0;
    for (;;) {
        if (a >= QA_MAX_ATTEMPTS) return -33;
        s->dt[a] = *dt;
        const double dta = *dt;
        double* rtaus = att_rtaus(s, a);
        if (a == 0) memcpy(rtaus, s->rtau, sizeof(double) * n);
        else {
            const double ratio = dta / s->dt[a - 1];
            const double* prev = att_rtaus(s, a - 1);
            for (int i = 0; i < n; ++i) rtaus[i] = prev[i] * ratio;
        }
        const double rdt = 1.0 / dta;
        double* scr = att_scrp(s, a);
        for (int i = 0; i < n; ++i) {
            const double r = s->rtau[i];
            const double den = pade_den(r);
            scr[i] = ((qprev[i] - dprev[i]) * den) / (den + pade_num(r));
        }
        for (int j = 0; j < o->itermax; ++j) {
            double* yj = att_y(s, a, j);
            for (int i = 0; i < n; ++i) yj[i] = dmax(ymin[i], fma(dta, scr[i], ys[i]));
            if (j == 0) tn = ts + dta;
            double *qj = att_q(s, a, j), *dj = att_d(s, a, j), *sj = att_scr(s, a, j);
            qa_eval(e, tn + c->tstart, yj, qj, dj, 1);
            for (int i = 0; i < n; ++i) {
                const double rb = en[i] ? 0.5 * (rtaus[i] + dta * dj[i] / yj[i]) : 0.0;
                const double an = pade_an(rb), ad = pade_den(rb);
                const double nm = fma(s->q0[i], ad - an, qj[i] * an) - ((ys[i] * rb) * ad) * rdt;
                sj[i] = nm / fma(an, rb, ad);
            }
            scr = sj;
        }
        const double* qL = att_q(s, a, o->itermax - 1);
        const double* dL = att_d(s, a, o->itermax - 1);
        const double* y1 = att_y(s, a, 0);
        double* scr2v = att_scr2(s, a);
        double* yf = att_yfin(s, a);
        double eps = 1e-10;
        int im = -1, br = 0;
        for (int i = 0; i < n; ++i) {
            double scr2 = fma(dta, scr[i], ys[i]);
            scr2v[i] = scr2;
            if (en[i]) scr2 = dmax(scr2, ymin[i]);
            double scr1 = fabs(scr2 - y1[i]);
            yf[i] = dmax(scr2, ymin[i]);
            if (fabs(yf[i]) > o->abstol && 0.25 * (ys[i] + yf[i]) > ymin[i]) {
                scr1 = scr1 / yf[i];
                const double g = fabs(qL[i] - dL[i]) / (qL[i] + dL[i] + 1e-30);
                const double el = .5 * (scr1 + dmin(g, scr1));
                if (!(el < eps)) { /* dmax(el, eps) takes el */
                    eps = el;
                    im = i;
                    br = (scr1 < g) ? 0 : 1; /* dmin(g, scr1): scr1 if scr1 < g, else g */
                }
            }
        }
        eps /= o->epsmin;
        s->eps[a] = eps;
        s->imax[a] = im;
        s->epsmin_branch[a] = br;
        if (dta <= o->dtmin + 1e-16 * tn) return -1;
        int accepted = eps <= o->epsmax;
        if (accepted && tf <= tn * c->tfd) {
            s->A = a + 1;
            s->dt[a + 1] = 0.0;
            s->dt_branch[a + 1] = -1;
            memcpy(y, yf, sizeof(double) * n);
            *tn_out = tn;
            return 0;
        }
        if (!accepted) tn = ts;
        double rteps = 0.5 * (eps + 1.0);
        rteps = 0.5 * (rteps + eps / rteps);
        rteps = 0.5 * (rteps + eps / rteps);
        s->rteps[a] = rteps;
        const double ca = dta * (1.0 / rteps + 0.005), cb = c->tfd * (tf - tn);
        double nd = dmin(ca, cb);
        int b = (cb < ca) ? 1 : 0;
        if (o->dtmax < nd) b = 2;
        nd = dmin(nd, o->dtmax);
        *dt = nd;
        s->dt_branch[a + 1] = b;
        if (!accepted) {
            qprev = qL;
            dprev = dL;
            ++a;
            continue;
        }
        s->A = a + 1;
        s->dt[a + 1] = nd;
        memcpy(y, yf, sizeof(double) * n);
        *tn_out = tn;
        return 0;
    }
}

/* ---- the backward pass of one step -------------------------------------- */

/* The adjoint of the right-hand side evaluation at y (corrector: with the
 * predictor's T, rrho, rrc of s). Accumulates into yb (n), pb (R), and for a
 * corrector call into *rrho_b, *rrc_b, *Tp_b (the predictor's frozen
 * quantities). A predictor call takes the correctors' adjoints of its rrho
 * and rrc (ext_rrho_b, ext_rrc_b) and also returns the temperature part in
 * yb[1]. */
static void qa_eval_adjoint(qa_ode* e, const qa_ctx* c, const qa_step* s, double t, const double* y,
                            const double* qb, const double* db, int corrector, double ext_rrho_b, double ext_rrc_b,
                            double* yb, double* pb, double* rrho_b, double* rrc_b, double* Tp_b, double* work) {
    const int n = c->n;
    double* q = work;
    double* d = q + n;
    double* q2 = d + n;
    double* d2 = q2 + n;
    double* scr = d2 + n;   /* 4 S */
    double* ycp = scr + 4 * (n - 2);
    if (corrector) {
        e->T = s->T;
        e->rrho = s->rrho;
        e->rrc = s->rrc;
    }
    qa_eval(e, t, y, q, d, corrector);
    if (corrector) {
        qa_vjp(e, y + 2, qb, db, 0.0, 0.0, yb + 2, pb, rrho_b, rrc_b, scr);
    } else {
        double own_rrho_b = 0.0, own_rrc_b = 0.0;
        /* the own uses of rrho / rrc first (qa_vjp's first loop), then the totals to rho and cp:
         * run qa_vjp twice would double the rates part, so split it by hand */
        const oracle_mech* m = e->m;
        const int S = m->S;
        for (int k = 0; k < S; ++k)
            own_rrho_b += qb[2 + k] * e->w->wq[k] * m->W[k] + db[2 + k] * e->w->wd[k] * m->W[k];
        own_rrc_b = qb[1] * e->qdot;
        const double rr_b = own_rrho_b + ext_rrho_b, rc_b = own_rrc_b + ext_rrc_b;
        const double rho_b = -rr_b * e->rrho * e->rrho - rc_b * e->rrc * e->rrc * e->cp_p;
        const double cp_b = -rc_b * e->rrc * e->rrc * e->rho_p;
        double dummy1 = 0.0, dummy2 = 0.0;
        qa_vjp(e, y + 2, qb, db, rho_b, cp_b, yb + 2, pb, &dummy1, &dummy2, scr);
    }
    /* temperature: forward difference */
    const double T0 = corrector ? s->T : y[1];
    const double dT = fabs(T0) * 1.4901161193847656e-08;
    double acc = 0.0;
    if (corrector) {
        e->T = T0 + dT;
        qa_eval(e, t, y, q2, d2, 1);
        e->T = T0;
    } else {
        memcpy(ycp, y, sizeof(double) * n);
        ycp[1] = T0 + dT;
        const double rrho0 = e->rrho, rrc0 = e->rrc;
        qa_eval(e, t, ycp, q2, d2, 0);
        acc += ext_rrho_b * (e->rrho - rrho0) + ext_rrc_b * (e->rrc - rrc0);
    }
    for (int i = 0; i < n; ++i) acc += qb[i] * (q2[i] - q[i]) + db[i] * (d2[i] - d[i]);
    const double rdT = 1.0 / ((T0 + dT) - T0);
    if (corrector) *Tp_b += acc * rdT;
    else yb[1] += acc * rdT;
}

/* Backward through one step recorded in s (by qa_step_run from ys at ts).
 * yb: in, the adjoint of the state after the step; out, of ys. *tsb: in, of
 * the time after the step; out, of ts. *dtb: in, of the step size the step
 * handed to the next one (0 for the last step); out, of the step size it
 * started with (0 for the first step, whose initial step size depends on
 * ys). */
static void qa_step_back(qa_ode* e, const qa_ctx* c, qa_step* s, double ts, int first, int last, double* yb,
                         double* tsb, double* dtb, double* pb, double* work) {
    const int n = c->n, I = c->P.itermax, A = s->A;
    const int* en = c->en;
    const double* ymin = c->ymin;
    const double* ys = s->ys;
    const double tf = c->tf, tfd = c->tfd, epsmin = c->P.epsmin;
    double* ysb = work;
    double* q0b = ysb + n;
    double* d0b = q0b + n;
    double* rtaub = d0b + n;
    double* qnb = rtaub + n;          /* adjoint of the q, d handed to the next attempt's predictor */
    double* dnb = qnb + n;
    double* rtsb = dnb + n;           /* adjoint of rtaus of the attempt after the current one */
    double* rtsb_cur = rtsb + n;
    double* scrb = rtsb_cur + n;      /* adjoint of the current scratch */
    double* yjb = scrb + n;           /* I vectors */
    double* qjb = yjb + (size_t)I * n;
    double* djb = qjb + n;
    double* ework = djb + n;
    double dtb_a[QA_MAX_ATTEMPTS + 1];
    for (int i = 0; i < n; ++i) ysb[i] = q0b[i] = d0b[i] = rtaub[i] = qnb[i] = dnb[i] = rtsb[i] = 0.0;
    for (int a = 0; a <= A; ++a) dtb_a[a] = 0.0;
    double rrho_b = 0.0, rrc_b = 0.0, Tp_b = 0.0, ts_b = 0.0;
    /* the time after the step: ts + dt of the accepted attempt */
    ts_b += *tsb;
    dtb_a[A - 1] += *tsb;
    if (!last) dtb_a[A] = *dtb;
    for (int a = A - 1; a >= 0; --a) {
        const double dta = s->dt[a];
        const double* rtaus = att_rtaus(s, a);
        /* rtaus of attempt a + 1 = rtaus_a * dt_{a+1} / dt_a */
        if (a < A - 1) {
            double rb = 0.0;
            const double ratio = s->dt[a + 1] / dta;
            for (int i = 0; i < n; ++i) {
                rb += rtsb[i] * rtaus[i];
                rtsb_cur[i] = rtsb[i] * ratio;
            }
            dtb_a[a + 1] += rb / dta;
            dtb_a[a] += -rb * s->dt[a + 1] / (dta * dta);
        } else {
            for (int i = 0; i < n; ++i) rtsb_cur[i] = 0.0;
        }
        /* the step size after attempt a (rejected: from ts; accepted, not last: from ts + dt_a) */
        double rtepsb = 0.0;
        if (!(a == A - 1 && last)) {
            const double g = dtb_a[a + 1];
            const int b = s->dt_branch[a + 1];
            if (b == 0) {
                const double rt = s->rteps[a];
                dtb_a[a] += g * (1.0 / rt + 0.005);
                rtepsb += -g * dta / (rt * rt);
            } else if (b == 1) {
                const double tnb = -tfd * g;
                ts_b += tnb;
                if (a == A - 1) dtb_a[a] += tnb;
            }
        }
        /* rteps = two Newton steps for sqrt(eps), eps = max(el_i, 1e-10) / epsmin */
        for (int j = 0; j < I; ++j)
            for (int i = 0; i < n; ++i) yjb[(size_t)j * n + i] = 0.0;
        for (int i = 0; i < n; ++i) {
            qjb[i] = qnb[i];
            djb[i] = dnb[i];
            scrb[i] = 0.0;
        }
        const double* qL = att_q(s, a, I - 1);
        const double* dL = att_d(s, a, I - 1);
        const double* y1 = att_y(s, a, 0);
        const double* raw = att_scr2(s, a);
        const double* yf = att_yfin(s, a);
        double* yfb = ework;  /* n */
        for (int i = 0; i < n; ++i) yfb[i] = (a == A - 1) ? yb[i] : 0.0;
        int ie = -1;          /* the component of eps's maximum, and the adjoint of its scr2c through scr1 */
        double ub_e = 0.0;
        if (rtepsb != 0.0 && s->imax[a] >= 0) {
            const double eps = s->eps[a];
            const double r0 = 0.5 * (eps + 1.0);
            const double r1 = 0.5 * (r0 + eps / r0);
            const double r1b = 0.5 * rtepsb * (1.0 - eps / (r1 * r1));
            double epsb = 0.5 * rtepsb / r1;
            const double r0b = 0.5 * r1b * (1.0 - eps / (r0 * r0));
            epsb += 0.5 * r1b / r0 + 0.5 * r0b;
            const double elb = epsb / epsmin;
            const int i = s->imax[a];
            double scr1b, gb = 0.0;
            if (s->epsmin_branch[a] == 0) scr1b = elb;
            else {
                scr1b = 0.5 * elb;
                gb = 0.5 * elb;
            }
            const double scr2c = en[i] ? dmax(raw[i], ymin[i]) : raw[i];
            const double u = scr2c - y1[i];
            const double ub = scr1b * rsign(u) / yf[i];
            yfb[i] += -scr1b * fabs(u) / (yf[i] * yf[i]);
            yjb[i] -= ub;     /* y1 is the first corrector input of the attempt */
            const double v = qL[i] - dL[i], wv = qL[i] + dL[i] + 1e-30;
            qjb[i] += gb * (rsign(v) / wv - fabs(v) / (wv * wv));
            djb[i] += gb * (-rsign(v) / wv - fabs(v) / (wv * wv));
            ie = i;
            ub_e = ub;
        }
        /* final state yf = max(scr2c, ymin), scr2c = en ? max(raw, ymin) : raw, raw = ys + dt scr_last */
        const double* scr_last = (I > 0) ? att_scr(s, a, I - 1) : att_scrp(s, a);
        double dtacc = 0.0;
        for (int i = 0; i < n; ++i) {
            const double scr2c = en[i] ? dmax(raw[i], ymin[i]) : raw[i];
            double sb2 = (scr2c < ymin[i]) ? 0.0 : yfb[i];
            if (i == ie) sb2 += ub_e;
            const double rawb = (en[i] && raw[i] < ymin[i]) ? 0.0 : sb2;
            scrb[i] = rawb * dta;
            ysb[i] += rawb;
            dtacc += rawb * scr_last[i];
        }
        dtb_a[a] += dtacc;
        /* corrector iterations, last first */
        const double rdt = 1.0 / dta;
        for (int j = I - 1; j >= 0; --j) {
            const double* yj = att_y(s, a, j);
            const double* qj = att_q(s, a, j);
            const double* dj = att_d(s, a, j);
            const double* sj = att_scr(s, a, j);
            double* ybj = yjb + (size_t)j * n;
            double rdtb = 0.0;
            dtacc = 0.0;
            for (int i = 0; i < n; ++i) {
                const double rb = en[i] ? 0.5 * (rtaus[i] + dta * dj[i] / yj[i]) : 0.0;
                const double an = pade_an(rb), ad = pade_den(rb);
                const double den = fma(an, rb, ad);
                const double sb = scrb[i];
                const double nmb = sb / den;
                const double denb = -sb * sj[i] / den;
                const double qs = s->q0[i];
                q0b[i] += nmb * (ad - an);
                qjb[i] += nmb * an;
                ysb[i] += -nmb * rb * ad * rdt;
                rdtb += -nmb * ys[i] * rb * ad;
                const double anb = nmb * (qj[i] - qs) + denb * rb;
                const double adb = nmb * (qs - ys[i] * rb * rdt) + denb;
                const double rbb = -nmb * ys[i] * ad * rdt + denb * an + anb * pade_an_d(rb) + adb * pade_den_d(rb);
                if (en[i]) {
                    rtsb_cur[i] += 0.5 * rbb;
                    dtacc += 0.5 * rbb * dj[i] / yj[i];
                    djb[i] += 0.5 * rbb * dta / yj[i];
                    ybj[i] += -0.5 * rbb * dta * dj[i] / (yj[i] * yj[i]);
                }
            }
            dtb_a[a] += dtacc + rdtb * (-rdt * rdt);
            /* the corrector evaluation at yj */
            qa_eval_adjoint(e, c, s, ts + dta + c->tstart, yj, qjb, djb, 1, 0.0, 0.0, ybj, pb, &rrho_b, &rrc_b,
                            &Tp_b, ework);
            /* yj = max(ymin, ys + dt scr_{j-1}) */
            const double* sp = (j > 0) ? att_scr(s, a, j - 1) : att_scrp(s, a);
            dtacc = 0.0;
            for (int i = 0; i < n; ++i) {
                const double rw = fma(dta, sp[i], ys[i]);
                const double b = (ymin[i] < rw) ? ybj[i] : 0.0;
                scrb[i] = b * dta;
                ysb[i] += b;
                dtacc += b * sp[i];
                qjb[i] = 0.0;
                djb[i] = 0.0;
            }
            dtb_a[a] += dtacc;
        }
        /* predictor: scr_p = (qprev - dprev) den(r) / (den(r) + num(r)), r = rtau */
        double* qpb = (a == 0) ? q0b : qnb;
        double* dpb = (a == 0) ? d0b : dnb;
        const double* qprev = (a == 0) ? s->q0 : att_q(s, a - 1, I - 1);
        const double* dprev = (a == 0) ? s->d0 : att_d(s, a - 1, I - 1);
        if (a > 0)
            for (int i = 0; i < n; ++i) qnb[i] = dnb[i] = 0.0;
        for (int i = 0; i < n; ++i) {
            const double r = s->rtau[i];
            const double den = pade_den(r), num = pade_num(r);
            const double P = den / (den + num);
            const double Pd = (pade_den_d(r) * num - den * pade_num_d(r)) / ((den + num) * (den + num));
            const double sb = scrb[i];
            qpb[i] += sb * P;
            dpb[i] -= sb * P;
            rtaub[i] += sb * (qprev[i] - dprev[i]) * Pd;
        }
        /* rtaus of this attempt: its adjoint goes to the one before (ratio) or to rtau */
        if (a == 0)
            for (int i = 0; i < n; ++i) rtaub[i] += rtsb_cur[i];
        else
            for (int i = 0; i < n; ++i) rtsb[i] = rtsb_cur[i];
    }
    /* rtau = dt_0 d0 / ys */
    const double dt0 = s->dt[0];
    double dtacc = 0.0;
    for (int i = 0; i < n; ++i) {
        if (!en[i]) continue;
        d0b[i] += rtaub[i] * dt0 / ys[i];
        ysb[i] += -rtaub[i] * dt0 * s->d0[i] / (ys[i] * ys[i]);
        dtacc += rtaub[i] * s->d0[i] / ys[i];
    }
    dtb_a[0] += dtacc;
    if (first) {
        const int i = s->dt0_imax;
        if (s->dt0_branch == 0 && i >= 0) {
            const double scb = dtb_a[0] * (-0.5 / (s->scrtch * s->scrtch));
            const double sg = rsign(0.1 * c->P.epsmin * fabs(s->q0[i]) - s->d0[i]);
            const double ay = fabs(1 / ys[i]);
            const double day = -rsign(ys[i]) / (ys[i] * ys[i]);   /* d |1/y| / dy */
            if (s->dt0_side == 0) {
                d0b[i] += scb * ay * sg;
                ysb[i] += scb * s->d0[i] * sg * day;
            } else {
                const double u = fabs(s->q0[i]) - s->d0[i];
                const double ub = -scb * rsign(u) * ay * sg;
                q0b[i] += ub * rsign(s->q0[i]);
                d0b[i] -= ub;
                ysb[i] += scb * (-fabs(u)) * sg * day;
            }
        }
        *dtb = 0.0;
    } else {
        *dtb = dtb_a[0];
    }
    /* the predictor evaluation at ys (its rrho, rrc also reached the correctors) */
    qa_eval_adjoint(e, c, s, ts + c->tstart, ys, q0b, d0b, 0, rrho_b, rrc_b, ysb, pb, NULL, NULL, NULL, ework);
    ysb[1] += Tp_b;
    memcpy(yb, ysb, sizeof(double) * n);
    *tsb = ts_b;
}

/* ---- one point ---------------------------------------------------------- */

/* Forward QSS integration of one point (as oracle_qss_point) and the
 * adjoint: ybar_in = d phi / d y_in and pbar += d phi / d ln(multiplier) for
 * phi = ybar_out . y_out. Returns the integrator's status, -33 (attempt cap),
 * -34 (stability check on) or -35 (out of memory). */
int oracle_qss_adjoint_point(const oracle_mech* m, oracle_ws* w, const oracle_source_options* o, const double* y_in,
                             const double* split, double tf, double t_start, double x, const double* ybar_out,
                             double* y_out, double* ybar_in, double* pbar, int* n_steps) {
    const int n = m->S + 2, S = m->S;
    if (o->qss_stability_check) return -34;
    const int I = o->qss_iteration_count;
    int ret = 0;
    int* en = (int*)malloc(sizeof(int) * n);
    double* ymin = (double*)malloc(sizeof(double) * n);
    for (int i = 0; i < n; ++i) {
        en[i] = (i != 0);
        ymin[i] = (i == 0) ? -1e4 : o->qss_minval;
    }
    qa_ctx c = {n, ymin, en, {o->qss_epsmin, o->qss_epsmax, o->qss_dtmin, o->qss_dtmax, o->qss_abstol, I, 0},
                tf, t_start, 1.000008};
    qa_step st;
    st.n = n;
    st.itermax = I;
    double* sbuf = (double*)malloc(sizeof(double) * (4 * (size_t)n + QA_MAX_ATTEMPTS * qa_att_doubles(n, I)));
    double* work = (double*)malloc(sizeof(double) * ((size_t)(24 + 2 * I) * n + 8 * (size_t)S + 64));
    st.q0 = sbuf; st.d0 = sbuf + n; st.rtau = sbuf + 2 * n; st.ys = sbuf + 3 * n; st.buf = sbuf + 4 * n;
    qa_ode e = {m, o, w, split, x, y_in[1], 1.0, 1.0, 1.0, 1.0, 0.0, 1.0};
    /* forward, keeping each step's start: ys, ts, the step size it starts with */
    int cap = 64, N = 0;
    double* tys = (double*)malloc(sizeof(double) * cap * n);
    double* tts = (double*)malloc(sizeof(double) * cap);
    double* tdt = (double*)malloc(sizeof(double) * cap);
    double* y = (double*)malloc(sizeof(double) * n);
    double* yn = (double*)malloc(sizeof(double) * n);
    if (!en || !ymin || !sbuf || !work || !tys || !tts || !tdt || !y || !yn) { ret = -35; goto done; }
    for (int i = 0; i < n; ++i) y[i] = en[i] ? dmax(y_in[i], ymin[i]) : y_in[i];
    double tn = 0.0, dt = 0.0;
    while (c.tfd * tn < tf) {
        if (N >= o->max_steps) { ret = -20; break; }
        if (N == cap) {
            cap *= 2;
            tys = (double*)realloc(tys, sizeof(double) * cap * n);
            tts = (double*)realloc(tts, sizeof(double) * cap);
            tdt = (double*)realloc(tdt, sizeof(double) * cap);
            if (!tys || !tts || !tdt) { ret = -35; goto done; }
        }
        memcpy(tys + (size_t)N * n, y, sizeof(double) * n);
        tts[N] = tn;
        tdt[N] = dt;
        double tnew = tn;
        ret = qa_step_run(&e, &c, &st, y, tn, N == 0, &dt, &tnew, yn);
        ++N;
        if (ret) break;
        tn = tnew;
        memcpy(y, yn, sizeof(double) * n);
    }
    memcpy(y_out, y, sizeof(double) * n);
    if (n_steps) *n_steps = N;
    if (ret) goto done;
    /* backward */
    double* yb = yn;
    memcpy(yb, ybar_out, sizeof(double) * n);
    double tsb = 0.0, dtb = 0.0;
    for (int k = N - 1; k >= 0; --k) {
        double dtk = tdt[k], tk = 0.0;
        const int r = qa_step_run(&e, &c, &st, tys + (size_t)k * n, tts[k], k == 0, &dtk, &tk, y);
        if (r) { ret = r; goto done; }
        qa_step_back(&e, &c, &st, tts[k], k == 0, k == N - 1, yb, &tsb, &dtb, pbar, work);
    }
    for (int i = 0; i < n; ++i) ybar_in[i] = (en[i] && y_in[i] < ymin[i]) ? 0.0 : yb[i];
done:
    free(en); free(ymin); free(sbuf); free(work); free(tys); free(tts); free(tdt); free(y); free(yn);
    return ret;
}

/* Batch of points, threaded over points. pbar: [n][R] per point. */
typedef struct {
    const oracle_mech* m;
    const oracle_source_options* o;
    int n;
    const double *state_in, *split, *dt, *x, *ybar_out;
    double t_start;
    double *state_out, *ybar_in, *pbar;
    int *status, *steps;
    int next;
    pthread_mutex_t lock;
} qa_batch;

static void* qa_worker(void* arg) {
    qa_batch* b = (qa_batch*)arg;
    const int n = b->m->S + 2, R = b->m->R;
    oracle_ws* w = oracle_ws_create(b->m);
    for (;;) {
        pthread_mutex_lock(&b->lock);
        const int j = b->next++;
        pthread_mutex_unlock(&b->lock);
        if (j >= b->n) break;
        double* pb = b->pbar + (size_t)j * R;
        for (int i = 0; i < R; ++i) pb[i] = 0.0;
        b->status[j] = oracle_qss_adjoint_point(b->m, w, b->o, b->state_in + (size_t)j * n,
                                                b->split ? b->split + (size_t)j * n : NULL, b->dt[j], b->t_start,
                                                b->x ? b->x[j] : 0.0, b->ybar_out + (size_t)j * n,
                                                b->state_out + (size_t)j * n, b->ybar_in + (size_t)j * n, pb,
                                                b->steps ? b->steps + j : NULL);
    }
    oracle_ws_free(w);
    return NULL;
}

void oracle_qss_adjoint_batch(const oracle_mech* m, int n, const double* state_in, const double* split,
                              const double* dt, double t_start, const double* x, const oracle_source_options* o,
                              const double* ybar_out, double* state_out, double* ybar_in, double* pbar, int* status,
                              int* steps, int n_threads) {
    qa_batch b = {m, o, n, state_in, split, dt, x, ybar_out, t_start, state_out, ybar_in, pbar, status, steps, 0};
    pthread_mutex_init(&b.lock, NULL);
    if (n_threads < 1) n_threads = 1;
    pthread_t th[256];
    if (n_threads > 256) n_threads = 256;
    for (int t = 0; t < n_threads; ++t) pthread_create(&th[t], NULL, qa_worker, &b);
    for (int t = 0; t < n_threads; ++t) pthread_join(th[t], NULL);
    pthread_mutex_destroy(&b.lock);
}
