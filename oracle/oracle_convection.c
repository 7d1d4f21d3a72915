/* Oracle (test infrastructure only, never a product path): CPU restatement of
 * the convection stage, ConvectionSystemSplit::integrateToTime
 * (src/convectionSystem.cpp:588-627), against which the GPU convection
 * kernels are checked bit for bit.
 *
 *  - ConvectionSystemUTW::f (src/convectionSystem.cpp:14-130): continuity
 *    integral for rV from the continuity boundary point, V = rV / r, upwinded
 *    derivatives of T, U and the mean molecular weight W, and their time
 *    derivatives with the strain-rate source of U;
 *  - the UTW system integrated in one-step mode with a stop time, V / rho
 *    recorded after every step (src/convectionSystem.cpp:592-611);
 *  - ConvectionSystemY::f (src/convectionSystem.cpp:307-359) per species, with
 *    v(t) interpolated from that record by ConvectionSystemY::update_v
 *    (src/convectionSystem.cpp:372-398), integrated to the end time
 *    (src/convectionSystem.cpp:616-627, SundialsCvode::integrateToTime);
 *  - setState's initial W from the mass fractions and setSplitConstants'
 *    W split constant (src/convectionSystem.cpp:485-511, 572-586).
 *
 * Both integrations use CVODE's Adams method with a zero-bandwidth
 * difference-quotient Jacobian (src/convectionSystem.cpp:467-478, 663-676;
 * src/sundialsUtils.cpp:104-130). The Adams integrator here is an own
 * variable-order (1..12) Nordsieck restatement of the published method (the
 * step and order control of the BDF integrator in oracle_bdf.c with the
 * Adams-Moulton coefficients), not SUNDIALS source: parity with CVODE itself
 * is unpinned; accuracy is checked against scipy. Norms are summed in the
 * order of the GPU CTA that integrates the system (256 slots for UTW, 32 for
 * a species) so that the GPU reproduces every bit.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

#define GAS_CONSTANT (6.02214076e26 * 1.380649e-23)
#define QA 12

double oracle_block_sum(const double* a, const double* b, int n, int W);

static double dmaxc(double a, double b) { return (a < b) ? b : a; }
static double dminc(double a, double b) { return (b < a) ? b : a; }
static double cpow_(double x, double e) { return oracle_exp(e * oracle_log(x)); }

/* ---- Adams-Moulton coefficients ---------------------------------------- */

/* g[j]: the Adams-Bashforth error constants gamma_j (gamma_0 = 1,
 * gamma_j = 1 - sum_{i<j} gamma_i / (j + 1 - i)); the Adams-Moulton constant
 * of order j is gamma_j - gamma_{j-1}. */
void oracle_adams_gammas(double* g) {
    g[0] = 1.0;
    for (int j = 1; j <= QA + 1; ++j) {
        double s = 0.0;
        for (int i = 0; i < j; ++i) s = s + g[i] / (double)(j + 1 - i);
        g[j] = 1.0 - s;
    }
}

/* l_j of the order-q Adams-Moulton corrector in Nordsieck form: the
 * coefficients of Lambda(x) = int_{-1}^{x} P(u) du / int_{-1}^{0} P(u) du with
 * P(u) = prod_{i=1}^{q-1} (u + i) (constant step). */
void oracle_adams_l(int q, double* l) {
    double p[QA + 2];
    for (int j = 0; j <= QA + 1; ++j) {
        p[j] = 0.0;
        l[j] = 0.0;
    }
    p[0] = 1.0;
    for (int i = 1; i <= q - 1; ++i) {
        for (int j = i; j >= 1; --j) p[j] = p[j - 1] + (double)i * p[j];
        p[0] = (double)i * p[0];
    }
    double q0 = 0.0;
    for (int j = 0; j < q; ++j) {
        const double tj = p[j] / (double)(j + 1);
        q0 = (j % 2 == 0) ? q0 + tj : q0 - tj;
    }
    l[0] = 1.0;
    for (int j = 0; j < q; ++j) l[j + 1] = (p[j] / (double)(j + 1)) / q0;
}

/* ---- the integrator ---------------------------------------------------- */

typedef struct adams_sys adams_sys;
struct adams_sys {
    void (*f)(adams_sys*, double t, const double* y, double* ydot);
    void (*on_step)(adams_sys*, double t); /* after every accepted step, or NULL */
    int n;
    int W; /* slots of the norms' partial sums: the GPU CTA width (UTW 256, species 32) */
};

/* Weighted RMS norm in the GPU's order: term i in slot i mod W (each slot in
 * increasing i), the slots folded into 32 in slot order, an xor butterfly. */
static double wrms_w(const double* v, const double* ewt, int n, double* tmp, int W) {
    for (int i = 0; i < n; ++i) tmp[i] = v[i] * ewt[i];
    return sqrt(oracle_block_sum(tmp, tmp, n, W) / n);
}
#define wrms_c(v, ewt, n, tmp) wrms_w(v, ewt, n, tmp, s->W)

/* Integrate y' = f(t, y) from t0 to tf. tstop != 0: never step past tf (the
 * last step ends on tf; one-step mode with a stop time); else step past tf
 * and interpolate (normal mode). atol: per component. Returns 0 or a
 * negative status (-11 too many steps, -13 error-test failures, -14
 * convergence failures). stats: steps, RHS calls, failures, Jacobians. */
static int adams_integrate(adams_sys* s, double* yio, const double* atol, double rtol, double t0, double tf,
                           int tstop, double hmin, int max_steps, int* stats) {
    const int n = s->n;
    double* buf = (double*)calloc((size_t)n * (2 * (QA + 2) + 14), sizeof(double));
    double* z[QA + 2];
    double* zs[QA + 2];
    for (int j = 0; j <= QA + 1; ++j) {
        z[j] = buf + (size_t)j * n;
        zs[j] = buf + (size_t)(QA + 2 + j) * n;
    }
    double* b0 = buf + (size_t)(2 * (QA + 2)) * n;
    double *acor = b0, *acorp = b0 + n, *ewt = b0 + 2 * (size_t)n, *y = b0 + 3 * (size_t)n;
    double *ft = b0 + 4 * (size_t)n, *bb = b0 + 5 * (size_t)n, *tmp = b0 + 6 * (size_t)n;
    double *f0 = b0 + 7 * (size_t)n, *ycopy = b0 + 8 * (size_t)n, *f1 = b0 + 9 * (size_t)n;
    double *jd = b0 + 10 * (size_t)n, *md = b0 + 11 * (size_t)n;
    const double uround = 2.220446049250313e-16;
    double g[QA + 2];
    oracle_adams_gammas(g);
    int nst = 0, nfe = 0, nje = 0, nfail = 0, status = 0;

#define SET_EWT(v) \
    for (int i = 0; i < n; ++i) ewt[i] = 1.0 / (rtol * fabs((v)[i]) + atol[i]);

    memcpy(z[0], yio, sizeof(double) * n);
    s->f(s, t0, z[0], f0);
    nfe++;
    SET_EWT(z[0]);
    /* initial step: as the BDF integrator, on the interval [t0, tf] */
    double t = t0;
    const double tdist = tf - t0;
    double hub = 0.1 * tdist;
    double rmax = 0.0;
    for (int i = 0; i < n; ++i) rmax = dmaxc(rmax, fabs(f0[i]) / (0.1 * fabs(z[0][i]) + atol[i]));
    if (rmax * hub > 1.0) hub = 1.0 / rmax;
    const double hlb = 100.0 * uround * dmaxc(fabs(t0), fabs(tf));
    double hg = sqrt(hlb * hub);
    double h;
    if (hub > hlb) {
        for (int it = 0; it < 4; ++it) {
            for (int i = 0; i < n; ++i) ycopy[i] = fma(hg, f0[i], z[0][i]);
            s->f(s, t0 + hg, ycopy, f1);
            nfe++;
            for (int i = 0; i < n; ++i) tmp[i] = (f1[i] - f0[i]) / hg;
            const double ydd = wrms_c(tmp, ewt, n, bb);
            const double hnew = (ydd * hub * hub > 2.0) ? sqrt(2.0 / ydd) : sqrt(hg * hub);
            const double ratio = hnew / hg;
            hg = hnew;
            if (ratio > 0.5 && ratio < 2.0) break;
        }
        h = dminc(dmaxc(0.5 * hg, hlb), hub);
    } else {
        h = hlb;
    }
    if (h < hmin) h = hmin;
    for (int i = 0; i < n; ++i) z[1][i] = h * f0[i];

    int q = 1, qwait = 2, nstlp = 0, nstlj = 0, have_m = 0, have_acorp = 0, qsave = 0;
    double gammap = 0.0, crate = 1.0, etamax = 10000.0, acnrm = 0.0, hsave = 0.0;
    double l[QA + 2];

    while (t < tf) {
        if (nst >= max_steps) {
            status = -11;
            break;
        }
        if (tstop && t + h > tf) {
            /* the step would pass the stop time: shorten it to end there */
            const double eta = (tf - t) / h;
            double sc = eta;
            for (int j = 1; j <= q; ++j) {
                for (int i = 0; i < n; ++i) z[j][i] *= sc;
                sc *= eta;
            }
            h = tf - t;
        }
        for (int j = 0; j <= q; ++j) memcpy(zs[j], z[j], sizeof(double) * n);
        int ncf = 0, nef = 0, convfail_bad_j = 0, force_setup = !have_m;
        double dsm = 0.0;
        for (;;) {
            for (int k = 1; k <= q; ++k)
                for (int j = q; j >= k; --j)
                    for (int i = 0; i < n; ++i) z[j - 1][i] += z[j][i];
            const double tn = t + h;
            oracle_adams_l(q, l);
            const double cq = fabs(g[q] - g[q - 1]) / g[q - 1];
            const double gamma = h / l[1];
            const double tq4 = 0.1 / cq;
            int jcur = 0;
            const double gamrat0 = have_m ? gamma / gammap : 1.0;
            if (force_setup || nst >= nstlp + 20 || fabs(gamrat0 - 1.0) > 0.3) {
                const int jbad = (nst == 0) || (nst >= nstlj + 51) || convfail_bad_j || !have_m;
                if (jbad) {
                    /* diagonal difference quotient: every component perturbed at once */
                    s->f(s, tn, z[0], ft);
                    nfe++;
                    const double fnorm = wrms_c(ft, ewt, n, tmp);
                    const double srur = sqrt(uround);
                    const double min_inc = (fnorm != 0.0) ? (1000.0 * fabs(h) * uround * n * fnorm) : 1.0;
                    for (int i = 0; i < n; ++i) {
                        const double inc = dmaxc(srur * fabs(z[0][i]), min_inc / ewt[i]);
                        bb[i] = inc;
                        ycopy[i] = z[0][i] + inc;
                    }
                    s->f(s, tn, ycopy, f1);
                    nfe++;
                    for (int i = 0; i < n; ++i) jd[i] = (f1[i] - ft[i]) / bb[i];
                    nje++;
                    nstlj = nst;
                    jcur = 1;
                }
                int sing = 0;
                for (int i = 0; i < n; ++i) {
                    md[i] = 1.0 - gamma * jd[i];
                    if (md[i] == 0.0) sing = 1;
                }
                gammap = gamma;
                nstlp = nst;
                crate = 1.0;
                have_m = !sing;
                force_setup = 0;
                convfail_bad_j = 0;
                if (sing) goto conv_fail;
            }
            {
                const double gamrat = gamma / gammap;
                memset(acor, 0, sizeof(double) * n);
                memcpy(y, z[0], sizeof(double) * n);
                double delp = 0.0, del = 0.0;
                int converged = 0;
                const double rl1 = 1.0 / l[1];
                for (int mit = 0; mit < 3; ++mit) {
                    s->f(s, tn, y, ft);
                    nfe++;
                    for (int i = 0; i < n; ++i) bb[i] = (gamma * ft[i] - fma(rl1, z[1][i], acor[i])) / md[i];
                    if (gamrat != 1.0) {
                        const double sc = 2.0 / (1.0 + gamrat);
                        for (int i = 0; i < n; ++i) bb[i] *= sc;
                    }
                    del = wrms_c(bb, ewt, n, tmp);
                    for (int i = 0; i < n; ++i) {
                        acor[i] += bb[i];
                        y[i] = z[0][i] + acor[i];
                    }
                    if (mit > 0) crate = dmaxc(0.3 * crate, del / delp);
                    const double dcon = del * dminc(1.0, crate) / tq4;
                    if (dcon <= 1.0) {
                        acnrm = (mit == 0) ? del : wrms_c(acor, ewt, n, tmp);
                        converged = 1;
                        break;
                    }
                    if (mit >= 1 && del > 2.0 * delp) break;
                    delp = del;
                }
                if (!converged) goto conv_fail;
            }
            dsm = acnrm * cq;
            if (dsm <= 1.0) break;
            nef++;
            nfail++;
            for (int j = 0; j <= q; ++j) memcpy(z[j], zs[j], sizeof(double) * n);
            if (nef >= 7 || h <= hmin * 1.0000000000000002) {
                status = -13;
                goto done;
            }
            {
                double eta;
                if (nef <= 3) {
                    eta = 1.0 / (cpow_(6.0 * dsm, 1.0 / (q + 1)) + 1e-6);
                    eta = dmaxc(0.1, dmaxc(eta, hmin / h));
                    if (nef >= 2) eta = dminc(eta, 0.2);
                    double sc = eta;
                    for (int j = 1; j <= q; ++j) {
                        for (int i = 0; i < n; ++i) z[j][i] *= sc;
                        sc *= eta;
                    }
                    h *= eta;
                } else {
                    eta = dmaxc(0.1, hmin / h);
                    h *= eta;
                    q = 1;
                    s->f(s, t, z[0], ft);
                    nfe++;
                    for (int i = 0; i < n; ++i) z[1][i] = h * ft[i];
                }
                qwait = q + 1;
                have_acorp = 0;
                etamax = 1.0;
                for (int j = 0; j <= q; ++j) memcpy(zs[j], z[j], sizeof(double) * n);
            }
            continue;
        conv_fail:
            for (int j = 0; j <= q; ++j) memcpy(z[j], zs[j], sizeof(double) * n);
            nfail++;
            if (!jcur && have_m) {
                force_setup = 1;
                convfail_bad_j = 1;
                continue;
            }
            ncf++;
            if (ncf >= 10 || h <= hmin * 1.0000000000000002) {
                status = -14;
                goto done;
            }
            {
                const double eta = dmaxc(0.25, hmin / h);
                double sc = eta;
                for (int j = 1; j <= q; ++j) {
                    for (int i = 0; i < n; ++i) z[j][i] *= sc;
                    sc *= eta;
                }
                h *= eta;
                qwait = q + 1;
                have_acorp = 0;
                etamax = 1.0;
                force_setup = 1;
                for (int j = 0; j <= q; ++j) memcpy(zs[j], z[j], sizeof(double) * n);
            }
        }
        /* ---- accepted step ---- */
        nst++;
        {
            const double tnew = t + h;
            t = (tstop && (tnew >= tf || tf - tnew <= 100.0 * uround * (fabs(tnew) + fabs(h)))) ? tf : tnew;
        }
        for (int j = 0; j <= q; ++j)
            for (int i = 0; i < n; ++i) z[j][i] = fma(l[j], acor[i], z[j][i]);
        SET_EWT(z[0]);
        if (s->on_step) s->on_step(s, t);
        const double etaq = 1.0 / (cpow_(6.0 * dsm, 1.0 / (q + 1)) + 1e-6);
        double eta = etaq;
        int qnew = q;
        qwait--;
        if (qwait == 0) {
            double etaqm1 = 0.0, etaqp1 = 0.0;
            if (q > 1) {
                /* order q-1: |gamma*_{q-1}| h^q |y^(q)| with h^q y^(q) = q! z_q */
                double fact = 1.0;
                for (int i = 2; i <= q; ++i) fact *= i;
                const double ddn = wrms_c(z[q], ewt, n, tmp) * (fabs(g[q - 1] - g[q - 2]) * fact);
                etaqm1 = 1.0 / (cpow_(6.0 * ddn, 1.0 / q) + 1e-6);
            }
            if (q < QA && have_acorp && qsave == q) {
                /* order q+1: the change of the correction over one step,
                 * acor ~ -gamma_{q-1} h^{q+1} y^(q+1) */
                const double cc = cpow_(h / hsave, (double)(q + 1));
                for (int i = 0; i < n; ++i) tmp[i] = fma(-cc, acorp[i], acor[i]);
                const double dup = wrms_c(tmp, ewt, n, bb) * (fabs(g[q + 1] - g[q]) / g[q - 1]);
                etaqp1 = 1.0 / (cpow_(10.0 * dup, 1.0 / (q + 2)) + 1e-6);
            }
            if (etaq >= etaqm1 && etaq >= etaqp1) {
                eta = etaq;
            } else if (etaqm1 >= etaqp1) {
                eta = etaqm1;
                qnew = q - 1;
            } else {
                eta = etaqp1;
                qnew = q + 1;
            }
            qwait = 2;
        } else if (qwait == 1 && q < QA) {
            memcpy(acorp, acor, sizeof(double) * n);
            hsave = h;
            qsave = q;
            have_acorp = 1;
        }
        if (etamax <= 1.0) {
            eta = 1.0;
            qnew = q;
        } else if (eta < 1.5 && qnew == q) {
            eta = 1.0;
        } else {
            eta = dminc(eta, etamax);
            if (h * eta < hmin) eta = hmin / h;
        }
        if (qnew > q) {
            /* new column z_{q+1} = h^{q+1} y^(q+1) / (q+1)! from the correction */
            double fact = 1.0;
            for (int i = 2; i <= q + 1; ++i) fact *= i;
            const double c = -1.0 / (g[q - 1] * fact);
            for (int i = 0; i < n; ++i) z[q + 1][i] = acor[i] * c;
        }
        if (qnew != q) {
            q = qnew;
            qwait = q + 1;
            have_acorp = 0;
        }
        if (eta != 1.0) {
            double sc = eta;
            for (int j = 1; j <= q; ++j) {
                for (int i = 0; i < n; ++i) z[j][i] *= sc;
                sc *= eta;
            }
            h *= eta;
        }
        etamax = 10.0;
    }
    {
        /* the solution at tf from the Nordsieck array */
        const double sv = (tf - t) / h;
        for (int i = 0; i < n; ++i) {
            double v = z[q][i];
            for (int j = q - 1; j >= 0; --j) v = fma(v, sv, z[j][i]);
            yio[i] = v;
        }
    }
done:
    if (status != 0) memcpy(yio, z[0], sizeof(double) * n);
    if (stats) {
        stats[0] = nst;
        stats[1] = nfe;
        stats[2] = nfail;
        stats[3] = nje;
    }
    free(buf);
    return status;
#undef SET_EWT
}

/* ---- the UTW system ---------------------------------------------------- */

static double center_volume(const double* x, int alpha) { return alpha == 0 ? x[1] : (x[1] * x[1]) / 2.0; }

/* a(t) and da/dt: LinearFunction (src/scalarFunction.cpp:12-22), or
   ChebyshevFunction (src/scalarFunction.cpp:31-87) with its coefficient
   padding (fewer than two coefficients count as zeros) and its derivative
   recurrence, which weights coefficient i by i U_i(x) (the reference's loop
   advances the U recurrence before using it; T'_i = i U_{i-1}). */
void oracle_convection_strain(const oracle_conv_flame* fl, double t, double* a, double* dadt) {
    if (fl->strain_type == 1) {
        double c[16];
        int n = fl->n_cheb;
        for (int i = 0; i < 16; ++i) c[i] = i < n ? fl->cheb[i] : 0.0;
        if (n < 2) n = 2;
        const double x = (2 * (t - fl->cheb_t0)) / (fl->cheb_t1 - fl->cheb_t0) - 1;
        double cm = 1, cn = x;
        double y = c[0] + x * c[1];
        for (int i = 2; i < n; ++i) {
            const double cp = (2 * x) * cn - cm;
            y += cp * c[i];
            cm = cn;
            cn = cp;
        }
        *a = y;
        cm = 1;
        cn = 2 * x;
        double dydx = c[1];
        for (int i = 2; i < n; ++i) {
            const double cp = (2 * x) * cn - cm;
            dydx += ((double)i * cp) * c[i];
            cm = cn;
            cn = cp;
        }
        *dadt = dydx * (2.0 / (fl->cheb_t1 - fl->cheb_t0));
        return;
    }
    const double a0 = fl->strain_initial, a1 = fl->strain_final, T0 = fl->strain_t0, Dt = fl->strain_dt;
    *a = (t <= T0) ? a0 : (t >= T0 + Dt) ? a1 : a0 + ((a1 - a0) * (t - T0)) / Dt;
    *dadt = (t >= T0 && t < T0 + Dt) ? (a1 - a0) / Dt : 0.0;
}

typedef struct {
    adams_sys base;
    const oracle_conv_flame* fl;
    int N;
    const double *x, *hh, *rph, *drhodt, *sU, *sT, *sW;
    double *rho, *rV, *V;
    int max_history, n_history, overflow;
    double *hist_t, *hist_v;
} utw_ctx;

void oracle_convection_utw_rhs(const oracle_conv_flame* fl, const double* x, const double* hh, const double* rph,
                               double t, const double* y, const double* drhodt, const double* sU,
                               const double* sT, const double* sW, double* ydot, double* rho, double* rV,
                               double* V) {
    const int N = fl->n_points, jj = N - 1, jc = fl->j_cont;
    const double beta = fl->beta;
#define T_(j) y[3 * (j) + 1]
#define U_(j) y[3 * (j) + 0]
#define W_(j) y[3 * (j) + 2]
    for (int j = 0; j < N; ++j) rho[j] = (fl->pressure * W_(j)) / (GAS_CONSTANT * T_(j));
#define MFLUX(j) ((hh[j] * rph[j]) * (drhodt[j] + (rho[j] * beta) * U_(j)))
    if (fl->continuity_bc == ORACLE_CONT_LEFT) {
        rV[0] = fl->rv_zero;
        for (int j = 0; j < N - 1; ++j) rV[j + 1] = rV[j] - MFLUX(j);
    } else if (fl->continuity_bc == ORACLE_CONT_ZERO) {
        int j = jc;
        double dVdx0 = -rph[j] * (drhodt[j] - (rho[j] * beta) * U_(j));
        if (jc != 0) dVdx0 = 0.5 * dVdx0 - (0.5 * rph[j - 1]) * (drhodt[j - 1] + (rho[j - 1] * beta) * U_(j - 1));
        rV[j] = (x[j] - fl->x_vzero) * dVdx0;
        for (j = jc; j < jj; ++j) rV[j + 1] = rV[j] - MFLUX(j);
        if (jc != 0) {
            j = jc - 1;
            rV[j] = (x[j] - fl->x_vzero) * dVdx0;
            for (j = jc - 1; j > 0; --j) rV[j - 1] = rV[j] + MFLUX(j - 1);
        }
    } else {
        if (fl->continuity_bc == ORACLE_CONT_TEMP) {
            const int j = jc;
            /* at the last point (where the update can put the temperature
               crossing) only the backward difference exists; the reference
               reads T[jj + 1] there */
            if (j == 0 || (j < jj && sT[j] / (T_(j + 1) - T_(j)) < 0))
                rV[j] = (((rph[j] * rho[j]) * sT[j]) * hh[j]) / (T_(j + 1) - T_(j));
            else
                rV[j] = (((rph[j - 1] * rho[j]) * sT[j]) * hh[j - 1]) / (T_(j) - T_(j - 1));
        } else {
            rV[jc] = fl->rv_cont;
        }
        for (int j = jc; j < N - 1; ++j) rV[j + 1] = rV[j] - MFLUX(j);
        for (int j = jc; j > 0; --j)
            rV[j - 1] = rV[j] + (hh[j - 1] * rph[j]) * (drhodt[j] + (rho[j] * beta) * U_(j));
    }
#undef MFLUX
    V[0] = rV[0];
    for (int j = 1; j < N; ++j) V[j] = fl->alpha == 0 ? rV[j] : rV[j] / x[j];
    double a, dadt;
    oracle_convection_strain(fl, t, &a, &dadt);
    const double K = dadt / beta + (a * a) / (beta * beta);
    /* left boundary */
    ydot[0] = (sU[0] - U_(0) * U_(0)) + (fl->rhou / rho[0]) * K;
    if (fl->left_bc == ORACLE_BC_CONTROL_VOLUME || fl->left_bc == ORACLE_BC_WALL_FLUX) {
        const double cvol = center_volume(x, fl->alpha);
        const double rvm = dmaxc(rV[0], 0.0);
        ydot[1] = (-rvm * (T_(0) - fl->t_left)) / (rho[0] * cvol) + sT[0];
        ydot[2] = (-rvm * (W_(0) - fl->w_left)) / (rho[0] * cvol) - (W_(0) * W_(0)) * sW[0];
    } else {
        ydot[1] = sT[0];
        ydot[2] = -((W_(0) * W_(0)) * sW[0]);
    }
    /* interior: upwinded derivatives */
    for (int j = 1; j < jj; ++j) {
        double dT, dU, dW;
        if (rV[j] < 0) {
            dT = (T_(j + 1) - T_(j)) / hh[j];
            dU = (U_(j + 1) - U_(j)) / hh[j];
            dW = (W_(j + 1) - W_(j)) / hh[j];
        } else {
            dT = (T_(j) - T_(j - 1)) / hh[j - 1];
            dU = (U_(j) - U_(j - 1)) / hh[j - 1];
            dW = (W_(j) - W_(j - 1)) / hh[j - 1];
        }
        ydot[3 * j + 0] = (((-V[j] * dU) / rho[j] - U_(j) * U_(j)) + (fl->rhou / rho[j]) * K) + sU[j];
        ydot[3 * j + 1] = (-V[j] * dT) / rho[j] + sT[j];
        ydot[3 * j + 2] = (-V[j] * dW) / rho[j] - (W_(j) * W_(j)) * sW[j];
    }
    /* right boundary */
    if (rV[jj] < 0 || fl->right_bc == ORACLE_BC_FIXED_VALUE) {
        ydot[3 * jj + 0] = (sU[jj] - U_(jj) * U_(jj)) + (fl->rhou / rho[jj]) * K;
        ydot[3 * jj + 1] = sT[jj];
        ydot[3 * jj + 2] = -((W_(jj) * W_(jj)) * sW[jj]);
    } else {
        const double hl = hh[jj - 1];
        ydot[3 * jj + 0] =
            ((sU[jj] - ((V[jj] * (U_(jj) - U_(jj - 1))) / hl) / rho[jj]) - U_(jj) * U_(jj)) + (fl->rhou / rho[jj]) * K;
        ydot[3 * jj + 1] = sT[jj] - ((V[jj] * (T_(jj) - T_(jj - 1))) / hl) / rho[jj];
        ydot[3 * jj + 2] = -((W_(jj) * W_(jj)) * sW[jj]) - ((V[jj] * (W_(jj) - W_(jj - 1))) / hl) / rho[jj];
    }
#undef T_
#undef U_
#undef W_
}

static void utw_f(adams_sys* s, double t, const double* y, double* ydot) {
    utw_ctx* c = (utw_ctx*)s;
    oracle_convection_utw_rhs(c->fl, c->x, c->hh, c->rph, t, y, c->drhodt, c->sU, c->sT, c->sW, ydot, c->rho, c->rV,
                              c->V);
}

/* V / rho of the last right-hand side, recorded with the time */
static void utw_record(utw_ctx* c, double t) {
    if (c->n_history >= c->max_history) {
        c->overflow = 1;
        return;
    }
    c->hist_t[c->n_history] = t;
    double* v = c->hist_v + (size_t)c->n_history * c->N;
    for (int j = 0; j < c->N; ++j) v[j] = c->V[j] / c->rho[j];
    c->n_history++;
}

static void utw_on_step(adams_sys* s, double t) { utw_record((utw_ctx*)s, t); }

/* ---- species systems --------------------------------------------------- */

typedef struct {
    adams_sys base;
    const oracle_conv_flame* fl;
    int N;
    const double *x, *hh, *split;
    double y_left;
    int n_history;
    const double *hist_t, *hist_v;
} spec_ctx;

/* ConvectionSystemY::update_v: the interval is [lower_bound(t), next], moved
 * back by one at the end of the record. Returns the left index, s. */
int oracle_convection_interval(const double* ht, int H, double t, double* s) {
    if (H == 1) {
        *s = 0.0;
        return -1;
    }
    int iL = 0;
    while (iL < H && ht[iL] < t) ++iL;
    if (iL == H) iL--;
    if (iL + 1 == H) iL--;
    *s = (t - ht[iL]) / (ht[iL + 1] - ht[iL]);
    return iL;
}

static void spec_f(adams_sys* sy, double t, const double* y, double* ydot) {
    spec_ctx* c = (spec_ctx*)sy;
    const oracle_conv_flame* fl = c->fl;
    const int N = c->N, jj = N - 1;
    double s;
    const int iL = oracle_convection_interval(c->hist_t, c->n_history, t, &s);
    const double* vL = c->hist_v + (size_t)(iL < 0 ? 0 : iL) * N;
    const double* vR = iL < 0 ? vL : vL + N;
#define VV(j) (iL < 0 ? vL[j] : vL[j] * (1 - s) + vR[j] * s)
    if (fl->left_bc == ORACLE_BC_CONTROL_VOLUME || fl->left_bc == ORACLE_BC_WALL_FLUX) {
        const double cvol = center_volume(c->x, fl->alpha);
        const double rvm = dmaxc(VV(0), 0.0);
        ydot[0] = (-rvm * (y[0] - c->y_left)) / cvol + c->split[0];
    } else {
        ydot[0] = c->split[0];
    }
    for (int j = 1; j < jj; ++j) {
        const double v = VV(j);
        const double dYdx = (v < 0) ? (y[j + 1] - y[j]) / c->hh[j] : (y[j] - y[j - 1]) / c->hh[j - 1];
        ydot[j] = -v * dYdx + c->split[j];
    }
    const double vj = VV(jj);
    if (vj < 0 || fl->right_bc == ORACLE_BC_FIXED_VALUE)
        ydot[jj] = c->split[jj];
    else
        ydot[jj] = c->split[jj] - (vj * (y[jj] - y[jj - 1])) / c->hh[jj - 1];
#undef VV
}

/* ---- the stage ----------------------------------------------------------- */

/* hh and the half-point radius factor rphalf = r^alpha (OneDimGrid,
 * src/grid.cpp:52-58). rph[N-1] extends rphalf by the factor at the last
 * point: ConvectionSystemUTW::f reads rphalf[jj] for the fixedRight and
 * stagnation-point conditions (src/convectionSystem.cpp:31, 62), one past the
 * end of the reference's array. */
void oracle_convection_grid(int N, const double* x, int alpha, double* hh, double* rph) {
    for (int j = 0; j < N - 1; ++j) {
        hh[j] = x[j + 1] - x[j];
        const double xm = 0.5 * (x[j] + x[j + 1]);
        rph[j] = alpha == 0 ? 1.0 : xm;
    }
    hh[N - 1] = 0.0;
    rph[N - 1] = alpha == 0 ? 1.0 : x[N - 1];
}

void oracle_convection_prepare(int N, int S, const double* W, const double* state, const double* split,
                               double* Wmx, double* sW) {
    for (int j = 0; j < N; ++j) {
        double ysum = 0.0;
        for (int k = 0; k < S; ++k) ysum = ysum + dmaxc(state[(size_t)(2 + k) * N + j], 0.0);
        const double rnorm = 1.0 / ysum;
        double acc = 0.0;
        for (int k = 0; k < S; ++k) acc = acc + (dmaxc(state[(size_t)(2 + k) * N + j], 0.0) * rnorm) / W[k];
        Wmx[j] = 1.0 / acc;
        double sw = 0.0;
        for (int k = 0; k < S; ++k) sw = sw + split[(size_t)(2 + k) * N + j] / W[k];
        sW[j] = sw;
    }
}

int oracle_convection_flame(const oracle_conv_flame* fl, int S, const double* W, const double* x,
                            const double* y_left, double t0, double tf, const double* drhodt, const double* split,
                            double* state, const oracle_conv_options* o, int* status, int* stats,
                            int* n_history_out, double* hist_t_out, double* hist_v_out, double* v_last,
                            double* rv_last) {
    const int N = fl->n_points;
    double* hh = (double*)calloc((size_t)N, sizeof(double));
    double* rph = (double*)calloc((size_t)N, sizeof(double));
    double* Wmx = (double*)calloc((size_t)N, sizeof(double));
    double* sW = (double*)calloc((size_t)N, sizeof(double));
    double* rho = (double*)calloc((size_t)N, sizeof(double));
    double* rV = (double*)calloc((size_t)N, sizeof(double));
    double* V = (double*)calloc((size_t)N, sizeof(double));
    double* y3 = (double*)calloc((size_t)3 * N, sizeof(double));
    double* yd3 = (double*)calloc((size_t)3 * N, sizeof(double));
    double* at3 = (double*)calloc((size_t)3 * N, sizeof(double));
    double* atN = (double*)calloc((size_t)N, sizeof(double));
    double* ht = (double*)calloc((size_t)o->max_history, sizeof(double));
    double* hv = (double*)calloc((size_t)o->max_history * N, sizeof(double));
    oracle_convection_grid(N, x, fl->alpha, hh, rph);
    oracle_convection_prepare(N, S, W, state, split, Wmx, sW);
    for (int j = 0; j < N; ++j) {
        y3[3 * j + 0] = state[j];
        y3[3 * j + 1] = state[(size_t)N + j];
        y3[3 * j + 2] = Wmx[j];
        at3[3 * j + 0] = o->abstol_u;
        at3[3 * j + 1] = o->abstol_t;
        at3[3 * j + 2] = 20.0 * o->abstol_y;
        atN[j] = o->abstol_y;
    }
    utw_ctx uc = {{utw_f, utw_on_step, 3 * N, 256}, fl, N, x, hh, rph, drhodt, split, split + N, sW,
                  rho, rV, V, o->max_history, 0, 0, ht, hv};
    /* the record starts with V / rho of the initial state */
    oracle_convection_utw_rhs(fl, x, hh, rph, t0, y3, drhodt, split, split + N, sW, yd3, rho, rV, V);
    utw_record(&uc, t0);
    int st[4] = {0, 0, 0, 0};
    int rc = adams_integrate(&uc.base, y3, at3, o->reltol, t0, tf, 1, o->min_step, o->max_steps, st);
    if (uc.overflow) rc = -20;
    status[0] = rc;
    if (stats) {
        stats[0] = st[0];
        stats[1] = st[1];
        stats[2] = 0;
        stats[3] = 0;
    }
    for (int j = 0; j < N; ++j) {
        state[j] = y3[3 * j + 0];
        state[(size_t)N + j] = y3[3 * j + 1];
    }
    /* V and rV of the last right-hand side evaluation (ConvectionSystemUTW's
       members after the stage: the next step's continuity point reads them) */
    if (v_last) memcpy(v_last, V, sizeof(double) * N);
    if (rv_last) memcpy(rv_last, rV, sizeof(double) * N);
    if (n_history_out) *n_history_out = uc.n_history;
    if (hist_t_out) memcpy(hist_t_out, ht, sizeof(double) * uc.n_history);
    if (hist_v_out) memcpy(hist_v_out, hv, sizeof(double) * (size_t)uc.n_history * N);
    for (int k = 0; k < S; ++k) {
        if (rc != 0) {
            status[1 + k] = rc;
            continue;
        }
        spec_ctx sc = {{spec_f, NULL, N, 32}, fl, N, x, hh, split + (size_t)(2 + k) * N, y_left[k], uc.n_history, ht, hv};
        int sst[4] = {0, 0, 0, 0};
        status[1 + k] =
            adams_integrate(&sc.base, state + (size_t)(2 + k) * N, atN, o->reltol, t0, tf, 0, o->min_step,
                            o->max_steps, sst);
        if (stats) {
            stats[2] += sst[0];
            stats[3] += sst[1];
        }
    }
    free(hh);
    free(rph);
    free(Wmx);
    free(sW);
    free(rho);
    free(rV);
    free(V);
    free(y3);
    free(yd3);
    free(at3);
    free(atN);
    free(ht);
    free(hv);
    return rc;
}

static double ddt_sum(size_t e, int balanced, const double* c, const double* d, const double* p, const double* x) {
    double v = (c[e] + d[e]) + p[e];
    if (balanced && x) v = v + x[e];
    return v;
}

/* FlameSolver::prepareIntegrators' density derivative for the convection
 * stage (src/flameSolver.cpp:208-212), point-major [n_pts][n] arrays:
 * ddt = ddtConv + ddtDiff + ddtProd (+ ddtCross when balanced),
 * drho/dt = -rho (ddt_T / T + W sum_k ddt_Yk / W_k) with rho and the mean
 * molecular weight W of the state (mass fractions clipped at zero and
 * normalised; sums in species order). */
void oracle_convection_drhodt(int n_pts, int n, int balanced, double pressure, const double* W, const double* state,
                              const double* ddt_conv, const double* ddt_diff, const double* ddt_prod,
                              const double* ddt_cross, double* drhodt) {
    for (int p = 0; p < n_pts; ++p) {
        const double* s = state + (size_t)p * n;
        const size_t e0 = (size_t)p * n;
        double ysum = 0.0;
        for (int k = 2; k < n; ++k) ysum = ysum + (s[k] < 0.0 ? 0.0 : s[k]);
        const double rnorm = 1.0 / ysum;
        double acc = 0.0;
        for (int k = 2; k < n; ++k) acc = acc + ((s[k] < 0.0 ? 0.0 : s[k]) * rnorm) / W[k - 2];
        const double wmx = 1.0 / acc;
        const double T = s[1];
        const double rho = (pressure * wmx) / (GAS_CONSTANT * T);
        double tmp = 0.0;
        for (int k = 2; k < n; ++k) tmp = tmp + ddt_sum(e0 + k, balanced, ddt_conv, ddt_diff, ddt_prod, ddt_cross) / W[k - 2];
        drhodt[p] = -rho * (ddt_sum(e0 + 1, balanced, ddt_conv, ddt_diff, ddt_prod, ddt_cross) / T + tmp * wmx);
    }
}
