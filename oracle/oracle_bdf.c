/*
 * CPU ORACLE -- test infrastructure only (see oracle_tridiag.c).
 *
 * The CVODE source-term path of the reference: SourceSystemCVODE::f
 * (src/sourceSystem.cpp:128-164) integrated by CVODE in BDF mode with a
 * dense direct linear solver (src/sundialsUtils.cpp:33-172; maxNumSteps 1e6,
 * scalar rtol, vector atol for U / T / Y, minStep; integrateToTime steps past
 * the output time and interpolates back, CV_NORMAL).
 *
 * SUNDIALS is absent here; this restates the published method: a
 * variable-step, variable-order (1-5) BDF in Nordsieck form with the array
 * rescaled on step-size changes (the LSODE/EPISODE form: Byrne & Hindmarsh
 * 1975, Hindmarsh 1983), with CVODE's documented Newton iteration (modified
 * Newton on M = I - gamma J, convergence-rate estimate with factor 0.3,
 * divergence test, at most 3 iterations, test constant 0.1), WRMS norm with
 * weights 1/(rtol|y|+atol), local error test, step/order selection from the
 * error estimates at orders q-1, q, q+1 (safety factors 6, 6, 10), failure
 * handling (step x0.25 after a convergence failure, up to 10; error-test
 * failures: eta from the estimate, order 1 and x0.1 after 3, give up after
 * 7) and Jacobian / iteration-matrix reuse (new M every 20 steps or when
 * gamma moves by more than 30%, new Jacobian every 51 steps or after a
 * failure with a stale one) (Hindmarsh et al., ACM TOMS 31, 2005; CVODE
 * user guide, "Mathematical considerations"). The Jacobian is analytic in
 * the species (mass action, third-body and falloff [M] terms; the falloff
 * F factor is held fixed) with a forward-difference temperature column --
 * the reference differences every column (fdJacobian, sourceSystem.cpp:
 * 268-293); the Jacobian only steers the Newton iteration.
 *
 * Parity: unpinned against the reference (CVODE is absent); checked in the
 * tests against a tight implicit Runge-Kutta solution (scipy Radau).
 * Operation order matches the GPU code (ember_gb300/csrc/bdf.cu) so the two
 * agree bitwise.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

#define GAS_CONSTANT (6.02214076e26 * 1.380649e-23)
#define QMAX 5

static double dmaxb(double a, double b) { return (a < b) ? b : a; }
static double dminb(double a, double b) { return (b < a) ? b : a; }

/* Reduction order of the GPU block (see oracle_chem.c). */
double oracle_block_sum(const double* a, const double* b, int n, int W);
int oracle_reduction_width(int S);

typedef struct {
    const oracle_mech* m;
    const oracle_source_options* o;
    oracle_ws* w;
    const double* split;
    double x;
    double A, B;       /* sum Y/W and sum Y cp_R / W of the last call */
    double rho, cp, qdot;
} bdf_ode;

/* SourceSystemCVODE::f (src/sourceSystem.cpp:128-164): ydot of [U, T, Y]. */
static void bdf_f(bdf_ode* ode, double t, const double* y, double* ydot) {
    const oracle_mech* m = ode->m;
    oracle_ws* w = ode->w;
    const int S = m->S, W = oracle_reduction_width(S);
    double rho, cp;
    oracle_rates(m, w, ode->o->pressure, ode->o->kinetics_model, ORACLE_STATE_NO_NORM, y[1], y + 2, &rho, &cp);
    for (int k = 0; k < S; ++k) w->tmp[k] = w->wn[k];
    double qdot = -oracle_block_sum(w->tmp, w->hk, S, W);
    if (ode->o->ignition_energy != 0.0) {
        const double ti = ode->o->ignition_tstart;
        if (t >= ti && t < ti + ode->o->ignition_duration) {
            const double pi = 3.14159265358979323846, dx = ode->x - ode->o->ignition_center;
            qdot += ode->o->ignition_energy / (ode->o->ignition_stddev * sqrt(2 * pi) * ode->o->ignition_duration) *
                    oracle_exp(-(dx * dx) / (2 * (ode->o->ignition_stddev * ode->o->ignition_stddev)));
        }
    }
    const double* sc = ode->split;
    const double rrho = 1.0 / rho;
    ydot[0] = sc ? sc[0] : 0.0;
    ydot[1] = fma(qdot, 1.0 / (rho * cp), sc ? sc[1] : 0.0);
    for (int k = 0; k < S; ++k) ydot[2 + k] = fma(w->wn[k] * m->W[k], rrho, sc ? sc[2 + k] : 0.0);
    ode->rho = rho;
    ode->cp = cp;
    ode->qdot = qdot;
}

/* Weighted RMS norm sqrt(sum (v_i w_i)^2 / n) in the GPU reduction order. */
static double wrms(const double* v, const double* ewt, int n, double* tmp) {
    for (int i = 0; i < n; ++i) tmp[i] = v[i] * ewt[i];
    return sqrt(oracle_block_sum(tmp, tmp, n, oracle_reduction_width(n - 2)) / n);
}

/* ---- analytic Jacobian ------------------------------------------------ */

/* J (row-major n x n) of f at y; f0 = f(y) (with ode->rho/cp/qdot and the
 * rates in ode->w from that call). Uses ws: Jc (S x S), scratch. */
static void bdf_jacobian(bdf_ode* ode, double t, const double* y, const double* f0, double* J, double* Jc,
                         double* ycopy, double* f1) {
    const oracle_mech* m = ode->m;
    oracle_ws* w = ode->w;
    const int S = m->S, n = S + 2, Wd = oracle_reduction_width(S);
    const double T = y[1];
    const double A = 1.0 / w->mmw;                                     /* sum Y/W */
    for (int k = 0; k < S; ++k) w->tmp[k] = y[2 + k] * m->rW[k];
    const double B = oracle_block_sum(w->tmp, w->cp_R, S, Wd);          /* sum Y cp_R / W */
    const double rho = ode->rho, rc = rho * ode->cp;
    /* dwdot/dc (S x S), rows k: sum over reactions of nu_k * d(rop)/dc_j */
    memset(Jc, 0, sizeof(double) * S * S);
    for (int k = 0; k < S; ++k) w->jdense[k] = 0.0;
    for (int i = 0; i < m->R; ++i) {
        const int ty = m->type[i];
        const int* rc_ = m->reac + i * ORACLE_MAX_STOICH;
        const int* pd = m->prod + i * ORACLE_MAX_STOICH;
        const int fall = (ty == ORACLE_RXN_LINDEMANN || ty == ORACLE_RXN_TROE);
        double rf = (fall ? w->kf_fall[i] : w->kf[i]) * m->mult[i];
        double pf = 1.0, pp = 1.0;
        for (int o = 0; o < ORACLE_MAX_STOICH; ++o)
            if (rc_[o] >= 0) pf *= w->c[rc_[o]];
        if (m->rev[i])
            for (int o = 0; o < ORACLE_MAX_STOICH; ++o)
                if (pd[o] >= 0) pp *= w->c[pd[o]];
        const double kr = m->rev[i] ? w->rkc[i] : 0.0;
        double dropdm = 0.0;                                             /* d rop / d[M] */
        if (ty == ORACLE_RXN_THREE_BODY) {
            dropdm = rf * (pf - kr * pp);
            rf = rf * w->concm[i];
        } else if (fall) {
            /* d/d[M] of kinf mult Pr/(1+Pr) F(Pr), Pr = k0 [M] / kinf */
            const double pr1 = 1.0 + w->pr_fall[i];
            const double k0m = w->k0_fall[i] * m->mult[i];
            dropdm = ((w->F_fall[i] * k0m) / (pr1 * pr1) + (k0m * (w->pr_fall[i] / pr1)) * w->dF_fall[i]) *
                     (pf - kr * pp);
        }
        /* derivative of the net rate of progress w.r.t. each species occurrence */
        double dv[2 * ORACLE_MAX_STOICH];
        int dj[2 * ORACLE_MAX_STOICH];
        int nd = 0;
        for (int o = 0; o < ORACLE_MAX_STOICH; ++o) {
            if (rc_[o] < 0) continue;
            double d = rf;
            for (int q = 0; q < ORACLE_MAX_STOICH; ++q)
                if (q != o && rc_[q] >= 0) d *= w->c[rc_[q]];
            dj[nd] = rc_[o];
            dv[nd++] = d;
        }
        if (m->rev[i]) {
            for (int o = 0; o < ORACLE_MAX_STOICH; ++o) {
                if (pd[o] < 0) continue;
                double d = rf * kr;
                for (int q = 0; q < ORACLE_MAX_STOICH; ++q)
                    if (q != o && pd[q] >= 0) d *= w->c[pd[q]];
                dj[nd] = pd[o];
                dv[nd++] = -d;
            }
        }
        /* rows of the species of the reaction: +1 per product, -1 per reactant occurrence */
        for (int side = 0; side < 2; ++side) {
            const int* lst = side == 0 ? pd : rc_;
            const double sgn = side == 0 ? 1.0 : -1.0;
            for (int o = 0; o < ORACLE_MAX_STOICH; ++o) {
                const int k = lst[o];
                if (k < 0) continue;
                double* row = Jc + (size_t)k * S;
                for (int e = 0; e < nd; ++e) row[dj[e]] = fma(sgn, dv[e], row[dj[e]]);
                if (ty != ORACLE_RXN_ELEMENTARY) {
                    const double de = m->def_eff[i];
                    /* d[M]/dc_j = de for every j, plus (eff - de) for the listed species */
                    w->jdense[k] = fma(sgn * dropdm, de, w->jdense[k]);
                    for (int64_t e = m->eff_off[i]; e < m->eff_off[i + 1]; ++e)
                        row[m->eff_sp[e]] = fma(sgn * dropdm, m->eff_val[e] - de, row[m->eff_sp[e]]);
                }
            }
        }
    }
    /* chain rule to mass fractions; rows 2+k, columns 2+m (sums sequential in
     * the summation index, as one GPU thread per row / column computes them) */
    memset(J, 0, sizeof(double) * n * n);
    const double p = ode->o->pressure, RT = GAS_CONSTANT * T;
    const double rtp = RT / p;
    for (int k = 0; k < S; ++k) {
        double* row = Jc + (size_t)k * S;
        const double dk = w->jdense[k];
        for (int j = 0; j < S; ++j) row[j] += dk;
        double s_k = 0.0;                                                /* sum_j Jc[k][j] c_j */
        for (int j = 0; j < S; ++j) s_k = fma(row[j], w->c[j], s_k);
        const double sA = s_k / A;
        for (int mm = 0; mm < S; ++mm) row[mm] = (rho * row[mm] - sA) * m->rW[mm];   /* d wdot_k / dY_m */
    }
    const double wr = 1.0 / rho;
    for (int k = 0; k < S; ++k) {
        const double a = m->W[k] * wr, b = (w->wn[k] * m->W[k]) * rtp;
        for (int mm = 0; mm < S; ++mm)
            J[(size_t)(2 + k) * n + 2 + mm] = fma(a, Jc[(size_t)k * S + mm], b * m->rW[mm]);
    }
    /* energy row: dfT/dY_m = (-sum_k h_k dw_k/dY_m)/(rho cp) - qdot/(rho cp)^2 d(rho cp)/dY_m */
    const double rrc = 1.0 / rc, qrc2 = ode->qdot / (rc * rc), pT = p / T;
    for (int mm = 0; mm < S; ++mm) {
        double hsum = 0.0;
        for (int k = 0; k < S; ++k) hsum = fma(Jc[(size_t)k * S + mm], w->hk[k], hsum);
        const double drc = pT * ((w->cp_R[mm] * m->rW[mm]) / A - (B * m->rW[mm]) / (A * A));
        J[(size_t)1 * n + 2 + mm] = -hsum * rrc - qrc2 * drc;
    }
    /* temperature column by forward difference (dy = |T| sqrt(eps), as fdJacobian) */
    memcpy(ycopy, y, sizeof(double) * n);
    const double dT = fabs(T) * 1.4901161193847656e-08;
    ycopy[1] = T + dT;
    bdf_ode tmp_ode = *ode;
    bdf_f(&tmp_ode, t, ycopy, f1);
    const double rdT = 1.0 / ((T + dT) - T);
    for (int i = 0; i < n; ++i) J[(size_t)i * n + 1] = (f1[i] - f0[i]) * rdT;
}

/* ---- dense LU with partial pivoting ----------------------------------- */

/* In place on row-major M (n x n); pivot row = first maximum of |a_ik|.
 * Multipliers are a_ik * (1/a_kk); the reciprocals 1/a_kk of the pivots are
 * kept in rdiag for the back substitution. Returns 0, or k+1 when column k
 * has no usable pivot (all zeros, or a NaN anywhere in it). */
static int lu_factor(double* M, int* piv, double* rdiag, int n) {
    for (int k = 0; k < n; ++k) {
        int p = k;
        double best = fabs(M[(size_t)k * n + k]);
        int has_nan = best != best;
        for (int i = k + 1; i < n; ++i) {
            const double v = fabs(M[(size_t)i * n + k]);
            if (v != v) has_nan = 1;
            if (v > best) {
                best = v;
                p = i;
            }
        }
        piv[k] = p;
        if (has_nan || best == 0.0) return k + 1;
        if (p != k)
            for (int j = 0; j < n; ++j) {
                const double t = M[(size_t)k * n + j];
                M[(size_t)k * n + j] = M[(size_t)p * n + j];
                M[(size_t)p * n + j] = t;
            }
        const double r = 1.0 / M[(size_t)k * n + k];
        rdiag[k] = r;
        for (int i = k + 1; i < n; ++i) M[(size_t)i * n + k] *= r;
        for (int i = k + 1; i < n; ++i) {
            const double l = M[(size_t)i * n + k];
            for (int j = k + 1; j < n; ++j) M[(size_t)i * n + j] = fma(-l, M[(size_t)k * n + j], M[(size_t)i * n + j]);
        }
    }
    return 0;
}

/* Forward and back substitution (SUNDIALS' dense getrs) with the factors of
 * lu_factor. The back substitution multiplies by the pivot reciprocal the
 * factorisation computed, where getrs divides by the pivot (one rounding of
 * 1/a_kk more; a division costs about eight times a multiply on the GPU). */
static void lu_solve(const double* M, const int* piv, const double* rdiag, int n, double* b) {
    for (int k = 0; k < n; ++k)
        if (piv[k] != k) {
            const double t = b[k];
            b[k] = b[piv[k]];
            b[piv[k]] = t;
        }
    for (int k = 0; k < n; ++k)
        for (int i = k + 1; i < n; ++i) b[i] = fma(-M[(size_t)i * n + k], b[k], b[i]);
    for (int k = n - 1; k >= 0; --k) {
        b[k] = b[k] * rdiag[k];
        for (int i = 0; i < k; ++i) b[i] = fma(-M[(size_t)i * n + k], b[k], b[i]);
    }
}

/* ---- the integrator --------------------------------------------------- */

/* l_j: coefficients of prod_{i=1..q} (1 + x/i) (constant-step BDF of order q). */
static void bdf_l(int q, double* l) {
    for (int j = 0; j <= QMAX + 1; ++j) l[j] = 0.0;
    l[0] = 1.0;
    for (int i = 1; i <= q; ++i) {
        const double ri = 1.0 / i;
        for (int j = i; j >= 1; --j) l[j] = fma(l[j - 1], ri, l[j]);
    }
}

static double bdf_pow(double x, double e) { return oracle_exp(e * oracle_log(x)); }

int oracle_bdf_point(const oracle_mech* m, oracle_ws* w, const oracle_source_options* o, double* yio,
                     const double* split, double tf, double t_start, double xpos, int* stats) {
    const int S = m->S, n = S + 2;
    /* work arrays */
    double* buf = (double*)calloc((size_t)n * (24 + (QMAX + 1) * 2) + (size_t)S * S + (size_t)2 * n * n, sizeof(double));
    double* z[QMAX + 2];
    double* zs[QMAX + 2];
    for (int j = 0; j <= QMAX + 1; ++j) {
        z[j] = buf + (size_t)j * n;
        zs[j] = buf + (size_t)(QMAX + 2 + j) * n;
    }
    double* base = buf + (size_t)(2 * (QMAX + 2)) * n;
    double *acor = base, *acorp = base + n, *ewt = base + 2 * n, *y = base + 3 * n, *ft = base + 4 * n;
    double *bb = base + 5 * n, *tmp = base + 6 * n, *f0 = base + 7 * n, *ycopy = base + 8 * n, *f1 = base + 9 * n;
    double* Jc = base + 10 * n;
    double* J = Jc + (size_t)S * S;
    double* M = J + (size_t)n * n;
    int* piv = (int*)malloc(sizeof(int) * n);
    double* rdiag = (double*)malloc(sizeof(double) * n);
    double atol[2];
    atol[0] = o->bdf_abstol_momentum;
    atol[1] = o->bdf_abstol_energy;
    bdf_ode ode = {m, o, w, split, xpos, 0, 0, 1, 1, 0};

    const double rtol = o->bdf_reltol, hmin = o->bdf_min_step;
    const double uround = 2.220446049250313e-16;
    int nst = 0, nfe = 0, nje = 0, nsetups = 0, nef_total = 0, ncf_total = 0;
    int status = 0;

#define ATOL(i) ((i) == 0 ? atol[0] : ((i) == 1 ? atol[1] : o->bdf_abstol_species))
#define SET_EWT(v)                                                                  \
    for (int i = 0; i < n; ++i) ewt[i] = 1.0 / (rtol * fabs((v)[i]) + ATOL(i));

    /* initial state and derivative */
    memcpy(z[0], yio, sizeof(double) * n);
    bdf_f(&ode, t_start, z[0], f0);
    nfe++;
    SET_EWT(z[0]);
    /* initial step: second-derivative estimate so that ||h^2/2 y''|| = 1 (own form
     * of CVODE's documented estimate), bounded by 0.1 of the interval and by
     * 0.1 |y|/|y'| componentwise */
    double t = 0.0;
    double hub = 0.1 * tf;
    double rmax = 0.0;
    for (int i = 0; i < n; ++i) {
        const double den = 0.1 * fabs(z[0][i]) + ATOL(i);
        rmax = dmaxb(rmax, fabs(f0[i]) / den);
    }
    if (rmax * hub > 1.0) hub = 1.0 / rmax;
    double hlb = 100.0 * uround * tf;
    double hg = sqrt(hlb * hub);
    double h = hg;
    if (hub > hlb) {
        for (int it = 0; it < 4; ++it) {
            for (int i = 0; i < n; ++i) ycopy[i] = fma(hg, f0[i], z[0][i]);
            bdf_f(&ode, t_start + hg, ycopy, f1);
            nfe++;
            for (int i = 0; i < n; ++i) tmp[i] = (f1[i] - f0[i]) / hg;
            const double ydd = wrms(tmp, ewt, n, bb);
            const double hnew = (ydd * hub * hub > 2.0) ? sqrt(2.0 / ydd) : sqrt(hg * hub);
            const double ratio = hnew / hg;
            hg = hnew;
            if (ratio > 0.5 && ratio < 2.0) break;
        }
        h = dminb(dmaxb(0.5 * hg, hlb), hub);
    } else {
        h = hlb;
    }
    if (h < hmin) h = hmin;
    for (int i = 0; i < n; ++i) z[1][i] = h * f0[i];

    int q = 1, qwait = 2, nstlp = 0, nstlj = 0, have_m = 0, have_acorp = 0, qsave = 0;
    double gammap = 0.0, crate = 1.0, etamax = 10000.0, acnrm = 0.0, hsave = 0.0;
    double l[QMAX + 2];

    while (t < tf) {
        if (nst >= o->bdf_max_num_steps) {
            status = -11;
            break;
        }
        /* save the Nordsieck array for retries */
        for (int j = 0; j <= q; ++j) memcpy(zs[j], z[j], sizeof(double) * n);
        int ncf = 0, nef = 0, convfail_bad_j = 0, force_setup = !have_m;
        double dsm = 0.0;
        for (;;) {
            /* predict */
            for (int k = 1; k <= q; ++k)
                for (int j = q; j >= k; --j)
                    for (int i = 0; i < n; ++i) z[j - 1][i] += z[j][i];
            const double tn = t + h;
            bdf_l(q, l);
            const double cq = 1.0 / ((q + 1) * l[1]);   /* error constant, order q */
            const double gamma = h / l[1];
            const double tq4 = 0.1 / cq;
            /* iteration matrix */
            int jcur = 0;
            const double gamrat0 = have_m ? gamma / gammap : 1.0;
            if (force_setup || nst >= nstlp + 20 || fabs(gamrat0 - 1.0) > 0.3) {
                const int jbad = (nst == 0) || (nst >= nstlj + 51) || convfail_bad_j || !have_m;
                if (jbad) {
                    bdf_f(&ode, t_start + tn, z[0], ft);
                    nfe++;
                    bdf_jacobian(&ode, t_start + tn, z[0], ft, J, Jc, ycopy, f1);
                    nfe += 1;
                    nje++;
                    nstlj = nst;
                    jcur = 1;
                }
                for (int i = 0; i < n; ++i)
                    for (int j = 0; j < n; ++j)
                        M[(size_t)i * n + j] = (i == j ? 1.0 : 0.0) - gamma * J[(size_t)i * n + j];
                const int sing = lu_factor(M, piv, rdiag, n);
                nsetups++;
                gammap = gamma;
                nstlp = nst;
                crate = 1.0;
                have_m = !sing;
                force_setup = 0;
                convfail_bad_j = 0;
                if (sing) {
                    /* singular iteration matrix: treated as a convergence failure */
                    goto conv_fail;
                }
            }
            {
                const double gamrat = gamma / gammap;
                /* Newton iteration on acor, y = z0 + acor */
                memset(acor, 0, sizeof(double) * n);
                memcpy(y, z[0], sizeof(double) * n);
                double delp = 0.0, del = 0.0;
                int converged = 0;
                const double rl1 = 1.0 / l[1];
                for (int mit = 0; mit < 3; ++mit) {
                    bdf_f(&ode, t_start + tn, y, ft);
                    nfe++;
                    for (int i = 0; i < n; ++i) bb[i] = gamma * ft[i] - fma(rl1, z[1][i], acor[i]);
                    lu_solve(M, piv, rdiag, n, bb);
                    if (gamrat != 1.0) {
                        const double sc = 2.0 / (1.0 + gamrat);
                        for (int i = 0; i < n; ++i) bb[i] *= sc;
                    }
                    del = wrms(bb, ewt, n, tmp);
                    for (int i = 0; i < n; ++i) {
                        acor[i] += bb[i];
                        y[i] = z[0][i] + acor[i];
                    }
                    if (mit > 0) crate = dmaxb(0.3 * crate, del / delp);
                    const double dcon = del * dminb(1.0, crate) / tq4;
                    if (dcon <= 1.0) {
                        acnrm = (mit == 0) ? del : wrms(acor, ewt, n, tmp);
                        converged = 1;
                        break;
                    }
                    if (mit >= 1 && del > 2.0 * delp) break;
                    delp = del;
                }
                if (!converged) goto conv_fail;
            }
            /* local error test */
            dsm = acnrm * cq;
            if (dsm <= 1.0) break;  /* step accepted */
            /* error-test failure */
            nef++;
            nef_total++;
            for (int j = 0; j <= q; ++j) memcpy(z[j], zs[j], sizeof(double) * n);
            if (nef >= 7 || h <= hmin * 1.0000000000000002) {
                status = -13;
                goto done;
            }
            {
                double eta;
                if (nef <= 3) {
                    eta = 1.0 / (bdf_pow(6.0 * dsm, 1.0 / (q + 1)) + 1e-6);
                    eta = dmaxb(0.1, dmaxb(eta, hmin / h));
                    if (nef >= 2) eta = dminb(eta, 0.2);
                    double s = eta;
                    for (int j = 1; j <= q; ++j) {
                        for (int i = 0; i < n; ++i) z[j][i] *= s;
                        s *= eta;
                    }
                    h *= eta;
                } else {
                    /* restart at order 1 with a tenth of the step */
                    eta = dmaxb(0.1, hmin / h);
                    h *= eta;
                    q = 1;
                    bdf_f(&ode, t_start + t, z[0], ft);
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
            ncf_total++;
            if (!jcur && have_m) {
                /* retry the step with a fresh Jacobian */
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
                const double eta = dmaxb(0.25, hmin / h);
                double s = eta;
                for (int j = 1; j <= q; ++j) {
                    for (int i = 0; i < n; ++i) z[j][i] *= s;
                    s *= eta;
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
        t += h;
        for (int j = 0; j <= q; ++j)
            for (int i = 0; i < n; ++i) z[j][i] = fma(l[j], acor[i], z[j][i]);
        SET_EWT(z[0]);
        /* step size and order for the next step (CVODE's order-selection
         * rhythm: the order may change after q+1 steps at the current order;
         * the correction of the step before is saved one step ahead and
         * rescaled by (h/h_saved)^(q+1) for the order q+1 estimate) */
        const double etaq = 1.0 / (bdf_pow(6.0 * dsm, 1.0 / (q + 1)) + 1e-6);
        double eta = etaq;
        int qnew = q;
        qwait--;
        if (qwait == 0) {
            double etaqm1 = 0.0, etaqp1 = 0.0;
            if (q > 1) {
                double lm[QMAX + 2];
                bdf_l(q - 1, lm);
                /* order q-1: error ~ h^q y^(q) / (q l1(q-1)) with h^q y^(q) = q! z_q */
                double fact = 1.0;
                for (int i = 2; i <= q; ++i) fact *= i;
                const double ddn = wrms(z[q], ewt, n, tmp) * (fact / (q * lm[1]));
                etaqm1 = 1.0 / (bdf_pow(6.0 * ddn, 1.0 / q) + 1e-6);
            }
            if (q < QMAX && have_acorp && qsave == q) {
                double lp[QMAX + 2];
                bdf_l(q + 1, lp);
                const double cq = bdf_pow(h / hsave, (double)(q + 1));
                for (int i = 0; i < n; ++i) tmp[i] = fma(-cq, acorp[i], acor[i]);
                const double dup = wrms(tmp, ewt, n, bb) / ((q + 2) * lp[1]);
                etaqp1 = 1.0 / (bdf_pow(10.0 * dup, 1.0 / (q + 2)) + 1e-6);
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
        } else if (qwait == 1 && q < QMAX) {
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
            eta = dminb(eta, etamax);
            if (h * eta < hmin) eta = hmin / h;
        }
        if (qnew > q) {
            /* new column z_{q+1} = acor l_q / (q+1) */
            const double c = l[q] / (q + 1);
            for (int i = 0; i < n; ++i) z[q + 1][i] = acor[i] * c;
        }
        if (qnew != q) {
            q = qnew;
            qwait = q + 1;
            have_acorp = 0;
        }
        if (eta != 1.0) {
            double s = eta;
            for (int j = 1; j <= q; ++j) {
                for (int i = 0; i < n; ++i) z[j][i] *= s;
                s *= eta;
            }
            h *= eta;
        }
        etamax = 10.0;
    }
    /* interpolate the solution at tf from the Nordsieck array (CV_NORMAL) */
    if (status == 0) {
        const double s = (tf - t) / h;
        for (int i = 0; i < n; ++i) {
            double v = z[q][i];
            for (int j = q - 1; j >= 0; --j) v = fma(v, s, z[j][i]);
            yio[i] = v;
        }
    } else {
        memcpy(yio, z[0], sizeof(double) * n);
    }
done:
    if (status != 0) memcpy(yio, z[0], sizeof(double) * n);
    if (stats) {
        stats[0] = nst;
        stats[1] = nfe;
        stats[2] = nef_total + ncf_total;
        stats[3] = nje;
    }
    (void)nsetups;
    free(piv);
    free(rdiag);
    free(buf);
    return status;
#undef ATOL
#undef SET_EWT
}
