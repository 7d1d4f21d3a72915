/*
 * CPU ORACLE -- test infrastructure only (see oracle_tridiag.c).
 *
 * Plain-C restatement of the chemistry source term of the reference:
 *   SourceSystemQSS::odefun / setState / setOptions  src/sourceSystem.cpp:403-531
 *   QssIntegrator (setState, getInitialStepSize,
 *     integrateToTime, integrateOneStep)            src/qssintegrator.cpp:9-265
 *   SourceSystemCVODE::f                            src/sourceSystem.cpp:128-164
 *   SourceSystem::updateThermo / getQdotIgniter     src/sourceSystem.cpp:24-45
 *   InterpKinetics::updateROP tables                src/chemistry0d.cpp:271-357
 *   MultiArrheniusInterp::rebuildInterpData/update  src/chemistry0d.cpp:401-436, chemistry0d.h:140-163
 * and of the Cantera 3.2 calls they make (the library is absent here; its
 * published formulas are restated): ideal-gas state setters
 * (setState_TPY normalises Y after clipping negative values to zero;
 * setMassFractions_NoNorm does not), NASA7 polynomials, modified Arrhenius
 * rates, third-body efficiencies, Lindemann and Troe falloff, reverse rates
 * from the equilibrium constant Kc = exp(-dG0/RT) (p0/RT)^dn, creation /
 * destruction / net production rates.
 *
 * Parity: the QSS integrator is pinned by the CHEMEQ2 cesium test problem of
 * test/old/test_qssintegrator.cpp. The kinetics/thermo restatement is
 * PARITY UNPINNED: the reference's tests hold no rates, equilibrium constants
 * or thermo values, and Cantera and its mechanism files are absent.
 *
 * Sums over species use one fixed order (see block_sum), the order of the
 * GPU block reductions; the reference leaves this order to Eigen. Where the
 * GPU code fuses a multiply-add, this file writes the same fma().
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

#define GAS_CONSTANT (6.02214076e26 * 1.380649e-23)
#define ONE_ATM 101325.0
#define BIG_NUMBER 1e300
#define SMALL_NUMBER 1e-300

/* ---- exp / log (same method and constants as the product's device code:
 * Cody-Waite reduction + degree-13 Taylor; log via 2 atanh(s) series) ---- */

static double pow2i(int k) {
    uint64_t b = (uint64_t)(k + 1023) << 52;
    double d;
    memcpy(&d, &b, sizeof d);
    return d;
}

double oracle_exp(double x) {
    if (x != x) return x;
    if (x > 709.782712893384) return INFINITY;
    if (x < -745.1332191019412) return 0.0;
    const double kd = rint(x * 1.4426950408889634);
    double r = fma(-kd, 0.6931471805599453, x);
    r = fma(-kd, 2.3190468138462996e-17, r);
    double p = 1.6059043836821613e-10;
    p = fma(p, r, 2.08767569878681e-09);
    p = fma(p, r, 2.505210838544172e-08);
    p = fma(p, r, 2.755731922398589e-07);
    p = fma(p, r, 2.7557319223985893e-06);
    p = fma(p, r, 2.48015873015873e-05);
    p = fma(p, r, 0.0001984126984126984);
    p = fma(p, r, 0.001388888888888889);
    p = fma(p, r, 0.008333333333333333);
    p = fma(p, r, 0.041666666666666664);
    p = fma(p, r, 0.16666666666666666);
    p = fma(p, r, 0.5);
    p = fma(p, r, 1.0);
    p = fma(p, r, 1.0);
    int k = (int)kd;
    if (k > 1023) return (p * pow2i(1023)) * pow2i(k - 1023);
    if (k < -1022) return (p * pow2i(k + 1000)) * pow2i(-1000);
    return p * pow2i(k);
}

double oracle_log(double x) {
    if (!(x > 0.0)) return x == 0.0 ? -INFINITY : NAN;
    uint64_t bits;
    memcpy(&bits, &x, sizeof bits);
    if (bits >= 0x7ff0000000000000ULL) return x;
    int e = 0;
    if (bits < 0x0010000000000000ULL) {
        x *= 18014398509481984.0;
        memcpy(&bits, &x, sizeof bits);
        e = -54;
    }
    e += (int)((bits >> 52) & 0x7ff) - 1023;
    uint64_t mb = (bits & 0x000fffffffffffffULL) | 0x3ff0000000000000ULL;
    double m;
    memcpy(&m, &mb, sizeof m);
    if (m > 1.4142135623730951) {
        m *= 0.5;
        e += 1;
    }
    const double s = (m - 1.0) / (m + 1.0);
    const double s2 = s * s;
    double q = 0.09523809523809523;
    q = fma(q, s2, 0.10526315789473684);
    q = fma(q, s2, 0.11764705882352941);
    q = fma(q, s2, 0.13333333333333333);
    q = fma(q, s2, 0.15384615384615385);
    q = fma(q, s2, 0.18181818181818182);
    q = fma(q, s2, 0.2222222222222222);
    q = fma(q, s2, 0.2857142857142857);
    q = fma(q, s2, 0.4);
    q = fma(q, s2, 0.6666666666666666);
    const double t = fma(s, s2 * q, 2.0 * s);
    const double ed = (double)e;
    return fma(ed, 0.6931471805599453, fma(ed, 2.3190468138462996e-17, t));
}

static double oracle_log10(double x) { return oracle_log(x) * 0.4342944819032518; }
static double oracle_exp10(double x) { return oracle_exp(x * 2.302585092994046); }

static double dmax(double a, double b) { return (a < b) ? b : a; } /* std::max */
static double dmin(double a, double b) { return (b < a) ? b : a; } /* std::min */

/* Width of the reduction order of the GPU kernels: 32 lanes, whatever the
 * number of threads per grid point. */
static int reduction_width(int S) {
    (void)S;
    return 32;
}

/* Sum of a[k] (b == NULL) or of a[k] * b[k] accumulated by fma, in the fixed
 * order of the GPU block reduction: element k goes to the partial sum of
 * lane k mod W (sequential in k; W = 32 for the kernels); the W partials are
 * folded into 32 as p[l] + p[l+32] + p[l+64] + ... (in that order) and
 * combined by an xor butterfly. */
double oracle_block_sum(const double* a, const double* b, int n, int W);
int oracle_reduction_width(int S) { return reduction_width(S); }
#define block_sum oracle_block_sum
double oracle_block_sum(const double* a, const double* b, int n, int W) {
    double p[256], q[32];
    for (int l = 0; l < W; ++l) p[l] = 0.0;
    for (int k = 0; k < n; ++k) p[k % W] = b ? fma(a[k], b[k], p[k % W]) : p[k % W] + a[k];
    for (int l = 0; l < 32; ++l) {
        double v = p[l];
        for (int w = 1; w < W / 32; ++w) v = v + p[l + 32 * w];
        q[l] = v;
    }
    for (int off = 16; off >= 1; off >>= 1) {
        double r[32];
        for (int l = 0; l < 32; ++l) r[l] = q[l] + q[l ^ off];
        memcpy(q, r, sizeof q);
    }
    return q[0];
}

/* ---- mechanism ------------------------------------------------------- */

oracle_mech* oracle_mech_create(const oracle_mech_desc* d) {
    oracle_mech* m = (oracle_mech*)calloc(1, sizeof(oracle_mech));
    const int S = d->n_species, R = d->n_reactions;
    m->S = S;
    m->R = R;
    m->W = (double*)malloc(sizeof(double) * S);
    m->rW = (double*)malloc(sizeof(double) * S);
    m->tmid = (double*)malloc(sizeof(double) * S);
    m->nasa = (double*)malloc(sizeof(double) * S * 14);
    m->hc = (double*)malloc(sizeof(double) * S * 10);
    m->sc = (double*)malloc(sizeof(double) * S * 8);
    memcpy(m->W, d->mol_weight, sizeof(double) * S);
    memcpy(m->tmid, d->nasa_tmid, sizeof(double) * S);
    memcpy(m->nasa, d->nasa_coeffs, sizeof(double) * S * 14);
    for (int k = 0; k < S; ++k) {
        m->rW[k] = 1.0 / m->W[k];
        for (int r = 0; r < 2; ++r) {
            const double* a = m->nasa + 14 * k + 7 * r;
            double* h = m->hc + 10 * k + 5 * r;
            double* s = m->sc + 8 * k + 4 * r;
            h[0] = a[0];
            h[1] = a[1] / 2.0;
            h[2] = a[2] / 3.0;
            h[3] = a[3] / 4.0;
            h[4] = a[4] / 5.0;
            s[0] = a[1];
            s[1] = a[2] / 2.0;
            s[2] = a[3] / 3.0;
            s[3] = a[4] / 4.0;
        }
    }
    m->type = (int*)malloc(sizeof(int) * R);
    m->rev = (int*)malloc(sizeof(int) * R);
    m->reac = (int*)malloc(sizeof(int) * R * ORACLE_MAX_STOICH);
    m->prod = (int*)malloc(sizeof(int) * R * ORACLE_MAX_STOICH);
    m->arr = (double*)malloc(sizeof(double) * R * 3);
    m->arr_low = (double*)malloc(sizeof(double) * R * 3);
    m->troe = (double*)malloc(sizeof(double) * R * 4);
    m->def_eff = (double*)malloc(sizeof(double) * R);
    m->eff_off = (int64_t*)malloc(sizeof(int64_t) * (R + 1));
    memcpy(m->type, d->rxn_type, sizeof(int) * R);
    memcpy(m->rev, d->reversible, sizeof(int) * R);
    memcpy(m->reac, d->reactants, sizeof(int) * R * ORACLE_MAX_STOICH);
    memcpy(m->prod, d->products, sizeof(int) * R * ORACLE_MAX_STOICH);
    memcpy(m->arr, d->arrhenius, sizeof(double) * R * 3);
    memcpy(m->arr_low, d->arrhenius_low, sizeof(double) * R * 3);
    memcpy(m->troe, d->troe, sizeof(double) * R * 4);
    memcpy(m->def_eff, d->default_efficiency, sizeof(double) * R);
    memcpy(m->eff_off, d->efficiency_offsets, sizeof(int64_t) * (R + 1));
    const int64_t ne = m->eff_off[R];
    m->eff_sp = (int*)malloc(sizeof(int) * (ne ? ne : 1));
    m->eff_val = (double*)malloc(sizeof(double) * (ne ? ne : 1));
    if (ne) {
        memcpy(m->eff_sp, d->efficiency_species, sizeof(int) * ne);
        memcpy(m->eff_val, d->efficiency_values, sizeof(double) * ne);
    }
    m->mult = (double*)malloc(sizeof(double) * R);
    m->dn = (double*)malloc(sizeof(double) * R);
    for (int i = 0; i < R; ++i) {
        m->mult[i] = 1.0;
        int np = 0, nr = 0;
        for (int o = 0; o < ORACLE_MAX_STOICH; ++o) {
            np += m->prod[i * ORACLE_MAX_STOICH + o] >= 0;
            nr += m->reac[i * ORACLE_MAX_STOICH + o] >= 0;
        }
        m->dn[i] = (double)(np - nr);
    }
    /* Interpolation tables of the 'interp' kinetics model: 200 nodes on
     * [273, 3500] K (chemistry0d.h:70-72, 171-173). */
    m->nT = 200;
    m->Tmin = 273.0;
    m->Tmax = 3500.0;
    m->kf_c = (double*)calloc((size_t)R * m->nT, sizeof(double));
    m->kf_s = (double*)calloc((size_t)R * m->nT, sizeof(double));
    m->kc_c = (double*)calloc((size_t)R * m->nT, sizeof(double));
    m->kc_s = (double*)calloc((size_t)R * m->nT, sizeof(double));
    oracle_ws* ws = oracle_ws_create(m);
    for (int n = 0; n < m->nT; ++n) {
        double T = m->Tmin + ((double)n) / (m->nT - 1) * (m->Tmax - m->Tmin);
        oracle_rate_constants(m, ws, T, 0);
        for (int i = 0; i < R; ++i) {
            m->kf_c[(size_t)i * m->nT + n] = ws->kf[i];
            m->kc_c[(size_t)i * m->nT + n] = ws->rkc[i];
        }
    }
    oracle_ws_free(ws);
    const double dT = (m->Tmax - m->Tmin) / (m->nT - 1);
    for (int i = 0; i < R; ++i) {
        double* kc = m->kf_c + (size_t)i * m->nT;
        double* ks = m->kf_s + (size_t)i * m->nT;
        double* cc = m->kc_c + (size_t)i * m->nT;
        double* cs = m->kc_s + (size_t)i * m->nT;
        for (int n = 0; n < m->nT - 1; ++n) {
            ks[n] = (kc[n + 1] - kc[n]) / dT;
            cs[n] = (cc[n + 1] - cc[n]) / dT;
        }
    }
    return m;
}

void oracle_mech_destroy(oracle_mech* m) {
    if (!m) return;
    free(m->W); free(m->rW); free(m->tmid); free(m->nasa); free(m->hc); free(m->sc);
    free(m->type); free(m->rev); free(m->reac); free(m->prod); free(m->arr); free(m->arr_low);
    free(m->troe); free(m->def_eff); free(m->eff_off); free(m->eff_sp); free(m->eff_val);
    free(m->mult); free(m->dn); free(m->kf_c); free(m->kf_s); free(m->kc_c); free(m->kc_s);
    free(m);
}

void oracle_mech_set_multipliers(oracle_mech* m, const double* mult) {
    for (int i = 0; i < m->R; ++i) m->mult[i] = mult ? mult[i] : 1.0;
}

oracle_ws* oracle_ws_create(const oracle_mech* m) {
    oracle_ws* w = (oracle_ws*)calloc(1, sizeof(oracle_ws));
    const int S = m->S, R = m->R, n = S + 2;
    w->cp_R = (double*)calloc(S, sizeof(double));
    w->h_RT = (double*)calloc(S, sizeof(double));
    w->g_RT = (double*)calloc(S, sizeof(double));
    w->c = (double*)calloc(S, sizeof(double));
    w->ym = (double*)calloc(S, sizeof(double));
    w->tmp = (double*)calloc(S > n ? S : n, sizeof(double));
    w->kf = (double*)calloc(R, sizeof(double));
    w->rkc = (double*)calloc(R, sizeof(double));
    w->ropf = (double*)calloc(R, sizeof(double));
    w->ropr = (double*)calloc(R, sizeof(double));
    w->wq = (double*)calloc(S, sizeof(double));
    w->wd = (double*)calloc(S, sizeof(double));
    w->wn = (double*)calloc(S, sizeof(double));
    w->hk = (double*)calloc(S, sizeof(double));
    w->v = (double*)calloc((size_t)n * 16, sizeof(double));
    w->kf_fall = (double*)calloc(R, sizeof(double));
    w->k0_fall = (double*)calloc(R, sizeof(double));
    w->F_fall = (double*)calloc(R, sizeof(double));
    w->pr_fall = (double*)calloc(R, sizeof(double));
    w->dF_fall = (double*)calloc(R, sizeof(double));
    w->concm = (double*)calloc(R, sizeof(double));
    w->jdense = (double*)calloc(S, sizeof(double));
    w->kT = NAN;
    return w;
}

void oracle_ws_free(oracle_ws* w) {
    if (!w) return;
    free(w->cp_R); free(w->h_RT); free(w->g_RT); free(w->c); free(w->ym); free(w->tmp);
    free(w->kf); free(w->rkc); free(w->ropf); free(w->ropr); free(w->wq); free(w->wd); free(w->wn);
    free(w->hk); free(w->v);
    free(w->kf_fall); free(w->k0_fall); free(w->F_fall); free(w->pr_fall); free(w->dF_fall); free(w->concm); free(w->jdense);
    free(w);
}

/* NASA7 cp/R, h/RT and g/RT = h/RT - s/R of every species at T. */
static void thermo(const oracle_mech* m, oracle_ws* w, double T) {
    const double lnT = oracle_log(T), rT = 1.0 / T;
    for (int k = 0; k < m->S; ++k) {
        const int r = (T <= m->tmid[k]) ? 0 : 1;
        const double* a = m->nasa + 14 * k + 7 * r;
        const double* h = m->hc + 10 * k + 5 * r;
        const double* s = m->sc + 8 * k + 4 * r;
        double cp = fma(fma(fma(fma(a[4], T, a[3]), T, a[2]), T, a[1]), T, a[0]);
        double hr = fma(fma(fma(fma(h[4], T, h[3]), T, h[2]), T, h[1]), T, h[0]) + a[5] * rT;
        double sp = fma(fma(fma(s[3], T, s[2]), T, s[1]), T, s[0]);
        double sr = fma(a[0], lnT, fma(sp, T, a[6]));
        w->cp_R[k] = cp;
        w->h_RT[k] = hr;
        w->g_RT[k] = hr - sr;
    }
}

static double arrhenius(const double* p, double lnT, double rT) {
    return p[0] * oracle_exp(fma(p[1], lnT, -(p[2] * rT)));
}

/* Rate constants (without the falloff part, which needs [M]) and reverse
 * factors 1/Kc at T. use_tables selects the interp model where T lies in
 * the tables' range. Also fills the thermo arrays at T. */
void oracle_rate_constants(const oracle_mech* m, oracle_ws* w, double T, int use_tables) {
    thermo(m, w, T);
    const double lnT = oracle_log(T), rT = 1.0 / T;
    const double lnRTp = oracle_log((GAS_CONSTANT * T) / ONE_ATM);  /* RT / p0 */
    const int in_table = use_tables && T >= m->Tmin && T <= m->Tmax;
    size_t n = 0;
    double dT = 0.0;
    if (in_table) {
        n = (size_t)floor((T - m->Tmin) / (m->Tmax - m->Tmin) * (m->nT - 1));
        if (n > (size_t)(m->nT - 1)) n = m->nT - 1;
        dT = T - n * (m->Tmax - m->Tmin) / (m->nT - 1) - m->Tmin;
    }
    for (int i = 0; i < m->R; ++i) {
        const int ty = m->type[i];
        if (ty == ORACLE_RXN_ELEMENTARY || ty == ORACLE_RXN_THREE_BODY) {
            if (in_table)
                w->kf[i] = fma(m->kf_s[(size_t)i * m->nT + n], dT, m->kf_c[(size_t)i * m->nT + n]);
            else
                w->kf[i] = arrhenius(m->arr + 3 * i, lnT, rT);
        } else {
            w->kf[i] = 0.0; /* falloff: evaluated with [M] */
        }
        if (!m->rev[i]) {
            w->rkc[i] = 0.0;
        } else if (in_table) {
            w->rkc[i] = fma(m->kc_s[(size_t)i * m->nT + n], dT, m->kc_c[(size_t)i * m->nT + n]);
        } else {
            double dg = 0.0;
            for (int o = 0; o < ORACLE_MAX_STOICH; ++o) {
                int k = m->prod[i * ORACLE_MAX_STOICH + o];
                if (k >= 0) dg += w->g_RT[k];
            }
            for (int o = 0; o < ORACLE_MAX_STOICH; ++o) {
                int k = m->reac[i * ORACLE_MAX_STOICH + o];
                if (k >= 0) dg -= w->g_RT[k];
            }
            w->rkc[i] = dmin(oracle_exp(fma(m->dn[i], lnRTp, dg)), BIG_NUMBER);
        }
    }
    w->kT = T;
    w->kModel = use_tables;
}

/* Composition part of the state setter; returns rho and fills c, ym. */
static void set_composition(const oracle_mech* m, oracle_ws* w, double p, double T, const double* Y, int mode,
                            double* rho_out, double* mmw_out) {
    const int S = m->S;
    if (mode == ORACLE_STATE_NORMALIZED) {
        for (int k = 0; k < S; ++k) w->tmp[k] = dmax(Y[k], 0.0);
        const double rnorm = 1.0 / block_sum(w->tmp, NULL, S, reduction_width(S));
        for (int k = 0; k < S; ++k) w->ym[k] = (w->tmp[k] * rnorm) * m->rW[k];
    } else {
        for (int k = 0; k < S; ++k) w->ym[k] = Y[k] * m->rW[k];
    }
    const double mmw = 1.0 / block_sum(w->ym, NULL, S, reduction_width(S));
    const double rho = (p * mmw) / (GAS_CONSTANT * T);
    for (int k = 0; k < S; ++k) w->c[k] = w->ym[k] * rho;
    *rho_out = rho;
    *mmw_out = mmw;
}

/* Rates of progress and production rates at (T, Y); thermo at T is left in w. */
void oracle_rates(const oracle_mech* m, oracle_ws* w, double p, int model, int mode, double T, const double* Y,
                  double* rho_out, double* cp_out) {
    const int S = m->S, R = m->R;
    if (!(w->kT == T) || w->kModel != model) oracle_rate_constants(m, w, T, model);
    double rho, mmw;
    set_composition(m, w, p, T, Y, mode, &rho, &mmw);
    const double ctot = rho / mmw;
    w->ctot = ctot;
    w->mmw = mmw;
    const double lnT = oracle_log(T), rT = 1.0 / T;
    for (int i = 0; i < R; ++i) {
        const int ty = m->type[i];
        double kf = w->kf[i];
        double concm = 0.0;
        if (ty != ORACLE_RXN_ELEMENTARY) {
            const double de = m->def_eff[i];
            concm = de * ctot;
            for (int64_t e = m->eff_off[i]; e < m->eff_off[i + 1]; ++e)
                concm = fma(m->eff_val[e] - de, w->c[m->eff_sp[e]], concm);
        }
        if (ty == ORACLE_RXN_LINDEMANN || ty == ORACLE_RXN_TROE) {
            const double kinf = arrhenius(m->arr + 3 * i, lnT, rT);
            const double k0 = arrhenius(m->arr_low + 3 * i, lnT, rT);
            const double pr = (concm * k0) * (1.0 / (kinf + SMALL_NUMBER));
            double F = 1.0, dF = 0.0; /* dF: dF/dPr */
            if (ty == ORACLE_RXN_TROE) {
                const double* tp = m->troe + 4 * i;
                /* Fcent with the reciprocals 1/T3, 1/T1, as Cantera's Troe rate keeps them */
                double fc = fma(1.0 - tp[0], oracle_exp(-T * (1.0 / tp[1])), tp[0] * oracle_exp(-T * (1.0 / tp[2])));
                if (tp[3] != 0.0) fc += oracle_exp(-tp[3] * rT);
                const double lfc = oracle_log10(dmax(fc, SMALL_NUMBER));
                const double lpr = oracle_log10(dmax(pr, SMALL_NUMBER));
                const double cc = fma(-0.67, lfc, -0.4);   /* -0.4 - 0.67 log Fcent */
                const double nn = fma(-1.27, lfc, 0.75);   /* 0.75 - 1.27 log Fcent */
                const double x = lpr + cc;
                const double f1 = x / fma(-0.14, x, nn);
                const double g = fma(f1, f1, 1.0);
                F = oracle_exp10(lfc / g);
                if (pr > SMALL_NUMBER) {
                    /* d log10 F / d f1 = -2 lfc f1 / g^2; d f1 / dx = nn / (nn - 0.14 x)^2; dx / dPr = 1/(Pr ln 10) */
                    const double den = fma(-0.14, x, nn);
                    dF = ((F * ((-2.0 * lfc * f1) / (g * g))) * (nn / (den * den))) / pr;
                }
            }
            kf = (pr * (F / (1.0 + pr))) * kinf;
            w->kf_fall[i] = kf;
            w->k0_fall[i] = k0;
            w->F_fall[i] = F;
            w->dF_fall[i] = dF;
            w->pr_fall[i] = pr;
        }
        w->concm[i] = concm;
        double rf = kf * m->mult[i];
        if (ty == ORACLE_RXN_THREE_BODY) rf *= concm;
        double ropf = rf, ropr = 0.0;
        for (int o = 0; o < ORACLE_MAX_STOICH; ++o) {
            int k = m->reac[i * ORACLE_MAX_STOICH + o];
            if (k >= 0) ropf *= w->c[k];
        }
        if (m->rev[i]) {
            ropr = rf * w->rkc[i];
            for (int o = 0; o < ORACLE_MAX_STOICH; ++o) {
                int k = m->prod[i * ORACLE_MAX_STOICH + o];
                if (k >= 0) ropr *= w->c[k];
            }
        }
        w->ropf[i] = ropf;
        w->ropr[i] = ropr;
    }
    for (int k = 0; k < S; ++k) w->wq[k] = w->wd[k] = w->wn[k] = 0.0;
    for (int i = 0; i < R; ++i) {
        const double f = w->ropf[i], r = w->ropr[i], net = f - r;
        const int* pr = m->prod + i * ORACLE_MAX_STOICH;
        const int* rc = m->reac + i * ORACLE_MAX_STOICH;
        for (int o = 0; o < ORACLE_MAX_STOICH; ++o)
            if (pr[o] >= 0) { w->wq[pr[o]] += f; w->wn[pr[o]] += net; }
        for (int o = 0; o < ORACLE_MAX_STOICH; ++o)
            if (rc[o] >= 0) { w->wq[rc[o]] += r; w->wd[rc[o]] += f; w->wn[rc[o]] -= net; }
        for (int o = 0; o < ORACLE_MAX_STOICH; ++o)
            if (pr[o] >= 0) w->wd[pr[o]] += r;
    }
    /* updateThermo: h_k [J/kmol], rho, cp_mass */
    const double RT = GAS_CONSTANT * T;
    for (int k = 0; k < S; ++k) {
        w->hk[k] = w->h_RT[k] * RT;
        w->tmp[k] = w->ym[k] * mmw;
    }
    *cp_out = (GAS_CONSTANT * block_sum(w->tmp, w->cp_R, S, reduction_width(S))) / mmw;
    *rho_out = rho;
}

void oracle_gas_eval(const oracle_mech* m, double p, int model, int mode, int n, const double* T, const double* Y,
                     double* creation, double* destruction, double* net, double* hk, double* cp_mass,
                     double* density) {
    oracle_ws* w = oracle_ws_create(m);
    const int S = m->S;
    for (int j = 0; j < n; ++j) {
        double rho, cp;
        oracle_rates(m, w, p, model, mode, T[j], Y + (size_t)j * S, &rho, &cp);
        if (creation) memcpy(creation + (size_t)j * S, w->wq, sizeof(double) * S);
        if (destruction) memcpy(destruction + (size_t)j * S, w->wd, sizeof(double) * S);
        if (net) memcpy(net + (size_t)j * S, w->wn, sizeof(double) * S);
        if (hk) memcpy(hk + (size_t)j * S, w->hk, sizeof(double) * S);
        if (cp_mass) cp_mass[j] = cp;
        if (density) density[j] = rho;
    }
    oracle_ws_free(w);
}

/* ---- SourceSystem pieces ---------------------------------------------- */

static double qdot_igniter(const oracle_source_options* o, double t, double x) {
    if (o->ignition_energy != 0.0 && t >= o->ignition_tstart && t < o->ignition_tstart + o->ignition_duration) {
        const double pi = 3.14159265358979323846;
        const double dx = x - o->ignition_center;
        return o->ignition_energy / (o->ignition_stddev * sqrt(2 * pi) * o->ignition_duration) *
               oracle_exp(-(dx * dx) / (2 * (o->ignition_stddev * o->ignition_stddev)));
    }
    return 0.0;
}

typedef struct {
    const oracle_mech* m;
    const oracle_source_options* o;
    oracle_ws* w;
    const double* split;
    double x;
    double T;               /* temperature frozen during corrector calls */
    double rrho, rrc;       /* 1/rho and 1/(rho cp) of the last predictor call */
} qss_ode;

/* SourceSystemQSS::odefun (src/sourceSystem.cpp:445-499) */
static void qss_odefun(qss_ode* ode, double t, const double* y, double* q, double* d, int corrector) {
    const oracle_mech* m = ode->m;
    oracle_ws* w = ode->w;
    const int S = m->S;
    if (!corrector) ode->T = y[1];
    double rho, cp;
    oracle_rates(m, w, ode->o->pressure, ode->o->kinetics_model, ORACLE_STATE_NORMALIZED, ode->T, y + 2, &rho, &cp);
    if (!corrector) {
        /* updateThermo on predictor calls only; h_k depends on T alone, which
         * the corrector calls keep, so w->hk is the predictor's */
        ode->rrho = 1.0 / rho;
        ode->rrc = 1.0 / (rho * cp);
    }
    for (int k = 0; k < S; ++k) w->tmp[k] = w->wq[k] - w->wd[k];
    const double qdot = -block_sum(w->tmp, w->hk, S, reduction_width(S)) + qdot_igniter(ode->o, t, ode->x);
    const double* sc = ode->split;
    q[0] = sc ? sc[0] : 0.0;
    d[0] = 0.0;
    q[1] = fma(qdot, ode->rrc, sc ? sc[1] : 0.0);
    d[1] = 0.0 * ode->rrc;
    for (int k = 0; k < S; ++k) {
        q[2 + k] = fma(w->wq[k] * m->W[k], ode->rrho, sc ? sc[2 + k] : 0.0);
        d[2 + k] = (w->wd[k] * m->W[k]) * ode->rrho;
    }
}

/* Pade numerator / denominator of the QSS predictor and corrector, Horner
 * form with fma (the same on the GPU). */
static double pade_num(double r) { return r * fma(r, fma(r, 11.0 + r, 60.0), 180.0); }
static double pade_den(double r) { return fma(r, fma(r, 12.0 + r, 60.0), 360.0); }
static double pade_an(double r) { return fma(r, fma(r, 11.0 + r, 60.0), 180.0); }

static double rsign(double x) { return (x > 0) ? 1.0 : (x < 0) ? -1.0 : 0.0; }

/* QssIntegrator working state; arrays of n entries. */
typedef struct {
    int n;
    double *y, *q, *d, *rtau, *rtaus, *y1, *ys, *qs, *ym1, *ym2, *scratch;
    const double* ymin;
    const int* enforce;
    double tn, ts, dt, tstart, tfd;
    int first_step, gcount, rcount;
} qss_state;

/* QssIntegrator::getInitialStepSize (src/qssintegrator.cpp:79-96) */
static void qss_initial_step(qss_state* s, const oracle_qss_params* o, double tf) {
    s->first_step = 0;
    double scrtch = 1.0e-25;
    for (int i = 0; i < s->n; ++i) {
        if (fabs(s->y[i]) > o->abstol) {
            double absq = fabs(s->q[i]);
            double scr2 = fabs(1 / s->y[i]) * rsign(0.1 * o->epsmin * absq - s->d[i]);
            double scr1 = scr2 * s->d[i];
            scrtch = dmax(dmax(scr1, -fabs(absq - s->d[i]) * scr2), scrtch);
        }
    }
    double sqreps = 0.5;
    s->dt = dmin(sqreps / scrtch, tf);
    s->dt = dmin(s->dt, o->dtmax);
}

/* QssIntegrator::integrateOneStep (src/qssintegrator.cpp:110-265) */
static int qss_one_step(qss_state* s, oracle_qss_fn f, void* ctx, const oracle_qss_params* o, double tf) {
    const int n = s->n;
    const int* en = s->enforce;
    f(ctx, s->tn + s->tstart, s->y, s->q, s->d, 0);
    s->gcount += 1;
    if (s->first_step) qss_initial_step(s, o, tf);
    s->ts = s->tn;
    for (int i = 0; i < n; ++i) s->rtau[i] = en[i] ? s->dt * s->d[i] / s->y[i] : 0.0;
    memcpy(s->qs, s->q, sizeof(double) * n);
    memcpy(s->ys, s->y, sizeof(double) * n);
    memcpy(s->rtaus, s->rtau, sizeof(double) * n);
    const int stab_on = o->stability_check;
    while (1) {
        /* The reference's predictor (q-d)/(1 + num/den) and corrector
         * (qs(1-a) + q a - ys rb/dt)/(1 + a rb), a = an/ad, each multiplied
         * through by den (ad) so that one division remains. */
        const double rdt = 1.0 / s->dt;
        for (int i = 0; i < n; ++i) {
            const double r = s->rtau[i];
            const double den = pade_den(r);
            s->scratch[i] = ((s->q[i] - s->d[i]) * den) / (den + pade_num(r));
        }
        double eps = 1e-10;
        for (int iter = 0; iter < o->itermax; ++iter) {
            if (stab_on) {
                memcpy(s->ym2, s->ym1, sizeof(double) * n);
                memcpy(s->ym1, s->y, sizeof(double) * n);
            }
            for (int i = 0; i < n; ++i) s->y[i] = dmax(s->ymin[i], fma(s->dt, s->scratch[i], s->ys[i]));
            if (iter == 0) {
                s->tn = s->ts + s->dt;
                memcpy(s->y1, s->y, sizeof(double) * n);
            }
            f(ctx, s->tn + s->tstart, s->y, s->q, s->d, 1);
            s->gcount += 1;
            eps = 1.0e-10;
            for (int i = 0; i < n; ++i) {
                const double rb = en[i] ? 0.5 * (s->rtaus[i] + s->dt * s->d[i] / s->y[i]) : 0.0;
                const double an = pade_an(rb), ad = pade_den(rb);
                const double num = fma(s->qs[i], ad - an, s->q[i] * an) - ((s->ys[i] * rb) * ad) * rdt;
                s->scratch[i] = num / fma(an, rb, ad);
            }
        }
        for (int i = 0; i < n; ++i) {
            double scr2 = fma(s->dt, s->scratch[i], s->ys[i]);
            if (en[i]) scr2 = dmax(scr2, s->ymin[i]);
            double scr1 = fabs(scr2 - s->y1[i]);
            s->y[i] = dmax(scr2, s->ymin[i]);
            if (fabs(s->y[i]) > o->abstol && 0.25 * (s->ys[i] + s->y[i]) > s->ymin[i]) {
                scr1 = scr1 / s->y[i];
                eps = dmax(.5 * (scr1 + dmin(fabs(s->q[i] - s->d[i]) / (s->q[i] + s->d[i] + 1e-30), scr1)), eps);
            }
        }
        if (stab_on) {
            memcpy(s->ym2, s->ym1, sizeof(double) * n);
            memcpy(s->ym1, s->y, sizeof(double) * n);
        }
        eps /= o->epsmin;
        if (s->dt <= o->dtmin + 1e-16 * s->tn) return -1;
        double stab = 0;
        if (stab_on && o->itermax >= 3) {
            stab = 0.01;
            for (int i = 0; i < n; ++i)
                if (fabs(s->y[i]) > o->abstol)
                    stab = dmax(stab, fabs(s->y[i] - s->ym1[i]) / (fabs(s->ym1[i] - s->ym2[i]) + 1e-20 * s->y[i]));
        }
        if (eps <= o->epsmax && stab <= 1.0) {
            if (tf <= s->tn * s->tfd) return 0;
        } else {
            s->tn = s->ts;
        }
        double rteps = 0.5 * (eps + 1.0);
        rteps = 0.5 * (rteps + eps / rteps);
        rteps = 0.5 * (rteps + eps / rteps);
        const double dto = s->dt;
        s->dt = dmin(s->dt * (1.0 / rteps + 0.005), s->tfd * (tf - s->tn));
        s->dt = dmin(s->dt, o->dtmax);
        if (stab_on) s->dt = dmin(s->dt, dto / (stab + .001));
        if (eps > o->epsmax || stab > 1) {
            s->rcount += 1;
            const double ratio = s->dt / dto;
            for (int i = 0; i < n; ++i) s->rtaus[i] *= ratio;
        } else {
            return 0;
        }
    }
}

/* QssIntegrator::setState + integrateToTime (src/qssintegrator.cpp:58-108)
 * for any q/d right-hand side. work: 11*n doubles. stats: steps, calls,
 * repeats (may be NULL). Returns 0, -1 (dtmin) or -20 (max_steps). */
int oracle_qss_integrate(int n, oracle_qss_fn f, void* ctx, const oracle_qss_params* o, double* y,
                         const double* ymin, const int* enforce, double tf, double tstart, int max_steps,
                         double* work, int* stats) {
    qss_state s;
    s.n = n;
    s.y = work; s.q = work + n; s.d = work + 2 * n; s.rtau = work + 3 * n; s.rtaus = work + 4 * n;
    s.y1 = work + 5 * n; s.ys = work + 6 * n; s.qs = work + 7 * n; s.ym1 = work + 8 * n; s.ym2 = work + 9 * n;
    s.scratch = work + 10 * n;
    s.ymin = ymin;
    s.enforce = enforce;
    for (int i = 0; i < n; ++i) {
        s.q[i] = s.d[i] = 0.0;
        s.ym1[i] = s.ym2[i] = 0.0;
        s.y[i] = enforce[i] ? dmax(y[i], ymin[i]) : y[i];
    }
    s.tn = 0.0; s.ts = 0.0; s.dt = 0.0; s.tstart = tstart; s.tfd = 1.000008;
    s.first_step = 1; s.gcount = 0; s.rcount = 0;
    int ret = 0, steps = 0;
    while (s.tfd * s.tn < tf) {
        if (steps >= max_steps) { ret = -20; break; }
        ret = qss_one_step(&s, f, ctx, o, tf);
        steps++;
        if (ret) break;
    }
    memcpy(y, s.y, sizeof(double) * n);
    if (stats) {
        stats[0] = steps;
        stats[1] = s.gcount;
        stats[2] = s.rcount;
        stats[3] = 0;
    }
    return ret;
}

static void qss_odefun_cb(void* ctx, double t, const double* y, double* q, double* d, int corrector) {
    qss_odefun((qss_ode*)ctx, t, y, q, d, corrector);
}

/* One point: SourceSystemQSS::setOptions/setState + integrateToTime(tf).
 * y is [U, T, Y...] in/out. */
int oracle_qss_point(const oracle_mech* m, oracle_ws* w, const oracle_source_options* o, double* y,
                     const double* split, double tf, double t_start, double x, int* stats) {
    const int n = m->S + 2;
    double* ymin = w->v + n;
    double* work = w->v + 2 * n;
    int* enforce = (int*)malloc(sizeof(int) * n);
    for (int i = 0; i < n; ++i) {
        enforce[i] = (i != 0);               /* enforce_ymin[kMomentum] = false */
        ymin[i] = (i == 0) ? -1e4 : o->qss_minval;
    }
    oracle_qss_params P = {o->qss_epsmin, o->qss_epsmax, o->qss_dtmin, o->qss_dtmax, o->qss_abstol,
                           o->qss_iteration_count, o->qss_stability_check};
    qss_ode ode = {m, o, w, split, x, y[1], 1.0, 1.0};
    int ret = oracle_qss_integrate(n, qss_odefun_cb, &ode, &P, y, ymin, enforce, tf, t_start, o->max_steps, work,
                                   stats);
    free(enforce);
    return ret;
}

/* ---- batch driver (threads over points, dynamic assignment) ------------ */

typedef struct {
    const oracle_mech* m;
    const oracle_source_options* o;
    int method, n;
    const double *state_in, *split, *dt, *x;
    double t_start;
    double* state_out;
    int *status, *stats;
    int next;
    pthread_mutex_t lock;
} batch_job;

static void* batch_worker(void* arg) {
    batch_job* J = (batch_job*)arg;
    const int nv = J->m->S + 2;
    oracle_ws* w = oracle_ws_create(J->m);
    for (;;) {
        pthread_mutex_lock(&J->lock);
        int j = J->next++;
        pthread_mutex_unlock(&J->lock);
        if (j >= J->n) break;
        double* y = J->state_out + (size_t)j * nv;
        memcpy(y, J->state_in + (size_t)j * nv, sizeof(double) * nv);
        const double* sc = J->split ? J->split + (size_t)j * nv : NULL;
        int* st = J->stats ? J->stats + (size_t)j * 4 : NULL;
        int r;
        if (J->method == 0)
            r = oracle_qss_point(J->m, w, J->o, y, sc, J->dt[j], J->t_start, J->x ? J->x[j] : 0.0, st);
        else
            r = oracle_bdf_point(J->m, w, J->o, y, sc, J->dt[j], J->t_start, J->x ? J->x[j] : 0.0, st);
        if (r == 0)
            for (int i = 0; i < nv; ++i)
                if (!isfinite(y[i])) { r = -21; break; }
        J->status[j] = r;
    }
    oracle_ws_free(w);
    return NULL;
}

void oracle_source_batch(const oracle_mech* m, int method, int n, const double* state_in, const double* split,
                         const double* dt, double t_start, const double* x, const oracle_source_options* o,
                         double* state_out, int* status, int* stats, int n_threads) {
    batch_job J = {m, o, method, n, state_in, split, dt, x, t_start, state_out, status, stats, 0};
    pthread_mutex_init(&J.lock, NULL);
    if (n_threads < 1) n_threads = 1;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * n_threads);
    for (int t = 0; t < n_threads; ++t) pthread_create(&th[t], NULL, batch_worker, &J);
    for (int t = 0; t < n_threads; ++t) pthread_join(th[t], NULL);
    free(th);
    pthread_mutex_destroy(&J.lock);
}
