/*
 * CPU ORACLE -- test infrastructure only (see oracle_tridiag.c header).
 *
 * Thermo and mixture-averaged transport properties of flame states, as
 * FlameSolver::updateChemicalProperties (src/flameSolver.cpp:652-699) gets
 * them from Cantera with the "Approx" transport model:
 *   - ApproxMixTransport::viscosity / updateViscosity_T
 *     (src/chemistry0d.cpp:22-52, 181-205): Wilke's rule over the species
 *     whose mole fraction is at least the threshold, the lower triangle of
 *     phi from the formula, the upper one from the identity
 *     phi_jk = phi_kj / ((mu_k / mu_j) (W_j / W_k));
 *   - ApproxMixTransport::getMixDiffCoeffsMass (src/chemistry0d.cpp:98-139)
 *     times the density (CanteraGas::getWeightedDiffusionCoefficientsMass,
 *     src/chemistry0d.cpp:583-591), binary coefficients p D_jk =
 *     T^(3/2) P(ln T) (updateDiff_T, src/chemistry0d.cpp:207-235);
 *   - the mixture conductivity of Cantera's MixTransport,
 *     (sum X lambda + 1 / sum X / lambda) / 2, species values
 *     lambda_k = T^(1/2) P(ln T) and sqrt(mu_k) = T^(1/4) P(ln T) (Cantera's
 *     non-CK fitting form), mole fractions floored at 1e-20 (Cantera's
 *     MixTransport::update_C).
 * Cantera is a third-party dependency (3.2.x) absent here: its part is
 * restated from its published mixture-averaged model and is PARITY UNPINNED
 * (no reference test holds transport values).
 *
 * Operation order equals the GPU kernel's (ember_gb300/csrc/transport.cu):
 * sums over species, and a major species' diffusion sums over its S - 1
 * partners, in the 32-lane order of oracle_block_sum (term m on lane m mod 32,
 * then the xor butterfly); the other per-species sums sequentially in species
 * order; no FMA contraction.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

#define GAS_CONSTANT (6.02214076e26 * 1.380649e-23)
#define MOLE_FRACTION_FLOOR 1e-20

double oracle_log(double x);
double oracle_block_sum(const double* a, const double* b, int n, int W);

static double dmax(double a, double b) { return (a < b) ? b : a; }

static long long pair_index(int S, int lo, int hi) {
    return (long long)lo * S - (long long)lo * (lo - 1) / 2 + (hi - lo);
}

static double fit5(const double* c, double x1, double x2, double x3, double x4) {
    double r = c[0];
    r = r + x1 * c[1];
    r = r + x2 * c[2];
    r = r + x3 * c[3];
    r = r + x4 * c[4];
    return r;
}

/* Sum over k of term[k] in the 32-lane order (term precomputed, plain adds). */
static double lane_sum(const double* term, int n) { return oracle_block_sum(term, NULL, n, 32); }

/* The xor butterfly that combines 32 lane partials (the GPU's warp shuffle). */
static double butterfly(double* q) {
    for (int off = 16; off >= 1; off >>= 1) {
        double r[32];
        for (int l = 0; l < 32; ++l) r[l] = q[l] + q[l ^ off];
        memcpy(q, r, sizeof r);
    }
    return q[0];
}

static double wilke_phi(int S, const double* w4, const double* s8w1, const double* sq, const double* mu,
                        const double* W, int r, int c) {
    if (r >= c) {
        const long long q = pair_index(S, c, r);
        const double f1 = 1.0 + (sq[r] / sq[c]) * w4[q];
        return (f1 * f1) / s8w1[q];
    }
    const long long q = pair_index(S, r, c);
    const double f1 = 1.0 + (sq[c] / sq[r]) * w4[q];
    const double phi_cr = (f1 * f1) / s8w1[q];
    return phi_cr / ((mu[c] / mu[r]) * (W[r] / W[c]));
}

void oracle_transport_eval(const oracle_mech* m, const double* visc_fit, const double* cond_fit,
                           const double* diff_fit, int n, double p, double thr, const double* Tin, const double* Yin,
                           double* density, double* mean_mw, double* cp_mass, double* cp_species, double* h_species,
                           double* conductivity, double* viscosity, double* rho_d) {
    const int S = m->S;
    const long long P = (long long)S * (S + 1) / 2;
    double* w4 = (double*)malloc(sizeof(double) * P);
    double* s8w1 = (double*)malloc(sizeof(double) * P);
    for (int lo = 0; lo < S; ++lo)
        for (int hi = lo; hi < S; ++hi) {
            const long long q = pair_index(S, lo, hi);
            w4[q] = sqrt(sqrt(m->W[lo] / m->W[hi]));
            s8w1[q] = sqrt(8.0) * sqrt(1.0 + m->W[hi] / m->W[lo]);
        }
    double* buf = (double*)malloc(sizeof(double) * 9 * S);
    int* majors = (int*)malloc(sizeof(int) * (S > 0 ? S : 1));
    double *ym = buf, *cpR = ym + S, *x = cpR + S, *sq = x + S, *mu = sq + S, *lam = mu + S, *sk = lam + S,
           *term = sk + S, *term2 = term + S;
    for (int j = 0; j < n; ++j) {
        const double T = Tin[j];
        const double* y = Yin + (size_t)j * S;
        const double lnT = oracle_log(T), rT = 1.0 / T;
        const double RT = GAS_CONSTANT * T;
        const double sqT = sqrt(T), t14 = sqrt(sqT), t15 = T * sqT;
        const double l2 = lnT * lnT, l3 = l2 * lnT, l4 = l3 * lnT;
        for (int k = 0; k < S; ++k) {
            const int r = (T <= m->tmid[k]) ? 0 : 1;
            const double* a = m->nasa + 14 * k + 7 * r;
            const double* h = m->hc + 10 * k + 5 * r;
            const double cp = fma(fma(fma(fma(a[4], T, a[3]), T, a[2]), T, a[1]), T, a[0]);
            const double hr = fma(fma(fma(fma(h[4], T, h[3]), T, h[2]), T, h[1]), T, h[0]) + a[5] * rT;
            cpR[k] = cp;
            if (cp_species) cp_species[(size_t)j * S + k] = cp * GAS_CONSTANT;
            if (h_species) h_species[(size_t)j * S + k] = hr * RT;
            const double s = t14 * fit5(visc_fit + 5 * k, lnT, l2, l3, l4);
            sq[k] = s;
            mu[k] = s * s;
            lam[k] = sqT * fit5(cond_fit + 5 * k, lnT, l2, l3, l4);
        }
        for (int k = 0; k < S; ++k) term[k] = dmax(y[k], 0.0);
        const double rnorm = 1.0 / lane_sum(term, S);
        for (int k = 0; k < S; ++k) ym[k] = (dmax(y[k], 0.0) * rnorm) * m->rW[k];
        const double mmw = 1.0 / lane_sum(ym, S);
        const double rho = (p * mmw) / (GAS_CONSTANT * T);
        for (int k = 0; k < S; ++k) term[k] = ym[k] * mmw;
        const double cpsum = oracle_block_sum(term, cpR, S, 32);
        for (int k = 0; k < S; ++k) x[k] = dmax(ym[k] * mmw, MOLE_FRACTION_FLOOR);
        for (int k = 0; k < S; ++k) {
            term[k] = x[k] * lam[k];
            term2[k] = x[k] / lam[k];
        }
        const double s1 = lane_sum(term, S);
        const double s2 = lane_sum(term2, S);
        /* the major species, in order: every partner list below is a
         * sequence whose term m goes to lane m mod 32 */
        int K = 0;
        for (int k = 0; k < S; ++k)
            if (x[k] >= thr) majors[K++] = k;
        for (int k = 0; k < S; ++k) {
            double s = 0.0;
            if (x[k] >= thr)
                for (int ci = 0; ci < K; ++ci) {
                    const int c = majors[ci];
                    s = s + x[c] * wilke_phi(S, w4, s8w1, sq, mu, m->W, k, c);
                }
            sk[k] = s;
        }
        /* terms of the major species; the others add exact zeros (q + 0 == q for q != -0) */
        for (int k = 0; k < S; ++k) term[k] = x[k] >= thr ? (x[k] * mu[k]) / sk[k] : 0.0;
        const double vis = lane_sum(term, S);
        if (rho_d) {
            for (int k = 0; k < S; ++k) {
                double d;
                if (S == 1) {
                    d = (t15 * fit5(diff_fit, lnT, l2, l3, l4)) / p;
                } else {
                    /* a major species: term m of its S - 1 partners on lane m mod 32,
                     * then the butterfly; a minor one: sequentially over the majors */
                    const int major = x[k] >= thr;
                    const int count = major ? S - 1 : K;
                    double q1[32] = {0.0}, q2[32] = {0.0};
                    for (int mi = 0; mi < count; ++mi) {
                        const int i = major ? (mi < k ? mi : mi + 1) : majors[mi];
                        const int lane = major ? mi % 32 : 0;
                        const long long q = i < k ? pair_index(S, i, k) : pair_index(S, k, i);
                        const double bd = t15 * fit5(diff_fit + 5 * q, lnT, l2, l3, l4);
                        q1[lane] = q1[lane] + x[i] / bd;
                        q2[lane] = q2[lane] + (x[i] * m->W[i]) / bd;
                    }
                    double a1 = major ? butterfly(q1) : q1[0], a2 = major ? butterfly(q2) : q2[0];
                    a1 = a1 * p;
                    a2 = a2 * ((p * x[k]) / (mmw - m->W[k] * x[k]));
                    d = 1.0 / (a1 + a2);
                }
                rho_d[(size_t)j * S + k] = d * rho;
            }
        }
        if (density) density[j] = rho;
        if (mean_mw) mean_mw[j] = mmw;
        if (cp_mass) cp_mass[j] = (GAS_CONSTANT * cpsum) / mmw;
        if (conductivity) conductivity[j] = 0.5 * (s1 + 1.0 / s2);
        if (viscosity) viscosity[j] = vis;
    }
    free(buf);
    free(majors);
    free(w4);
    free(s8w1);
}

/* ---- threaded batch (CPU baseline): contiguous ranges of points per thread */

#include <pthread.h>

typedef struct {
    const oracle_mech* m;
    const double *visc, *cond, *diff, *T, *Y;
    double p, thr;
    int j0, j1;
    double *density, *mean_mw, *cp_mass, *cp_species, *h_species, *conductivity, *viscosity, *rho_d;
} transport_job;

static void* transport_worker(void* arg) {
    const transport_job* J = (const transport_job*)arg;
    const int S = J->m->S, j0 = J->j0, n = J->j1 - J->j0;
#define OFF1(a) ((a) ? (a) + j0 : NULL)
#define OFFS(a) ((a) ? (a) + (size_t)j0 * S : NULL)
    oracle_transport_eval(J->m, J->visc, J->cond, J->diff, n, J->p, J->thr, J->T + j0, J->Y + (size_t)j0 * S,
                          OFF1(J->density), OFF1(J->mean_mw), OFF1(J->cp_mass), OFFS(J->cp_species),
                          OFFS(J->h_species), OFF1(J->conductivity), OFF1(J->viscosity), OFFS(J->rho_d));
#undef OFF1
#undef OFFS
    return NULL;
}

void oracle_transport_eval_threads(const oracle_mech* m, const double* visc_fit, const double* cond_fit,
                                   const double* diff_fit, int n, double p, double thr, const double* T,
                                   const double* Y, double* density, double* mean_mw, double* cp_mass,
                                   double* cp_species, double* h_species, double* conductivity, double* viscosity,
                                   double* rho_d, int n_threads) {
    if (n_threads < 1) n_threads = 1;
    if (n_threads > n) n_threads = n > 0 ? n : 1;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * n_threads);
    transport_job* jobs = (transport_job*)malloc(sizeof(transport_job) * n_threads);
    for (int t = 0; t < n_threads; ++t) {
        transport_job J = {m, visc_fit, cond_fit, diff_fit, T, Y, p, thr, (int)((long long)n * t / n_threads),
                           (int)((long long)n * (t + 1) / n_threads), density, mean_mw, cp_mass, cp_species,
                           h_species, conductivity, viscosity, rho_d};
        jobs[t] = J;
        pthread_create(&th[t], NULL, transport_worker, &jobs[t]);
    }
    for (int t = 0; t < n_threads; ++t) pthread_join(th[t], NULL);
    free(jobs);
    free(th);
}
