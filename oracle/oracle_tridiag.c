/*
 * CPU ORACLE -- test infrastructure only. Never linked into, or called by,
 * the product library; only tests/, the smoke check and bench.py's CPU
 * baseline load it, to compare the GPU results with.
 *
 * Plain-C restatement of the reference's tridiagonal integrator and
 * diffusion matrix:
 *   TridiagonalIntegrator::step           src/integrator.cpp:133-204
 *   Integrator::integrateToTime           src/integrator.cpp:37-47
 *   TridiagonalIntegrator::get_ydot       src/integrator.cpp:124-131
 *   DiffusionSystem::get_A / get_k        src/diffusionSystem.cpp:10-76
 *   OneDimGrid::updateValues (metrics)    src/grid.cpp:43-69
 *   FlameSolver::setDiffusionSolverState  src/flameSolver.cpp:702-718
 *   FlameSolver::integrateDiffusionTerms  src/flameSolver.cpp:838-854
 * Operation order follows the reference statement by statement. Built with
 * -ffp-contract=off so that no multiply-add is fused (the reference's x86-64
 * build has no FMA), which makes results reproducible across hosts.
 *
 * Parity pin: the integrator reproduces the reference's golden table
 * (test/tridiagonalIntegrator.cpp:4-10, generated by test/reference/bdf.py)
 * and the analytic/property tests of test/test_diffusionSystem.cpp.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

/* ---- TridiagonalIntegrator ------------------------------------------- */

static void factor(int N, const double* a, const double* b, const double* c, double shift, double* luc,
                   double* inv, double* lu_b0) {
    double lb0 = b[0] - shift;
    luc[0] = c[0] / lb0;
    for (int i = 1; i < N; ++i) {
        inv[i] = 1.0 / ((b[i] - shift) - luc[i - 1] * a[i]);
        luc[i] = c[i] * inv[i];
    }
    *lu_b0 = lb0;
}

static void solve(int N, const double* a, const double* luc, const double* inv, double lu_b0, double* y,
                  double* lud) {
    lud[0] = y[0] / lu_b0;
    for (int i = 1; i < N; ++i) lud[i] = (y[i] - lud[i - 1] * a[i]) * inv[i];
    y[N - 1] = lud[N - 1];
    for (int i = N - 2; i >= 0; --i) y[i] = lud[i] - luc[i] * y[i + 1];
}

void oracle_tridiag_init(oracle_tridiag* s, int N, const double* a, const double* b, const double* c,
                         const double* k, const double* y0) {
    s->N = N;
    s->buf = (double*)calloc((size_t)N * 9, sizeof(double));
    s->a = s->buf;
    s->b = s->a + N;
    s->c = s->b + N;
    s->k = s->c + N;
    s->y = s->k + N;
    s->yprev = s->y + N;
    s->luc = s->yprev + N;
    s->inv = s->luc + N;
    s->lud = s->inv + N;
    memcpy(s->a, a, sizeof(double) * N);
    memcpy(s->b, b, sizeof(double) * N);
    memcpy(s->c, c, sizeof(double) * N);
    memcpy(s->k, k, sizeof(double) * N);
    memcpy(s->y, y0, sizeof(double) * N);
    s->t = 0.0;
    s->h = 0.0;
    s->lu_b0 = 0.0;
    s->step_count = 0;
}

void oracle_tridiag_free(oracle_tridiag* s) {
    free(s->buf);
    s->buf = NULL;
}

void oracle_tridiag_initialize(oracle_tridiag* s, double t0, double h) {
    s->t = t0;
    s->h = h;
    s->step_count = 0;
}

void oracle_tridiag_step(oracle_tridiag* s) {
    const int N = s->N;
    if (s->step_count == 0) {
        memcpy(s->yprev, s->y, sizeof(double) * N);
        factor(N, s->a, s->b, s->c, 1.0 / (s->h / 8.0), s->luc, s->inv, &s->lu_b0);
        for (int j = 0; j < 8; ++j) {
            for (int i = 0; i < N; ++i) s->y[i] = -s->y[i] / (s->h / 8.0) - s->k[i];
            solve(N, s->a, s->luc, s->inv, s->lu_b0, s->y, s->lud);
        }
    } else {
        if (s->step_count == 1) factor(N, s->a, s->b, s->c, 3.0 / (2.0 * s->h), s->luc, s->inv, &s->lu_b0);
        for (int i = 0; i < N; ++i) {
            double ynm1 = s->y[i];
            s->y[i] = -2 * ynm1 / s->h + s->yprev[i] / (2 * s->h) - s->k[i];
            s->yprev[i] = ynm1;
        }
        solve(N, s->a, s->luc, s->inv, s->lu_b0, s->y, s->lud);
    }
    s->step_count++;
    s->t += s->h;
}

void oracle_tridiag_integrate_to_time(oracle_tridiag* s, double t_end) {
    int n_steps = (int)((t_end - s->t) / s->h + 1e-5);
    if (n_steps < 1) n_steps = 1;
    s->h = (t_end - s->t) / n_steps;
    for (int i = 0; i < n_steps; ++i) oracle_tridiag_step(s);
}

void oracle_tridiag_ydot(const oracle_tridiag* s, double* ydot) {
    const int N = s->N;
    const double *a = s->a, *b = s->b, *c = s->c, *k = s->k, *y = s->y;
    ydot[0] = b[0] * y[0] + c[0] * y[1] + k[0];
    for (int i = 1; i < N - 1; ++i) ydot[i] = a[i] * y[i - 1] + b[i] * y[i] + c[i] * y[i + 1] + k[i];
    ydot[N - 1] = a[N - 1] * y[N - 2] + b[N - 1] * y[N - 1] + k[N - 1];
}

/* Whole-array convenience for ctypes: integrate one system from (t0, h) to t_end. */
void oracle_tridiag_run(int N, const double* a, const double* b, const double* c, const double* k,
                        double* y, double t0, double h, double t_end, int n_single_steps, double* t_out,
                        double* h_out) {
    oracle_tridiag s;
    oracle_tridiag_init(&s, N, a, b, c, k, y);
    oracle_tridiag_initialize(&s, t0, h);
    if (n_single_steps > 0) {
        for (int i = 0; i < n_single_steps; ++i) oracle_tridiag_step(&s);
    } else {
        oracle_tridiag_integrate_to_time(&s, t_end);
    }
    memcpy(y, s.y, sizeof(double) * N);
    if (t_out) *t_out = s.t;
    if (h_out) *h_out = s.h;
    oracle_tridiag_free(&s);
}

/* ---- grid metrics and DiffusionSystem -------------------------------- */

static double gpow(double v, int alpha) { return pow(v, (double)alpha); }

/* Rows a, b, c and constant k of one diffusion system (N points). */
void oracle_diffusion_matrix(int N, const double* x, int alpha, int left_bc, int right_bc, const double* B,
                             const double* D, const double* split_const, double wall_const, double y_inf,
                             double* a, double* b, double* c, double* k) {
    double* hh = (double*)calloc((size_t)N, sizeof(double));
    double* rphalf = (double*)calloc((size_t)N, sizeof(double));
    double* r = (double*)calloc((size_t)N, sizeof(double));
    double* dlj = (double*)calloc((size_t)N, sizeof(double));
    double* c1 = (double*)calloc((size_t)N, sizeof(double));
    double* c2 = (double*)calloc((size_t)N, sizeof(double));
    for (int j = 0; j < N - 1; ++j) {
        hh[j] = x[j + 1] - x[j];
        rphalf[j] = gpow(0.5 * (x[j] + x[j + 1]), alpha);
    }
    for (int j = 0; j < N; ++j) r[j] = gpow(x[j], alpha);
    for (int j = 1; j < N - 1; ++j) dlj[j] = 0.5 * (x[j + 1] - x[j - 1]);

    memset(a, 0, sizeof(double) * N);
    memset(b, 0, sizeof(double) * N);
    memset(c, 0, sizeof(double) * N);

    for (int j = 1; j <= N - 2; ++j) {
        c1[j] = 0.5 * B[j] / (dlj[j] * r[j]);
        c2[j] = rphalf[j] * (D[j] + D[j + 1]) / hh[j];
    }
    int jStart;
    if (left_bc == 0) { /* FixedValue */
        jStart = 1;
    } else if (left_bc == 2) { /* ControlVolume */
        jStart = 1;
        double c0 = B[0] * (alpha + 1) * (D[0] + D[1]) / (2 * hh[0] * hh[0]);
        b[0] = -c0;
        c[0] = c0;
    } else if (left_bc == 3) { /* WallFlux */
        jStart = 1;
        double c0 = B[0] * (alpha + 1) / hh[0];
        double d = 0.5 * (D[0] + D[1]);
        b[0] = -c0 * (d / hh[0] + wall_const);
        c[0] = d * c0 / hh[0];
    } else { /* ZeroGradient */
        jStart = 2;
        b[1] = -c1[1] * c2[1];
        c[1] = c1[1] * c2[1];
    }
    int jStop;
    if (right_bc == 0) {
        jStop = N - 1;
    } else {
        jStop = N - 2;
        a[N - 2] = c1[N - 2] * c2[N - 3];
        b[N - 2] = -c1[N - 2] * c2[N - 3];
    }
    for (int j = jStart; j < jStop; ++j) {
        a[j] = c1[j] * c2[j - 1];
        b[j] = -c1[j] * (c2[j - 1] + c2[j]);
        c[j] = c1[j] * c2[j];
    }
    for (int j = 0; j < N; ++j) k[j] = split_const ? split_const[j] : 0.0;
    if (left_bc == 3) k[0] += B[0] * (alpha + 1) / hh[0] * wall_const * y_inf;
    free(hh);
    free(rphalf);
    free(r);
    free(dlj);
    free(c1);
    free(c2);
}

double oracle_diffusion_step_size(int N, const double* x, const double* B, const double* D, double mult,
                                  double gdt) {
    double m = 0.0;
    for (int j = 1; j <= N - 2; ++j) {
        double dlj = 0.5 * (x[j + 1] - x[j - 1]);
        double v = dlj * dlj / (B[j] * D[j]);
        if (j == 1 || v < m) m = v;
    }
    double h = mult * m;
    return gdt < h ? gdt : h;
}

/* One diffusion system through one stage: initialize(t0, h) then
 * integrateToTime(t1). h <= 0 selects the setDiffusionSolverState rule. */
void oracle_diffusion_system(int N, const double* x, int alpha, int left_bc, int right_bc, const double* B,
                             const double* D, const double* split_const, double wall_const, double y_inf,
                             double h, double mult, double gdt, double t0, double t1, double* y) {
    double* buf = (double*)malloc(sizeof(double) * 4 * (size_t)N);
    double *a = buf, *b = buf + N, *c = buf + 2 * N, *k = buf + 3 * N;
    oracle_diffusion_matrix(N, x, alpha, left_bc, right_bc, B, D, split_const, wall_const, y_inf, a, b, c, k);
    if (!(h > 0)) h = oracle_diffusion_step_size(N, x, B, D, mult, gdt);
    oracle_tridiag s;
    oracle_tridiag_init(&s, N, a, b, c, k, y);
    oracle_tridiag_initialize(&s, t0, h);
    oracle_tridiag_integrate_to_time(&s, t1);
    memcpy(y, s.y, sizeof(double) * N);
    oracle_tridiag_free(&s);
    free(buf);
}

/* ---- threaded batch (CPU baseline of the diffusion stage) -------------- */

#include <pthread.h>

typedef struct {
    int n_flames, n_vars;
    const int* npts;
    const int* left_bc;
    const int* right_bc;
    const int* alpha;
    const int64_t* pt_off;   /* grid offsets per flame */
    const int64_t* val_off;  /* value offsets per flame */
    const double *x, *B, *D, *S, *h;
    double mult, gdt, t0, t1;
    double* y;
    int next;
    pthread_mutex_t lock;
} diff_job;

static void* diff_worker(void* arg) {
    diff_job* J = (diff_job*)arg;
    const int total = J->n_flames * J->n_vars;
    for (;;) {
        pthread_mutex_lock(&J->lock);
        int s = J->next++;
        pthread_mutex_unlock(&J->lock);
        if (s >= total) break;
        const int f = s / J->n_vars, v = s % J->n_vars;
        const int N = J->npts[f];
        const int64_t o = J->val_off[f] + (int64_t)v * N;
        oracle_diffusion_system(N, J->x + J->pt_off[f], J->alpha[f], J->left_bc[f], J->right_bc[f], J->B + o,
                                J->D + o, J->S ? J->S + o : NULL, 0.0, 0.0, J->h ? J->h[s] : 0.0, J->mult, J->gdt,
                                J->t0, J->t1, J->y + o);
    }
    return NULL;
}

void oracle_diffusion_batch(int n_flames, int n_vars, const int* npts, const int* left_bc, const int* right_bc,
                            const int* alpha, const double* x, const double* B, const double* D, const double* S,
                            const double* h, double mult, double gdt, double t0, double t1, double* y,
                            int n_threads) {
    int64_t* pt_off = (int64_t*)malloc(sizeof(int64_t) * (n_flames + 1));
    int64_t* val_off = (int64_t*)malloc(sizeof(int64_t) * (n_flames + 1));
    pt_off[0] = val_off[0] = 0;
    for (int f = 0; f < n_flames; ++f) {
        pt_off[f + 1] = pt_off[f] + npts[f];
        val_off[f + 1] = val_off[f] + (int64_t)npts[f] * n_vars;
    }
    diff_job J = {n_flames, n_vars, npts, left_bc, right_bc, alpha, pt_off, val_off, x, B, D, S, h,
                  mult, gdt, t0, t1, y, 0};
    pthread_mutex_init(&J.lock, NULL);
    if (n_threads < 1) n_threads = 1;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * n_threads);
    for (int t = 0; t < n_threads; ++t) pthread_create(&th[t], NULL, diff_worker, &J);
    for (int t = 0; t < n_threads; ++t) pthread_join(th[t], NULL);
    pthread_mutex_destroy(&J.lock);
    free(th);
    free(pt_off);
    free(val_off);
}
