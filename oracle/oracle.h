/*
 * CPU ORACLE -- test infrastructure only (see oracle_tridiag.c header).
 * Plain-C restatement of the reference's hot-path algorithms, exported with
 * a C ABI for the tests (ctypes) and for bench.py's CPU baseline leg.
 */
#ifndef EMBER_ORACLE_H
#define EMBER_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int N;
    double* buf;
    double *a, *b, *c, *k, *y, *yprev, *luc, *inv, *lud;
    double t, h, lu_b0;
    int step_count;
} oracle_tridiag;

void oracle_tridiag_init(oracle_tridiag* s, int N, const double* a, const double* b, const double* c,
                         const double* k, const double* y0);
void oracle_tridiag_free(oracle_tridiag* s);
void oracle_tridiag_initialize(oracle_tridiag* s, double t0, double h);
void oracle_tridiag_step(oracle_tridiag* s);
void oracle_tridiag_integrate_to_time(oracle_tridiag* s, double t_end);
void oracle_tridiag_ydot(const oracle_tridiag* s, double* ydot);
void oracle_tridiag_run(int N, const double* a, const double* b, const double* c, const double* k, double* y,
                        double t0, double h, double t_end, int n_single_steps, double* t_out, double* h_out);

void oracle_diffusion_matrix(int N, const double* x, int alpha, int left_bc, int right_bc, const double* B,
                             const double* D, const double* split_const, double wall_const, double y_inf,
                             double* a, double* b, double* c, double* k);
double oracle_diffusion_step_size(int N, const double* x, const double* B, const double* D, double mult,
                                  double gdt);
void oracle_diffusion_system(int N, const double* x, int alpha, int left_bc, int right_bc, const double* B,
                             const double* D, const double* split_const, double wall_const, double y_inf,
                             double h, double mult, double gdt, double t0, double t1, double* y);

#ifdef __cplusplus
}
#endif

#endif
