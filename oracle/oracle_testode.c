/*
 * CPU ORACLE -- test infrastructure only (see oracle_tridiag.c).
 *
 * The stiff test problem of the reference's legacy QSS test
 * (test/old/test_qssintegrator.cpp:11-83): atmospheric cesium / cesium-ion
 * relaxation (Edelson), seven components of which five are integrated; the
 * electron density is derived from charge balance. Used to pin the QSS
 * integrator restatement (and, through the same q/d right-hand side on the
 * device, the GPU integrator).
 */
#include <stdlib.h>

#include "oracle.h"

static void cesium_rhs(void* ctx, double t, const double* y, double* q, double* d, int corrector) {
    (void)ctx; (void)t; (void)corrector;
    const double o2m = y[0], csp = y[1], cs = y[2], cso2 = y[3], o2 = y[4], n2 = y[5];
    const double ne = (csp - o2m > 0.0) ? csp - o2m : 0.0;
    const double cr1 = 5.00e-08 * o2m * csp;
    const double cr2 = 1.00e-12 * csp * ne;
    const double cr3 = 3.24e-03 * cs;
    const double cr4 = 4.00e-01 * o2m;
    const double cr5 = 1.00e-31 * o2 * cs * (cs + cso2 + n2 + o2);
    const double cr6 = 1.24e-30 * o2 * o2 * ne;
    const double cr7 = 1.00e-31 * o2 * n2 * ne;
    for (int i = 0; i < 7; ++i) q[i] = d[i] = 0.0;
    q[0] = cr6 + cr7;
    d[0] = cr1 + cr4;
    q[1] = cr3;
    d[1] = cr1 + cr2;
    q[2] = cr1 + cr2;
    d[2] = cr3 + cr5;
    q[3] = cr5;
    q[4] = cr1 + cr4;
    d[4] = cr5 + cr6 + cr7;
}

int oracle_qss_cesium(const oracle_qss_params* o, double* y7, double tf, int max_steps, int* stats) {
    double ymin[7];
    int enforce[7];
    double work[11 * 7];
    for (int i = 0; i < 7; ++i) {
        ymin[i] = 1e-20;
        enforce[i] = 1;
    }
    int r = oracle_qss_integrate(7, cesium_rhs, NULL, o, y7, ymin, enforce, tf, 0.0, max_steps, work, stats);
    y7[6] = y7[1] - y7[0];  /* electron density from charge balance */
    return r;
}
