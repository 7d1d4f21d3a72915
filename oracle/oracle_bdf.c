/*
 * CPU ORACLE -- test infrastructure only (see oracle_tridiag.c).
 * Variable-order BDF for the CVODE source-term path (placeholder until the
 * restatement of CVODE's published method is added).
 */
#include "oracle.h"

int oracle_bdf_point(const oracle_mech* m, oracle_ws* w, const oracle_source_options* o, double* y,
                     const double* split, double tf, double t_start, double x, int* stats) {
    (void)m; (void)w; (void)o; (void)y; (void)split; (void)tf; (void)t_start; (void)x; (void)stats;
    return -99;
}
