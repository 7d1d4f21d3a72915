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

/* ---- chemistry ---------------------------------------------------------- */

#define ORACLE_MAX_STOICH 4
#define ORACLE_RXN_ELEMENTARY 0
#define ORACLE_RXN_THREE_BODY 1
#define ORACLE_RXN_LINDEMANN 2
#define ORACLE_RXN_TROE 3
#define ORACLE_STATE_NORMALIZED 0
#define ORACLE_STATE_NO_NORM 1

/* Same field layout as the product's ember_mech_desc. */
typedef struct {
    int n_species, n_reactions;
    const double *mol_weight, *nasa_tmid, *nasa_coeffs;
    const int *rxn_type, *reversible, *reactants, *products;
    const double *arrhenius, *arrhenius_low, *troe, *default_efficiency;
    const int64_t* efficiency_offsets;
    const int* efficiency_species;
    const double* efficiency_values;
} oracle_mech_desc;

typedef struct {
    int S, R;
    double *W, *rW, *tmid, *nasa, *hc, *sc;
    int *type, *rev, *reac, *prod;
    double *arr, *arr_low, *troe, *def_eff;
    int64_t* eff_off;
    int* eff_sp;
    double *eff_val, *mult, *dn;
    int nT;
    double Tmin, Tmax;
    double *kf_c, *kf_s, *kc_c, *kc_s;
} oracle_mech;

typedef struct {
    double *cp_R, *h_RT, *g_RT, *c, *ym, *tmp, *kf, *rkc, *ropf, *ropr, *wq, *wd, *wn, *hk, *v;
    double *kf_fall, *k0_fall, *F_fall, *pr_fall, *concm, *jdense;  /* falloff terms, [M], Jacobian scratch */
    double* dF_fall;                                                /* dF/dPr of the falloff blending */
    double ctot, mmw;
    double kT;
    int kModel;
} oracle_ws;

/* Same field layout as the product's ember_source_options. */
typedef struct {
    double pressure;
    int kinetics_model;
    int max_steps;
    double qss_epsmin, qss_epsmax, qss_dtmin, qss_dtmax, qss_abstol, qss_minval;
    int qss_iteration_count, qss_stability_check;
    double bdf_reltol, bdf_abstol_momentum, bdf_abstol_energy, bdf_abstol_species, bdf_min_step;
    int bdf_max_num_steps;
    int threads_per_point; /* launch width of the GPU kernel; no effect here */
    double ignition_tstart, ignition_duration, ignition_energy, ignition_center, ignition_stddev;
    int qss_tail_steps, qss_tail_threads; /* GPU schedule; no effect here */
} oracle_source_options;

/* QSS integrator on any q/d right-hand side (QssOde::odefun). */
typedef void (*oracle_qss_fn)(void* ctx, double t, const double* y, double* q, double* d, int corrector);
typedef struct {
    double epsmin, epsmax, dtmin, dtmax, abstol;
    int itermax, stability_check;
} oracle_qss_params;
int oracle_qss_integrate(int n, oracle_qss_fn f, void* ctx, const oracle_qss_params* o, double* y,
                         const double* ymin, const int* enforce, double tf, double tstart, int max_steps,
                         double* work, int* stats);
/* The CHEMEQ2 cesium problem of test/old/test_qssintegrator.cpp. */
int oracle_qss_cesium(const oracle_qss_params* o, double* y7, double tf, int max_steps, int* stats);

double oracle_exp(double x);
double oracle_log(double x);
oracle_mech* oracle_mech_create(const oracle_mech_desc* d);
void oracle_mech_destroy(oracle_mech* m);
void oracle_mech_set_multipliers(oracle_mech* m, const double* mult);
oracle_ws* oracle_ws_create(const oracle_mech* m);
void oracle_ws_free(oracle_ws* w);
void oracle_rate_constants(const oracle_mech* m, oracle_ws* w, double T, int use_tables);
void oracle_rates(const oracle_mech* m, oracle_ws* w, double p, int model, int mode, double T, const double* Y,
                  double* rho_out, double* cp_out);
void oracle_gas_eval(const oracle_mech* m, double p, int model, int mode, int n, const double* T, const double* Y,
                     double* creation, double* destruction, double* net, double* hk, double* cp_mass,
                     double* density);
int oracle_qss_point(const oracle_mech* m, oracle_ws* w, const oracle_source_options* o, double* y,
                     const double* split, double tf, double t_start, double x, int* stats);
int oracle_bdf_point(const oracle_mech* m, oracle_ws* w, const oracle_source_options* o, double* y,
                     const double* split, double tf, double t_start, double x, int* stats);
/* Sum over species in the GPU block reductions' order (oracle_chem.c). */
double oracle_block_sum(const double* a, const double* b, int n, int W);
int oracle_reduction_width(int S);
/* Discrete adjoint of the QSS source-term integration (oracle_qss_adjoint.c). */
int oracle_qss_adjoint_point(const oracle_mech* m, oracle_ws* w, const oracle_source_options* o, const double* y_in,
                             const double* split, double tf, double t_start, double x, const double* ybar_out,
                             double* y_out, double* ybar_in, double* pbar, int* n_steps);
void oracle_qss_adjoint_batch(const oracle_mech* m, int n, const double* state_in, const double* split,
                              const double* dt, double t_start, const double* x, const oracle_source_options* o,
                              const double* ybar_out, double* state_out, double* ybar_in, double* pbar, int* status,
                              int* steps, int n_threads);
void oracle_source_batch(const oracle_mech* m, int method, int n, const double* state_in, const double* split,
                         const double* dt, double t_start, const double* x, const oracle_source_options* o,
                         double* state_out, int* status, int* stats, int n_threads);

/* ---- transport (oracle_transport.c) ------------------------------------- */
void oracle_transport_eval(const oracle_mech* m, const double* visc_fit, const double* cond_fit,
                           const double* diff_fit, int n, double p, double thr, const double* T, const double* Y,
                           double* density, double* mean_mw, double* cp_mass, double* cp_species, double* h_species,
                           double* conductivity, double* viscosity, double* rho_d);
void oracle_transport_eval_threads(const oracle_mech* m, const double* visc_fit, const double* cond_fit,
                                   const double* diff_fit, int n, double p, double thr, const double* T,
                                   const double* Y, double* density, double* mean_mw, double* cp_mass,
                                   double* cp_species, double* h_species, double* conductivity, double* viscosity,
                                   double* rho_d, int n_threads);

/* ---- convection stage (oracle_convection.c) ------------------------------ */
#define ORACLE_BC_FIXED_VALUE 0
#define ORACLE_BC_ZERO_GRADIENT 1
#define ORACLE_BC_CONTROL_VOLUME 2
#define ORACLE_BC_WALL_FLUX 3
#define ORACLE_CONT_LEFT 0
#define ORACLE_CONT_RIGHT 1
#define ORACLE_CONT_ZERO 2
#define ORACLE_CONT_QDOT 3
#define ORACLE_CONT_TEMP 4
typedef struct {
    int n_points, left_bc, right_bc, alpha, continuity_bc, j_cont;
    double beta, x_vzero, rv_zero, rv_cont, t_left, w_left, rhou, pressure;
    double strain_initial, strain_final, strain_t0, strain_dt;
    int strain_type, n_cheb;          /* 0 linear, 1 Chebyshev (cheb_t0, cheb_t1, cheb[n_cheb]) */
    double cheb_t0, cheb_t1;
    double cheb[16];
} oracle_conv_flame;
typedef struct {
    double reltol, abstol_u, abstol_t, abstol_y, min_step;
    int max_steps, max_history;
} oracle_conv_options;
void oracle_convection_strain(const oracle_conv_flame* fl, double t, double* a, double* dadt);
void oracle_adams_gammas(double* g);
void oracle_adams_l(int q, double* l);
void oracle_convection_grid(int N, const double* x, int alpha, double* hh, double* rph);
void oracle_convection_prepare(int N, int S, const double* W, const double* state, const double* split,
                               double* Wmx, double* sW);
void oracle_convection_utw_rhs(const oracle_conv_flame* fl, const double* x, const double* hh, const double* rph,
                               double t, const double* y, const double* drhodt, const double* sU,
                               const double* sT, const double* sW, double* ydot, double* rho, double* rV,
                               double* V);
int oracle_convection_interval(const double* ht, int H, double t, double* s);
void oracle_convection_drhodt(int n_pts, int n, int balanced, double pressure, const double* W, const double* state,
                              const double* ddt_conv, const double* ddt_diff, const double* ddt_prod,
                              const double* ddt_cross, double* drhodt);
int oracle_convection_flame(const oracle_conv_flame* fl, int S, const double* W, const double* x,
                            const double* y_left, double t0, double tf, const double* drhodt, const double* split,
                            double* state, const oracle_conv_options* o, int* status, int* stats,
                            int* n_history_out, double* hist_t_out, double* hist_v_out,
                            double* v_last, double* rv_last);

#ifdef __cplusplus
}
#endif

#endif
