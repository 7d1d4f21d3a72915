/*
 * ember_gpu.h -- C ABI of the GB300 (sm_103a) split-step hot path of Ember.
 *
 * The library (libember_gpu.so) replaces, at the stage level, the two CPU
 * loops of Ember's operator-split step:
 *
 *   - the diffusion stage: one TridiagonalIntegrator per state variable,
 *     fed by a DiffusionSystem (src/integrator.cpp:37-204,
 *     src/diffusionSystem.cpp:10-90), driven by
 *     FlameSolver::integrateDiffusionTerms / setDiffusionSolverState
 *     (src/flameSolver.cpp:702-718, 838-854);
 *   - the production (chemistry source term) stage: one SourceSystem per grid
 *     point (src/sourceSystem.cpp, src/qssintegrator.cpp), driven by
 *     FlameSolver::integrateProductionTerms (src/flameSolver.cpp:754-836).
 *
 * Conventions
 *   - Every entry point returns int: EMBER_OK (0) on success, a negative
 *     EMBER_E* code on failure. None throws; the message of the last failure
 *     on the calling thread is available from ember_last_error().
 *   - Array arguments are borrowed for the duration of the call only.
 *     `mem` selects where they live: EMBER_MEM_HOST (pageable or pinned host
 *     memory; the call copies in and out and synchronises its stream) or
 *     EMBER_MEM_DEVICE (device pointers; the call is asynchronous on
 *     `stream` unless stated otherwise).
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default
 *     stream), so this header needs no CUDA include.
 *   - All arithmetic is IEEE binary64.
 */
#ifndef EMBER_GPU_H
#define EMBER_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define EMBER_OK          0
#define EMBER_EINVAL     -1   /* bad argument (size, pointer, option)          */
#define EMBER_ECUDA      -2   /* a CUDA runtime call failed                      */
#define EMBER_ENOMEM     -3   /* device allocation failed                        */
#define EMBER_EFAIL      -4   /* at least one system/point failed: see status[] */

#define EMBER_MEM_HOST    0
#define EMBER_MEM_DEVICE  1

/* Boundary conditions, same numbering as BoundaryCondition::BC in the
 * reference (src/grid.h:7-26). Floating behaves as ZeroGradient in the
 * diffusion matrix, as in DiffusionSystem::get_A (src/diffusionSystem.cpp:47-58). */
#define EMBER_BC_FIXED_VALUE     0
#define EMBER_BC_ZERO_GRADIENT   1
#define EMBER_BC_CONTROL_VOLUME  2
#define EMBER_BC_WALL_FLUX       3
#define EMBER_BC_FLOATING        4

/* Copy the last error message of the calling thread into buf (NUL-terminated,
 * truncated to n bytes). Returns the full message length. */
int ember_last_error(char* buf, size_t n);

/* Library version as major*10000 + minor*100 + patch. */
int ember_version(void);

/* Number of CUDA devices visible (0 when none; never fails). */
int ember_device_count(void);

/* Measured FP64 throughput of the current device in FLOP/s, used as the
 * roofline denominator of the FP64-bound kernels. kind 0: FP64 FMA pipe
 * (DFMA); kind 1: FP64 tensor path (DMMA m8n8k4). No reference counterpart
 * (the reference has no GPU code). */
int ember_probe_fp64_rate(int kind, double* flops_per_second);

/* Cycles per FP64 warp instruction as seen by one warp: one CTA of `warps`
 * warps on every SM, the first `active_lanes` lanes of each warp running
 * `chains` (1: a dependent chain, latency; 8: independent chains, issue
 * rate) of op 0 (DFMA), 1 (DADD), 2 (DMUL), 3 (division), 4 (fmax and a
 * DADD), 5 (a compare, a DADD and a select), 6 (the reciprocal 1.0 / x) or
 * 7 (the reciprocal __drcp_rn); the median over SMs. No reference
 * counterpart. */
int ember_probe_fp64_issue(int op, int chains, int warps, int active_lanes, double* cycles_per_inst);

/* y[i] = exp, log, log10 or exp10 (op 0..3) of x[i], i < n (n <= 2^26), host
 * arrays, as the kinetics kernels evaluate them (their own FP64 exp and log;
 * exp10 x = exp(x ln 10), log10 x = log(x) log10(e)). For parity tests of
 * those functions. No reference counterpart (the reference calls the C
 * library's exp and log). */
int ember_math_eval(int op, const double* x, double* y, int64_t n);

/* ======================================================================
 * Batched tridiagonal integrator
 *
 * A batch of independent linear ODE systems  y' = A y + k  with tridiagonal
 * A (sub-diagonal a, diagonal b, super-diagonal c), integrated with the
 * reference's TridiagonalIntegrator scheme (src/integrator.cpp:133-204):
 * the first step after initialize() is 8 BDF1 sub-steps of h/8, later steps
 * are BDF2, each a Thomas solve with the factorisation cached per step kind;
 * integrate_to_time() rounds to an integral number of steps
 * (src/integrator.cpp:37-47).
 *
 * System s occupies elements [offsets[s], offsets[s+1]) of every per-point
 * array (CSR layout). Each system needs at least 2 points.
 * The batch object keeps y, y_prev, t, h, the step count and the factorised
 * coefficients on the device between calls, like one TridiagonalIntegrator
 * per system.
 * ==================================================================== */
typedef struct ember_tridiag_s* ember_tridiag;

/* Create a batch of n_systems systems; offsets (host, n_systems+1 entries,
 * offsets[0] == 0, strictly increasing by >= 2) is copied.
 * Replaces: TridiagonalIntegrator(ode) + resize(N) (src/integrator.cpp:77-108). */
int ember_tridiag_create(int n_systems, const int64_t* offsets, ember_tridiag* out);
int ember_tridiag_destroy(ember_tridiag batch);

/* Set the constant ODE coefficients a, b, c, k (each offsets[n] values).
 * Replaces: TridiagonalODE::get_A / get_k (src/integrator.h:22-35). */
int ember_tridiag_set_coefficients(ember_tridiag batch, const double* a, const double* b,
                                   const double* c, const double* k, int mem, void* stream);

/* Set the state (offsets[n] values) and reset the step count.
 * Replaces: TridiagonalIntegrator::set_y0 (src/integrator.cpp:111-115). */
int ember_tridiag_set_y0(ember_tridiag batch, const double* y0, int mem, void* stream);

/* Set start time and step size per system (n_systems values each) and reset
 * the step count. Replaces: TridiagonalIntegrator::initialize (src/integrator.cpp:117-122). */
int ember_tridiag_initialize(ember_tridiag batch, const double* t0, const double* h,
                             int mem, void* stream);

/* One step of every system. Replaces: TridiagonalIntegrator::step (src/integrator.cpp:133-204). */
int ember_tridiag_step(ember_tridiag batch, void* stream);

/* Integrate every system to its t_end (n_systems values).
 * Replaces: Integrator::integrateToTime (src/integrator.cpp:37-47). */
int ember_tridiag_integrate_to_time(ember_tridiag batch, const double* t_end, int mem, void* stream);

/* Read back y (offsets[n] values), t and h (n_systems values each; either may be NULL).
 * Replaces: get_y / get_t / get_h (src/integrator.cpp:25-35). */
int ember_tridiag_get_state(ember_tridiag batch, double* y, double* t, double* h,
                            int mem, void* stream);

/* y' = A y + k for the current state (offsets[n] values).
 * Replaces: TridiagonalIntegrator::get_ydot (src/integrator.cpp:124-131). */
int ember_tridiag_get_ydot(ember_tridiag batch, double* ydot, int mem, void* stream);

/* ======================================================================
 * Diffusion stage
 *
 * One call = FlameSolver::integrateDiffusionTerms() for a batch of flames
 * (src/flameSolver.cpp:838-854 with setDiffusionSolverState, 702-718):
 * for every flame f and state variable v the matrix of DiffusionSystem::get_A
 * and the constant of get_k are built from the grid, B, D, the split constant
 * and the boundary conditions (src/diffusionSystem.cpp:10-76); the step size is
 *     h = min(dt_multiplier * min_{1<=j<=N-2} dlj_j^2 / (B_j D_j), global_timestep)
 * unless h is given explicitly; the system is initialised at t_start and
 * integrated to t_end with the tridiagonal scheme above.
 *
 * Layout: flame f has n_points N_f; per-point arrays are concatenated over
 * flames, and inside flame f they are variable-major: element (v, j) of
 * flame f is at  var_offset_f + v*N_f + j  where var_offset_f =
 * n_vars * sum_{g<f} N_g. (This is the row layout of DiffusionSystem::B/D/
 * splitConst and of state.row(v).) Grid coordinates x are concatenated over
 * flames (point_offset_f = sum_{g<f} N_g).
 * ==================================================================== */
typedef struct {
    int n_points;   /* N_f >= 3                                          */
    int left_bc;    /* EMBER_BC_*                                        */
    int right_bc;   /* EMBER_BC_FIXED_VALUE / ZERO_GRADIENT / FLOATING   */
    int alpha;      /* grid curvature exponent: 0 planar, 1 cylindrical  */
} ember_diffusion_grid;

typedef struct {
    double t_start;            /* tStageStart                                   */
    double t_end;              /* tStageEnd                                     */
    double dt_multiplier;      /* Times.diffusionTimestepMultiplier (10)        */
    double global_timestep;    /* Times.globalTimestep (2e-5)                   */
    const double* h;           /* NULL, or explicit step per (flame, var)       */
    const double* wall_const;  /* NULL (0), or per (flame, var): DiffusionSystem::wallConst */
    const double* y_inf;       /* NULL (0), or per (flame, var): DiffusionSystem::yInf      */
    int algorithm;             /* EMBER_DIFFUSION_PARALLEL (0) or EMBER_DIFFUSION_SERIAL (1) */
} ember_diffusion_options;

/* EMBER_DIFFUSION_PARALLEL: one warp per system; the Thomas factorisation and
 * every forward / backward sweep are split into 32 chunks joined by exact
 * prefix scans (Moebius 2x2 products for the factorisation, affine maps for
 * the sweeps); agrees with the reference's sequential Thomas algorithm to
 * rounding (~1e-15 relative).
 * EMBER_DIFFUSION_SERIAL: one thread per system in the reference's operation
 * order, bitwise identical to TridiagonalIntegrator on the CPU. */
#define EMBER_DIFFUSION_PARALLEL 0
#define EMBER_DIFFUSION_SERIAL   1

/* x: grid coordinates; B, D, split_const: per point and variable (layout
 * above); y: state in/out (same layout); status: n_flames*n_vars ints
 * (0 = ok), may be NULL. Per-(flame,var) option arrays live in the same
 * memory space as the other arrays. */
int ember_diffusion_integrate(int n_flames, const ember_diffusion_grid* grids, int n_vars,
                              const double* x, const double* B, const double* D,
                              const double* split_const, double* y,
                              const ember_diffusion_options* opts, int* status,
                              int mem, void* stream);

/* Adjoint of ember_diffusion_integrate with respect to the state: the stage
 * is linear in y (y_out = M y_in + terms of the split constants), so for
 * phi = ybar . y_out the gradient d phi / d y_in = M^T ybar; ybar (layout of
 * y) is replaced by it. The sub-steps are run backwards with transposed
 * Thomas solves (same rows, step-size rule and step count as the forward
 * stage). B, D, wall_const are held fixed; split_const and y_inf do not enter M. */
int ember_diffusion_adjoint(int n_flames, const ember_diffusion_grid* grids, int n_vars, const double* x,
                            const double* B, const double* D, double* ybar, const ember_diffusion_options* opts,
                            int* status, int mem, void* stream);

/* Allocation-free variant of ember_diffusion_integrate, for callers that
 * must not allocate device memory while they step: an application whose
 * device memory is owned by another allocator (a framework's caching pool or
 * a budget fixed at start-up), or code whose footprint must stay constant
 * after initialisation. It has no counterpart in the reference (which runs on
 * the CPU). Same arguments and results as ember_diffusion_integrate with
 * EMBER_MEM_DEVICE (all arrays are device pointers; the call is asynchronous
 * on `stream`; it always runs EMBER_DIFFUSION_SERIAL, whatever
 * opts->algorithm says), but its workspace is a fixed device array inside the library,
 * sized for EMBER_NOALLOC_MAX_VALUES values (n_vars x total points) and
 * EMBER_NOALLOC_MAX_SYSTEMS (flame, variable) systems, about 28.3 MiB that
 * every GPU which loads the library keeps until the process exits. Larger
 * problems are rejected with EMBER_EINVAL. The call makes no device
 * allocation (no cudaMalloc, cudaFree or allocating library routine) and no
 * host heap allocation: the per-system descriptors are built on the device
 * from kernel parameters. The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress); make that first call before any stream capture.
 * Every call uses the same array: calls whose kernels can overlap on the GPU
 * (other streams, other host threads) race and corrupt each other's results;
 * issue them on one stream. No part of the array needs to start at zero:
 * every element a call reads is written earlier in the same call. With
 * status == NULL the per-system status is kept in the array. */
#define EMBER_NOALLOC_MAX_VALUES  524288
#define EMBER_NOALLOC_MAX_SYSTEMS 8192
int ember_diffusion_integrate_noalloc(int n_flames, const ember_diffusion_grid* grids, int n_vars,
                                      const double* x, const double* B, const double* D,
                                      const double* split_const, double* y,
                                      const ember_diffusion_options* opts, int* status, void* stream);

/* ======================================================================
 * Convection stage
 *
 * One call = ConvectionSystemSplit::integrateToTime for a batch of flames
 * (src/convectionSystem.cpp:588-627, with setState 485-511 and
 * setSplitConstants 572-586): per flame the UTW system
 * (ConvectionSystemUTW::f, src/convectionSystem.cpp:14-130: continuity
 * integral for rV from the continuity point, upwinded convection of U, T and
 * the mean molecular weight W, strain-rate source of U) is integrated from
 * t_start to t_end, stopping on t_end, and V / rho is recorded after every
 * step; then every species system (ConvectionSystemY::f, 307-359, upwinded
 * convection of Y_k) is integrated to t_end with v(t) interpolated from that
 * record as ConvectionSystemY::update_v does (372-398). The reference runs
 * CVODE's Adams method with a zero-bandwidth difference-quotient Jacobian for
 * both (src/convectionSystem.cpp:467-478, 663-676); this library runs an own
 * variable-order (1..12) Adams-Moulton integrator with a diagonal
 * difference-quotient Jacobian (same step and order control as its BDF).
 *
 * Layout: flame f has n_points N_f; x and drhodt are concatenated over
 * flames; state and split_const are variable-major per flame (U, T, Y_0 ..
 * Y_{S-1}; element (v, j) at var_offset_f + v*N_f + j, as for the diffusion
 * stage); y_left holds S mass fractions per flame. U, T and Y are replaced by
 * the stage's result; W is not part of the state (the reference keeps it
 * inside the convection system).
 * ==================================================================== */
#define EMBER_CONTINUITY_LEFT  0   /* fixedLeft: rV[0] = rv_zero                      */
#define EMBER_CONTINUITY_RIGHT 1   /* fixedRight: rV[j_cont] = rv_cont, j_cont = N-1  */
#define EMBER_CONTINUITY_ZERO  2   /* stagnationPoint: V = 0 at x_vzero               */
#define EMBER_CONTINUITY_QDOT  3   /* fixedQdot: rV[j_cont] = rv_cont                 */
#define EMBER_CONTINUITY_TEMP  4   /* fixedTemperature: dT/dt = 0 at j_cont           */

/* Largest flame: the continuity integral of a flame is staged in shared memory. */
#define EMBER_CONVECTION_MAX_POINTS 8192

/* Strain-rate function a(t) of a flame (src/scalarFunction.h). */
#define EMBER_STRAIN_LINEAR    0   /* LinearFunction: strain_initial/final/t0/dt          */
#define EMBER_STRAIN_CHEBYSHEV 1   /* ChebyshevFunction: cheb_t0, cheb_t1, cheb[n_cheb]   */
#define EMBER_CHEBYSHEV_MAX    16  /* coefficients per flame                              */

typedef struct {
    int n_points;          /* 3 <= N_f <= EMBER_CONVECTION_MAX_POINTS                 */
    int left_bc;           /* EMBER_BC_FIXED_VALUE / ZERO_GRADIENT / CONTROL_VOLUME / WALL_FLUX */
    int right_bc;          /* EMBER_BC_FIXED_VALUE, else outflow when V > 0 there     */
    int alpha;             /* 0 planar, 1 cylindrical                                 */
    int continuity_bc;     /* EMBER_CONTINUITY_*                                      */
    int j_cont;            /* jContBC (ignored for LEFT)                              */
    double beta;           /* grid.beta                                               */
    double x_vzero;        /* xVzero (ZERO)                                           */
    double rv_zero;        /* rVzero (LEFT)                                           */
    double rv_cont;        /* rV[jContBC] carried into the stage (RIGHT, QDOT): the
                              reference's f() leaves it as it was                    */
    double t_left;         /* Tleft                                                   */
    double w_left;         /* Wleft, mean molecular weight at the left boundary       */
    double rhou;           /* unburned density                                        */
    double pressure;       /* Pa                                                      */
    double strain_initial, strain_final, strain_t0, strain_dt;  /* a(t): LinearFunction
                              (src/scalarFunction.cpp:12-22); equal initial and final
                              values give a constant strain rate                     */
    int strain_type;       /* EMBER_STRAIN_LINEAR (the fields above) or
                              EMBER_STRAIN_CHEBYSHEV (the fields below)               */
    int n_cheb;            /* Chebyshev coefficients in cheb (0..EMBER_CHEBYSHEV_MAX):
                              ChebyshevFunction::setCoefficients(2 + n_cheb, {cheb_t0,
                              cheb_t1, cheb...}) (src/scalarFunction.cpp:31-49)        */
    double cheb_t0, cheb_t1;  /* the interval mapped onto [-1, 1]                      */
    double cheb[EMBER_CHEBYSHEV_MAX];
} ember_convection_flame;

typedef struct {
    double t_start, t_end;   /* tStageStart, tStageEnd                                */
    double reltol;           /* integratorRelTol (1e-6)                               */
    double abstol_u;         /* integratorMomentumAbsTol (1e-7)                       */
    double abstol_t;         /* integratorEnergyAbsTol (1e-8)                         */
    double abstol_y;         /* integratorSpeciesAbsTol (1e-13); W uses 20 times it   */
    double min_step;         /* minStep (1e-16)                                       */
    int max_steps;           /* per system                                            */
    int max_history;         /* recorded V / rho per flame: UTW steps + 1             */
    int species_threads;     /* CTA width of a species system: 0 or 32 (one warp)     */
} ember_convection_options;

/* status: n_flames * (1 + S) ints, may be NULL: per flame the UTW status
 * then one per species (0 ok; -11 too many steps, -13 error-test failures,
 * -14 convergence failures, -20 record full; a failed UTW integration marks
 * its species with its own status and leaves them unchanged). stats:
 * n_flames * 4 ints or NULL: UTW steps, UTW right-hand sides, species steps
 * and right-hand sides summed over species. Per-flame structs and opts are
 * host memory; every array is in the `mem` space. */
int ember_convection_integrate(int n_flames, const ember_convection_flame* flames, int n_species,
                               const double* mol_weight, const double* x, const double* y_left,
                               const double* drhodt, const double* split_const, double* state,
                               const ember_convection_options* opts, int* status, int* stats, int mem,
                               void* stream);

/* ======================================================================
 * Mechanism tables
 *
 * A gas-phase mechanism compiled once into structure-of-arrays device
 * tables: NASA7 thermo per species and, per reaction, modified Arrhenius
 * parameters, third-body efficiencies, Lindemann/Troe falloff data and the
 * species occurrences on each side. Units are Cantera's internal SI-kmol
 * units (kmol, m^3, s, K; activation energies as Ea/R in K).
 * Replaces the Cantera objects built by CanteraGas::initialize
 * (src/chemistry0d.cpp:455-485) for the kinetics/thermo the source term uses.
 * ==================================================================== */
#define EMBER_MAX_STOICH 4        /* species occurrences per reaction side */

#define EMBER_RXN_ELEMENTARY 0
#define EMBER_RXN_THREE_BODY 1    /* rate multiplied by [M]                  */
#define EMBER_RXN_LINDEMANN  2    /* falloff, F = 1                          */
#define EMBER_RXN_TROE       3    /* falloff, Troe F                         */

typedef struct {
    int n_species;
    int n_reactions;
    const double* mol_weight;        /* [S] kg/kmol                                        */
    const double* nasa_tmid;         /* [S] K; the low-T coefficients apply for T <= tmid  */
    const double* nasa_coeffs;       /* [S][14]: a0..a6 low range, then a0..a6 high range  */
    const int* rxn_type;             /* [R] EMBER_RXN_*                                     */
    const int* reversible;           /* [R] 0 or 1                                          */
    const int* reactants;            /* [R][EMBER_MAX_STOICH] species per occurrence, -1 = none */
    const int* products;             /* [R][EMBER_MAX_STOICH]                               */
    const double* arrhenius;         /* [R][3]: A, b, Ea/R; high-pressure limit for falloff */
    const double* arrhenius_low;     /* [R][3]: low-pressure limit (falloff rows only)      */
    const double* troe;              /* [R][4]: a, T3, T1, T2 (T2 == 0: term absent)        */
    const double* default_efficiency;/* [R] third-body default efficiency                   */
    const int64_t* efficiency_offsets;/* [R+1] CSR into the two arrays below                */
    const int* efficiency_species;
    const double* efficiency_values;
} ember_mech_desc;

typedef struct ember_mech_s* ember_mech;

/* Validate and upload a mechanism; builds the per-species reaction lists and
 * the interpolation tables of the 'interp' kinetics model on the device. */
int ember_mech_create(const ember_mech_desc* desc, ember_mech* out);
int ember_mech_destroy(ember_mech mech);

/* Per-reaction rate multipliers (n_reactions values; NULL resets to 1).
 * Replaces: Kinetics::setMultiplier as used by CanteraGas::setRateMultiplier
 * (src/chemistry0d.cpp:634-642), per reaction. */
int ember_mech_set_multipliers(ember_mech mech, const double* multipliers, int mem, void* stream);

/* Kinetics models (Chemistry.kineticsModel, python/ember/input.py:371). */
#define EMBER_KINETICS_STANDARD 0  /* rate constants and equilibrium constants from the formulas */
#define EMBER_KINETICS_INTERP   1  /* InterpKinetics + MultiArrheniusInterp tables
                                      (src/chemistry0d.cpp:271-436)          */

/* Composition handling of the state setter. */
#define EMBER_STATE_NORMALIZED 0   /* setState_TPY: negative Y clipped, sum normalised */
#define EMBER_STATE_NO_NORM    1   /* setMassFractions_NoNorm + setState_TP            */

/* Thermo and rates for a batch of states (n_points; Y point-major [n][S]).
 * Outputs (any may be NULL): creation/destruction/net production rates
 * [n][S] kmol/m^3/s, partial molar enthalpies hk [n][S] J/kmol, cp_mass [n]
 * J/kg/K, density [n] kg/m^3. Replaces: CanteraGas::setStateMass /
 * getCreationRates / getDestructionRates / getReactionRates / getEnthalpies /
 * getSpecificHeatCapacity / getDensity (src/chemistry0d.cpp:487-672). */
int ember_gas_eval(ember_mech mech, int n_points, double pressure, int kinetics_model, int state_mode,
                   const double* T, const double* Y, double* creation, double* destruction, double* net,
                   double* hk, double* cp_mass, double* density, int mem, void* stream);

/* ======================================================================
 * Thermo and transport properties of the flame state
 *
 * One call = FlameSolver::updateChemicalProperties (src/flameSolver.cpp:
 * 652-699) for a batch of grid points with the default transport model
 * "Approx" (ApproxMixTransport, src/chemistry0d.cpp:12-269): density, mean
 * molecular weight, cp, partial molar cp and enthalpies; mixture-averaged
 * thermal conductivity (0.5 (sum X_k lambda_k + 1 / sum X_k / lambda_k)),
 * viscosity (Wilke's rule over the species whose mole fraction is at least
 * `threshold`, ApproxMixTransport::viscosity / updateViscosity_T, 22-52 and
 * 181-205) and the mass-based mixture diffusion coefficients times density
 * (CanteraGas::getWeightedDiffusionCoefficientsMass, 583-591, over
 * ApproxMixTransport::getMixDiffCoeffsMass, 98-139, whose sums run over all
 * species for a major species and over the major species otherwise).
 * threshold = 0 gives Cantera's plain mixture-averaged model ("Mix").
 * Mole fractions are floored at 1e-20 for the transport sums, as Cantera's
 * MixTransport does. Species properties come from polynomial fits in ln T
 * (Cantera's non-CK fitting form):
 *   sqrt(mu_k) = T^(1/4) P(ln T),  lambda_k = T^(1/2) P(ln T),
 *   p D_jk     = T^(3/2) P(ln T)   (D at pressure p),
 * P(x) = c0 + c1 x + c2 x^2 + c3 x^3 + c4 x^4. Thermal diffusion (Soret) is
 * not computed: Ember turns it off for "Approx" (python/ember/input.py:377-383).
 * ==================================================================== */
typedef struct {
    int n_species;
    const double* visc_fit;   /* [S][5] mu_k in Pa s                                            */
    const double* cond_fit;   /* [S][5] lambda_k in W/m/K                                       */
    const double* diff_fit;   /* [S(S+1)/2][5] D_jk in m^2/s; pair j <= k at j S - j(j-1)/2 + k - j */
} ember_transport_desc;

typedef struct ember_transport_s* ember_transport;

/* Upload the fits of a mechanism's species (n_species must match mech). */
int ember_transport_create(ember_mech mech, const ember_transport_desc* desc, ember_transport* out);
int ember_transport_destroy(ember_transport tr);

/* Outputs of ember_transport_eval (point-major; any pointer may be NULL). */
typedef struct {
    double* density;       /* [n] kg/m^3                      (rho)     */
    double* mean_mol_weight;/* [n] kg/kmol                    (Wmx)     */
    double* cp_mass;       /* [n] J/kg/K                      (cp)      */
    double* cp_species;    /* [n][S] partial molar cp J/kmol/K (cpSpec) */
    double* h_species;     /* [n][S] partial molar h J/kmol   (hk)      */
    double* conductivity;  /* [n] W/m/K                       (lambda)  */
    double* viscosity;     /* [n] Pa s                        (mu)      */
    double* rho_d;         /* [n][S] rho D_k kg/m/s           (rhoD)    */
} ember_properties;

/* T [n], Y [n][S] (normalised as setState_TPY: negative Y clipped, sum 1). */
int ember_transport_eval(ember_transport tr, int n_points, double pressure, double threshold, const double* T,
                         const double* Y, const ember_properties* out, int mem, void* stream);

/* ======================================================================
 * Production (chemistry source term) stage
 *
 * One call = FlameSolver::integrateProductionTerms() for a batch of grid
 * points (src/flameSolver.cpp:754-836): every point is an independent
 * constant-pressure reactor with state [U, T, Y_0..Y_{S-1}] (nVars = S+2,
 * the column of FlameSolver::state), integrated over its own dt with the
 * split constant of SourceSystem::splitConst, by
 *   EMBER_SOURCE_QSS: SourceSystemQSS + QssIntegrator
 *                     (src/sourceSystem.cpp:403-531, src/qssintegrator.cpp);
 *   EMBER_SOURCE_BDF: SourceSystemCVODE's right-hand side integrated by a
 *                     variable-order BDF with Newton iteration over a dense
 *                     LU of an analytic Jacobian, following CVODE's published
 *                     method (replaces src/sundialsUtils.cpp:33-172).
 * Per-point arrays are point-major: element (j, i) at j*nVars + i.
 * ==================================================================== */
#define EMBER_SOURCE_QSS 0
#define EMBER_SOURCE_BDF 1

/* Per-point status (the int returned by SourceSystem::integrateToTime). */
#define EMBER_SRC_OK            0
#define EMBER_SRC_DTMIN        -1    /* QSS: step below dtmin (qssintegrator.cpp:198-215)      */
#define EMBER_SRC_TOO_MUCH_WORK -11  /* BDF: max_num_steps reached (CVODE CV_TOO_MUCH_WORK)     */
#define EMBER_SRC_ERR_FAILURE   -13  /* BDF: repeated error-test failures (CV_ERR_FAILURE)      */
#define EMBER_SRC_CONV_FAILURE  -14  /* BDF: repeated Newton failures (CV_CONV_FAILURE)         */
#define EMBER_SRC_STEP_LIMIT    -20  /* QSS: the device step cap max_steps was reached          */
#define EMBER_SRC_NONFINITE     -21  /* a NaN/inf appeared in the state                         */

#define EMBER_STATS_WIDTH 4          /* per point: steps, rhs calls, repeats/failures, Jacobians */

typedef struct {
    double pressure;              /* Pa (General.pressure)                              */
    int kinetics_model;           /* EMBER_KINETICS_*                                   */
    int max_steps;                /* device cap on internal steps per point (> 0)      */
    /* QssTolerances (python/ember/input.py:752-775) */
    double qss_epsmin, qss_epsmax, qss_dtmin, qss_dtmax, qss_abstol, qss_minval;
    int qss_iteration_count, qss_stability_check;
    /* CvodeTolerances (python/ember/input.py:733-745) */
    double bdf_reltol, bdf_abstol_momentum, bdf_abstol_energy, bdf_abstol_species, bdf_min_step;
    int bdf_max_num_steps;
    /* threads per grid point (one CTA per point): 0 = the width
     * ember_source_autotune chose for the mechanism, else the default for its
     * size; or 32, 64, 96, 128, 160, 192, 256 (QSS) / 32, 64, 128, 160, 256 (BDF;
     * other values give the mechanism's width). Results do not depend on it
     * (every reduction runs in one fixed 32-lane order). */
    int threads_per_point;
    /* ignition source of SourceSystem::getQdotIgniter (src/sourceSystem.cpp:33-45);
     * ignition_energy == 0 disables it */
    double ignition_tstart, ignition_duration, ignition_energy, ignition_center, ignition_stddev;
    /* QSS two-pass schedule: 0 = the mechanism's tuned schedule (none unless
     * ember_source_autotune found one faster). qss_tail_steps > 0: points
     * still running after that many steps are suspended and resumed, after
     * the others, on CTAs of qss_tail_threads threads (0: 256), so that the
     * stiffest points finish sooner. Results do not depend on it. Not with
     * qss_stability_check. */
    int qss_tail_steps, qss_tail_threads;
    /* BDF placement of the Jacobian and LU factors (codes of
     * ember_mech_get_tuning: 1 both in shared memory, 2 LU only, 3 neither,
     * 4 LU and the rates of progress); 0: the mechanism's tuned placement,
     * else the first that fits. Results do not depend on it. */
    int bdf_layout;
} ember_source_options;

/* Fill `opts` with the reference's defaults (pressure 1 atm, interp kinetics). */
int ember_source_options_default(ember_source_options* opts);

/* state_in/state_out: [n_points][nVars]; split_const: same layout or NULL (0);
 * dt: [n_points] integration interval (tf relative to t_start); x: grid
 * positions for the igniter or NULL; status: [n_points] EMBER_SRC_*; stats:
 * [n_points][EMBER_STATS_WIDTH] or NULL. Returns EMBER_EFAIL (after writing
 * every output) when at least one point failed. */
int ember_source_integrate(ember_mech mech, int method, int n_points, const double* state_in,
                           const double* split_const, const double* dt, double t_start, const double* x,
                           const ember_source_options* opts, double* state_out, int* status, int* stats,
                           int mem, void* stream);

/* Autotuner of the source-term launch: integrates the given points (a sample
 * of the workload; the same arguments as ember_source_integrate) once per
 * candidate, times each run on the stream with CUDA events (after one untimed
 * run), and stores the fastest candidate in the mechanism handle, where calls
 * whose threads_per_point is 0 pick it up. QSS candidates: every width of
 * EMBER_SOURCE_THREAD_CHOICES. BDF candidates: the widths 32, 64, 128, 160, 256
 * times every placement of the Jacobian and LU factors that fits (both in
 * shared memory, the LU factors alone, neither). threads_out: the chosen
 * width; ms_out: [EMBER_SOURCE_N_THREAD_CHOICES] milliseconds per width (the
 * best placement for BDF; 0 for widths not tried) or NULL. For QSS it then
 * tries two-pass schedules and work-queue granularities of 2 and 4 points
 * per claim with the best width. Integration results are identical for
 * every candidate. */
#define EMBER_SOURCE_N_THREAD_CHOICES 7
#define EMBER_SOURCE_THREAD_CHOICES {32, 64, 96, 128, 160, 192, 256}
int ember_source_autotune(ember_mech mech, int method, int n_points, const double* state_in, const double* split_const,
                          const double* dt, double t_start, const double* x, const ember_source_options* opts,
                          int* threads_out, double* ms_out, int mem, void* stream);

/* The launch configuration stored in the mechanism by ember_source_autotune
 * (0 where none was chosen): QSS width, QSS two-pass steps and tail width, QSS
 * work-queue granularity (points a CTA claims per atomic), BDF width, BDF
 * matrix placement (1: J and LU in shared memory, 2: LU only, 3: neither,
 * 4: LU and the rates of progress).
 * ember_source_autotune changes the mechanism handle: do not call it while
 * other threads launch work with the same mechanism. */
int ember_mech_get_tuning(ember_mech mech, int* qss_threads, int* qss_tail_steps, int* qss_tail_threads,
                          int* qss_chunk, int* bdf_threads, int* bdf_layout);

/* Discrete adjoint of a BDF source-term integration (EMBER_SOURCE_BDF, same
 * arguments as ember_source_integrate): for phi = sum over points of
 * state_bar . state_out, returns state_in_bar = d phi / d state_in
 * [n_points][nVars] and lnk_bar = d phi / d ln(multiplier_i) of every
 * reaction [n_reactions], summed over points (or NULL). The forward pass
 * records every accepted step (at most tape_cap per point; 0: 1024); the
 * backward pass linearises each step with its step size and order held
 * fixed and the corrector converged, with the analytic Jacobian recomputed at
 * the step's end state and the transposed solve on the LU of I - gamma J.
 * There is no counterpart in the reference (CVODE is run forward only); it
 * serves the gradients of FlameSolver's objectives. status: as
 * ember_source_integrate, or -30 (tape overflow), -32 (singular matrix). */
int ember_source_adjoint(ember_mech mech, int n_points, const double* state_in, const double* split_const,
                         const double* dt, double t_start, const double* x, const ember_source_options* opts,
                         const double* state_bar, int tape_cap, double* state_out, int* status,
                         double* state_in_bar, double* lnk_bar, int mem, void* stream);

/* Discrete adjoint of a QSS source-term integration (EMBER_SOURCE_QSS, the
 * reference's default integrator; same arguments as ember_source_adjoint).
 * For phi = sum over points of state_bar . state_out, returns state_in_bar =
 * d phi / d state_in [n_points][nVars] and lnk_bar = d phi / d
 * ln(multiplier_i) of every reaction [n_reactions], summed over points (or
 * NULL). The integration is differentiated as it runs: every attempt of every
 * step (a retried attempt's predictor uses the rejected attempt's corrector
 * rates), the step sizes as functions of the state (getInitialStepSize, the
 * error-estimate rule dt (1/sqrt(eps) + 0.005), the clip to the end time),
 * the right-hand side analytically in the mass fractions and by a forward
 * difference in T; accept / reject decisions are held fixed. Finite
 * differences of the adaptive forward map agree with it to their own noise
 * at the reference's default tolerances. Needs qss_stability_check = 0 and
 * qss_iteration_count 1-4. tape_cap: step starts the forward pass records per
 * point (0: 4096) while the whole record fits in 2 GiB; points that need more,
 * or all points beyond that size, are integrated again by the adjoint with a
 * record of max(tape_cap, 4096) step starts per point.
 * There is no counterpart in the reference (QssIntegrator runs forward
 * only); it serves the gradients of FlameSolver's objectives
 * (src/flameSolver.cpp:926-961) with the QSS source
 * (src/qssintegrator.cpp:58-265, src/sourceSystem.cpp:403-531).
 * status: as ember_source_integrate, or -30 (tape full), -33 (more than 32
 * attempts in one step). */
int ember_source_adjoint_qss(ember_mech mech, int n_points, const double* state_in, const double* split_const,
                             const double* dt, double t_start, const double* x, const ember_source_options* opts,
                             const double* state_bar, int tape_cap, double* state_out, int* status,
                             double* state_in_bar, double* lnk_bar, int mem, void* stream);

/* Known-answer self-test of the device QSS integrator: integrates the
 * CHEMEQ2 cesium relaxation problem of the reference's QSS test
 * (test/old/test_qssintegrator.cpp:11-83) from y7 (7 values, in/out) over
 * [0, tf] with the given QssIntegrator settings, and sets y7[6] from charge
 * balance as that test does. stats: steps, right-hand-side calls, repeats, 0.
 * Returns the integrator's status (0, -1 dtmin, -20 step cap) or an EMBER_E*
 * code. */
int ember_selftest_qss_cesium(double epsmin, double epsmax, double dtmin, double dtmax, double abstol,
                              int itermax, int stability_check, double tf, int max_steps, double* y7,
                              int* stats);

/* ======================================================================
 * Split step of a batch of flames on the device
 *
 * One ember_split_step = SplitSolver::step for every flame of the batch
 * (src/splitSolver.cpp:34-121): split constants from the previous step's
 * time derivatives; diffusion over [t, t+dt/4] and [t+dt/4, t+dt/2]; source
 * term over [t, t+dt]; diffusion over [t+dt/2, t+3dt/4] and [t+3dt/4, t+dt];
 * time derivatives ddt = delta/dt - split constant
 * (SplitSolver::calculateTimeDerivatives, 27-32); the mass-fraction
 * correction of FlameSolver::finishStep (src/flameSolver.cpp:219-224,
 * 942-949); t += dt. The stage hooks are those of FlameSolver
 * (integrateDiffusionTerms / integrateProductionTerms, src/flameSolver.cpp:
 * 702-854), batched over flames.
 *
 * Not integrated here: the convection stages (ConvectionSystemSplit is not
 * part of this library). A caller that runs them supplies their rate through
 * ddt_cross. With balanced splitting the split constants of the two
 * integrated operators give each half of the total rate,
 *   c_diff = (ddt_prod + ddt_cross - ddt_diff) / 2,
 *   c_prod = (ddt_diff + ddt_cross - ddt_prod) / 2
 * (the reference's three-operator rule gives 1/4, 1/4, 1/2); without it,
 * c_diff = ddt_cross and c_prod = 0 as in the reference.
 *
 * The state is point-major [n_points][S+2] (U, T, Y_0..), flames
 * concatenated, as FlameSolver::state. B and D are the diffusion
 * coefficients of every (flame, variable) row, variable-major per flame as
 * in ember_diffusion_integrate (DiffusionSystem::B, D: 1/rho and mu for U,
 * 1/(rho cp) and lambda for T, 1/rho and rho D_k for Y_k,
 * src/flameSolver.cpp:160-172); they are held fixed until the next
 * ember_split_set_transport. Every array lives on the device between calls;
 * a step launches kernels and device copies only, so it can be captured:
 * ember_split_step(.., use_graph = 1, ..) captures one step into a CUDA graph
 * on first use and replays it (stage times come from a device clock).
 * ==================================================================== */
typedef struct ember_split_s* ember_split;

typedef struct {
    int method;                  /* EMBER_SOURCE_QSS or EMBER_SOURCE_BDF           */
    int diffusion_algorithm;     /* EMBER_DIFFUSION_PARALLEL or _SERIAL            */
    int balanced;                /* splittingMethod == "balanced"                  */
    double dt;                   /* options.globalTimestep                         */
    double dt_multiplier;        /* options.diffusionTimestepMultiplier (10)       */
    ember_source_options source; /* source-term options                            */
} ember_split_options;

/* grids / x (host): the flames' grids (x concatenated). The mechanism must
 * outlive the split object. */
int ember_split_create(ember_mech mech, int n_flames, const ember_diffusion_grid* grids, const double* x,
                       const ember_split_options* opts, ember_split* out);
int ember_split_destroy(ember_split split);
/* State at time t; resets the time derivatives (and so the split
 * constants of the next step) and the failure counters. */
int ember_split_set_state(ember_split split, double t, const double* state, int mem, void* stream);
/* Replace the state values only: the time, the time derivatives (the next
 * step's split constants) and the failure counters are kept, as when a caller
 * that holds the state on the host hands back the state of the last step. */
int ember_split_load_state(ember_split split, const double* state, int mem, void* stream);
/* B, D: variable-major per flame; ddt_cross: point-major or NULL (zero). */
int ember_split_set_transport(ember_split split, const double* B, const double* D, const double* ddt_cross,
                              int mem, void* stream);
/* Attach a transport model (NULL detaches): every following step starts as
 * FlameSolver::step does (src/flameSolver.cpp:130-154, 156-172, 551-617),
 * from the state at the step start and on the device:
 *   updateChemicalProperties  ember_transport_eval with `threshold`;
 *   prepareIntegrators        B, D of every variable (1/rho and mu for U,
 *                             1/(rho cp) and lambda for T, 1/rho and rho D_k
 *                             for Y_k), replacing ember_split_set_transport's;
 *   updateCrossTerms          (cross_terms != 0) Fick fluxes, the correction
 *                             flux smoothed by a tridiagonal integration over
 *                             [0, dt] (B = lambda/(rho cp), D = 1, the jCorr
 *                             step-size rule), the species and temperature
 *                             cross terms into ddt_cross. Thermal diffusion
 *                             (Soret) is not included.
 * The properties are part of the captured graph. The split-step adjoint holds
 * B and D fixed and so requires no transport model. */
int ember_split_set_transport_model(ember_split split, ember_transport tr, double threshold, int cross_terms);

/* Add the convection stage to every split step: the step becomes the
 * reference's D(1/4) C(1/2) D(1/4) S D(1/4) C(1/2) D(1/4)
 * (SplitSolver::integrateSplitTerms, src/splitSolver.cpp:60-76) with the
 * three-operator balanced split constants (38-46) and the convection stage's
 * density derivative from the step's time derivatives (FlameSolver::
 * prepareIntegrators, src/flameSolver.cpp:208-213). flames: one per flame
 * of the handle (n_points and alpha as its grid); y_left: S mass fractions
 * per flame; opts: tolerances and limits of ember_convection_integrate
 * (t_start, t_end unused). flames == NULL detaches the stage. Host memory;
 * the handle keeps its own copies and a fixed workspace, so the stage is part
 * of the captured step graph. The flames' continuity points (j_cont, x_vzero,
 * rv_cont) are the caller's for the first step after this call or
 * ember_split_set_state; at the start of every later step they are updated on
 * the device as ConvectionSystemUTW::updateContinuityBoundaryCondition does
 * (src/convectionSystem.cpp:196-277), from the step-start temperature, its
 * heat release rate (fixedQdot) and V / rV of the last UTW evaluation. The split-step adjoint covers D-S-D only and
 * refuses a handle with the stage attached. */
int ember_split_set_convection(ember_split split, const ember_convection_flame* flames, const double* y_left,
                               const ember_convection_options* opts);
/* The strain rate of every flame becomes a Chebyshev series, as
 * FlameSolver's strainfunc after ChebyshevFunction::setCoefficients
 * (src/scalarFunction.cpp:31-49), which the Python layer calls before each
 * step with the series fitted over [tNow, tNow + dt]
 * (python/ember/_ember.pyx:521-531). coeffs: host, per flame 2 + n_coeffs
 * values {t0, t1, c_0 .. c_{n_coeffs-1}} (0 <= n_coeffs <=
 * EMBER_CHEBYSHEV_MAX). Needs the convection stage attached; takes effect
 * from the next step, captured graph included (the flames' records are
 * updated in device memory). Returns when the update is done on `stream`. */
int ember_split_set_strain(ember_split split, int n_coeffs, const double* coeffs, void* stream);
/* n_steps split steps, asynchronous on `stream`. */
int ember_split_step(ember_split split, int n_steps, int use_graph, void* stream);
int ember_split_get_state(ember_split split, double* state, double* t, int mem, void* stream);
/* ddtDiff and ddtProd of the last step, point-major. */
int ember_split_get_derivatives(ember_split split, double* ddt_diff, double* ddt_prod, int mem, void* stream);
/* ddtConv of the last step, point-major (convection stage attached): with
 * ember_split_get_derivatives, the three derivatives FlameSolver carries
 * through a regrid (src/flameSolver.cpp:300-340). */
int ember_split_get_convection_derivative(ember_split split, double* ddt_conv, int mem, void* stream);
/* The mass flux V of every point at the UTW system's last right-hand side
 * evaluation (convectionSystem.utwSystem.V; meaningful after a step),
 * point-major: what FlameSolver interpolates onto a new grid for rVzero and
 * the next continuity update (src/flameSolver.cpp:287-290, 336-338). */
int ember_split_get_velocity(ember_split split, double* V, int mem, void* stream);
/* Replace the time derivatives that set the next step's split constants
 * (point-major; ddt_conv only with the convection stage attached, NULL =
 * zero), as FlameSolver does after a regrid: ddtDiff, ddtProd and ddtConv
 * interpolated onto the new grid (src/flameSolver.cpp:331-336). */
int ember_split_set_derivatives(ember_split split, const double* ddt_diff, const double* ddt_prod,
                                const double* ddt_conv, int mem, void* stream);
/* Source-stage status [n_points] and stats [n_points][EMBER_STATS_WIDTH] of the last step. */
int ember_split_source_status(ember_split split, int* status, int* stats, int mem, void* stream);
/* Failed source points and diffusion systems summed over the steps since
 * ember_split_set_state (synchronises `stream`). */
int ember_split_failures(ember_split split, int64_t* source_points, int64_t* diffusion_systems, void* stream);
/* FlameSolver::calculateQdot / getHeatReleaseRate / getConsumptionSpeed
 * (src/flameSolver.cpp:926-961) of the current state: qdot [n_points]
 * (W/m^3), heat_release [n_flames] (integral of qdot dx, natural cubic
 * spline as mathUtils::integrate) and consumption_speed [n_flames]
 * (integral of qdot/cp dx / (rho_u (T[jb] - T[ju]))); any output may be
 * NULL; rho_u, ju, jb (per flame) are needed for the consumption speed. */
int ember_split_objectives(ember_split split, const double* rho_u, const int* ju, const int* jb, double* qdot,
                           double* heat_release, double* consumption_speed, int mem, void* stream);

/* One split step from the current state (which it advances, as
 * ember_split_step) and the gradient of
 *   J = sum_f w_heat_release[f] Q_f + w_consumption_speed[f] S_c,f
 * at the end of that step (either weight array may be NULL) with respect to
 * the state at its start (state_bar, point-major) and to ln(multiplier) of
 * every reaction (lnk_bar [n_reactions]). Backward pass: the objectives'
 * gradient at the end state (spline weights of mathUtils::integrate, the
 * analytic Jacobian of qdot and cp), the mass-fraction correction, the
 * transposed diffusion stages, the discrete adjoint of the source stage (BDF:
 * see ember_source_adjoint, tape_cap accepted steps per point, 0: 1024; QSS:
 * see ember_source_adjoint_qss, tape_cap step starts per point, 0: 4096,
 * needs qss_stability_check = 0), the first two diffusion stages. The
 * split constants of the step are held fixed (they come from the previous
 * step's time derivatives). Q_f and S_c,f of the step are returned in
 * heat_release / consumption_speed when given. */
int ember_split_adjoint(ember_split split, const double* w_heat_release, const double* w_consumption_speed,
                        const double* rho_u, const int* ju, const int* jb, int tape_cap, double* heat_release,
                        double* consumption_speed, double* state_bar, double* lnk_bar, int mem, void* stream);

/* ======================================================================
 * Adaptive grid of a flame (host code; needs no device)
 *
 * The regrid block of FlameSolver::finishStep (src/flameSolver.cpp:279-352)
 * with the rules of OneDimGrid (src/grid.cpp): boundary regrid (regrid /
 * regridUnstrained, src/grid.cpp:721-838: points added at a boundary that is
 * not flat to boundary_tol, removed while it is flat to boundary_tol_rm),
 * the damping values interpolated onto the new grid, then interior
 * adaptation (adapt, src/grid.cpp:77-359: insertion by the vtol / dvtol /
 * damping / grid_max / uniformity criteria, then removal with rm_tol of
 * margin). Inserted points take the natural cubic spline value of every row
 * (mathUtils::splines); boundary points repeat the boundary value.
 * After a change the caller re-creates its split handle on the new grids
 * (the step graph is captured for fixed sizes) and hands back the state
 * and time derivatives interpolated here.
 * ==================================================================== */
typedef struct {
    double vtol;                        /* Grid.vtol (0.12)                           */
    double dvtol;                       /* Grid.dvtol (0.2)                           */
    double absvtol;                     /* Grid.absvtol (1e-8)                        */
    double rm_tol;                      /* Grid.rmTol (0.6)                           */
    double uniformity_tol;              /* Grid.uniformityTol (2.5)                   */
    double grid_min, grid_max;          /* Grid.gridMin (5e-7), gridMax (2e-4) m      */
    double damp_const;                  /* Grid.dampConst (7)                         */
    double center_grid_min;             /* Grid.centerGridMin (1e-4) m                */
    double boundary_tol;                /* Grid.boundaryTol (5e-5)                    */
    double boundary_tol_rm;             /* Grid.boundaryTolRm (1e-5)                  */
    double unstrained_downstream_width; /* Grid.unstrainedDownstreamWidth (5)         */
    int add_point_count;                /* Grid.addPointCount (3)                     */
    int fixed_burned_val;               /* General.fixedBurnedVal (1)                 */
    int unburned_left;                  /* General.unburnedLeft (1)                   */
    int fixed_left_loc;                 /* General.fixedLeftLocation (0)              */
    int twin_flame, cylindrical_flame;  /* General.twinFlame, curvedFlame (0, 0)      */
    int left_bc, right_bc;              /* EMBER_BC_* of the flame's grid             */
} ember_grid_options;

typedef struct ember_grid_s* ember_grid;

/* The reference's defaults (python/ember/input.py, classes Grid and General). */
int ember_grid_options_default(ember_grid_options* opts);
/* A grid of n_points >= 3 strictly increasing coordinates x (copied).
 * Replaces: OneDimGrid with setOptions (src/grid.cpp:9-41). */
int ember_grid_create(const ember_grid_options* opts, int n_points, const double* x, ember_grid* out);
int ember_grid_destroy(ember_grid grid);
/* One regrid of the current grid. rows: n_rows rows of the current number of
 * points each (row-major; the first n_adapt drive the criteria: FlameSolver
 * passes the state rows U, T, Y_k, followed by the rows of ddtConv, ddtDiff
 * and ddtProd, which are only carried along). damp_val: the damping length
 * per point (ember_grid_damping). boundaries != 0 moves the domain ends first:
 * with strain_rate != 0 by the flatness criteria (regrid), with strain_rate
 * == 0 from qdot (regridUnstrained; qdot: per point). Returns the new number
 * of points and whether the grid changed; ember_grid_get reads the result. */
int ember_grid_regrid(ember_grid grid, int n_rows, int n_adapt, const double* rows, const double* damp_val,
                      const double* qdot, double strain_rate, int boundaries, int* n_points_out, int* updated);
/* The grid after the last regrid: x and rows (n_rows rows of the new number
 * of points; either may be NULL) and the unburned / burned boundary indices. */
int ember_grid_get(ember_grid grid, double* x, double* rows, int* ju, int* jb);
/* Damping length per point as FlameSolver computes it before a regrid
 * (src/flameSolver.cpp:292-303): sqrt(min(mu, lambda/cp, rho D_k > 0) /
 * max(|rho a|, 1e-100)); rho_d point-major [n][S]. */
int ember_grid_damping(int n_points, int n_species, const double* mu, const double* conductivity, const double* cp,
                       const double* rho_d, const double* rho, double strain_rate, double* damp_val);

#ifdef __cplusplus
}
#endif

#endif /* EMBER_GPU_H */
