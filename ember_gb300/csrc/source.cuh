// Shared declarations of the source-term kernels (QSS in source.cu, BDF in bdf.cu).
#pragma once

#include <cuda_runtime.h>

#include "../../include/ember_gpu.h"
#include "chem.cuh"
#include "qss.cuh"

namespace ember {

// Flattened arguments of one source-term launch (device pointers).
struct SourceArgs {
    int n;
    int threads;              // threads per point requested (0: the mechanism's tuned or default width)
    int bdf_layout;           // BDF matrix layout requested (0: the mechanism's tuned one or by size, else 1 + layout)
    const double* state_in;   // [n][S+2]
    const double* split;      // [n][S+2] or null
    const double* dt;         // [n]
    double t_start;
    const double* t_start_dev;  // null, or device scalar used instead of t_start (graph replays)
    const double* x;          // [n] or null
    double* state_out;        // [n][S+2]
    int* status;              // [n]
    int* stats;               // [n][4] or null
    double pressure;
    int kinetics_model;
    int max_steps;
    double qss_epsmin, qss_epsmax, qss_dtmin, qss_dtmax, qss_abstol, qss_minval;
    int qss_itermax, qss_stability_check;
    double bdf_reltol, bdf_atol_u, bdf_atol_t, bdf_atol_y, bdf_min_step;
    int bdf_max_steps;
    double ign_tstart, ign_duration, ign_energy, ign_center, ign_stddev;
    // Trajectory tape for the adjoint (null: none), per point at tape + j *
    // tape_stride. BDF: a header of kTapeHeader doubles and one record of
    // n + 4 doubles per accepted step (at most tape_cap records). QSS: a
    // header of kQssTapeHeader doubles and one record of n + 2 doubles per
    // step start (at most tape_cap).
    double* tape;
    int64_t tape_stride;
    int tape_cap;
    // QSS two-pass schedule (see launch_source_qss): suspend after step_cap
    // steps into resume[j], listing the point in susp_list; a resuming launch
    // takes its points from work_list (susp_n of them) and continues them.
    int step_cap;
    int resuming;
    QssResume* resume;
    int* susp_list;
    int* susp_n;
    int tail_steps, tail_threads;  // requested (0: the mechanism's tuned values)
    int queue_chunk;               // work-queue slots claimed per atomic (0: the mechanism's tuned value)
};

// Tape header: accepted steps recorded, order after the last step, t after
// the last step, overflow flag, integrator status, tf. Record: t after the
// step, h, q, restart flag (a q = 1 restart with z1 = h f(z0) preceded the
// step), then y after the step (n values).
constexpr int kTapeHeader = 8;
__host__ __device__ inline int64_t bdf_tape_doubles(int n, int cap) { return kTapeHeader + int64_t(cap) * (n + 4); }

// SourceSystem::getQdotIgniter (src/sourceSystem.cpp:33-45).
__device__ __forceinline__ double igniter(const SourceArgs& a, double t, double x) {
    if (a.ign_energy != 0.0 && t >= a.ign_tstart && t < a.ign_tstart + a.ign_duration) {
        const double pi = 3.14159265358979323846;
        const double dx = x - a.ign_center;
        return a.ign_energy / (a.ign_stddev * sqrt(2 * pi) * a.ign_duration) *
               em_exp(-(dx * dx) / (2 * (a.ign_stddev * a.ign_stddev)));
    }
    return 0.0;
}

// Shared memory (doubles) of one QSS point: kinetics work area and QSS vectors.
__host__ __device__ inline size_t qss_smem_doubles(const MechView& m, bool stab) {
    return ChemSmem::doubles(m.S, m.R, m.n_tb, m.n_fo, false) + QssSmem::doubles(m.S + 2, stab);
}

class Scratch;
int make_work_order(const SourceArgs& a, Scratch& sc, cudaStream_t st, int** order_out);
int launch_source_qss(const MechView& m, const SourceArgs& a, int* counter, Scratch& sc, cudaStream_t st);
int launch_source_bdf(const MechView& m, const SourceArgs& a, int* counter, Scratch& sc, cudaStream_t st);
// Discrete adjoint of a BDF launch that recorded a tape (a.tape): from the
// adjoint of the end states (ybar_out, [n][S+2]) to that of the start states
// (ybar_in) and, per point, of ln(multiplier) of every reaction (pbar,
// [n][R]); adj_status [n]: 0, the forward status, or -30 (tape overflow),
// -31 (no step), -32 (singular matrix).
int launch_source_bdf_adjoint(const MechView& m, const SourceArgs& a, int* counter, const double* ybar_out,
                              double* ybar_in, double* pbar, int* adj_status, Scratch& sc, cudaStream_t st);
// Gradient at point-major states of psi = gq qdot + gcp cp + gT T per point
// (qdot, cp of the normalised state): ybar [n_pts][S+2], pbar [n_pts][R]
// (d psi / d ln multiplier). `a` supplies pressure and kinetics model.
int launch_objective_vjp(const MechView& m, const SourceArgs& a, int n_pts, const double* state, const double* gq,
                         const double* gcp, const double* gT, double* ybar, double* pbar, Scratch& sc,
                         cudaStream_t st);
// Forward BDF with a tape (tape_cap accepted steps per point) followed by its
// adjoint; lnk_bar: gradient summed over points ([R], or null);
// lnk_bar_points: per point ([n][R], or null: scratch).
int source_bdf_adjoint_run(const MechView& m, SourceArgs a, int tape_cap, const double* ybar_out, double* ybar_in,
                           double* lnk_bar, double* lnk_bar_points, int* adj_status, Scratch& sc, cudaStream_t st);
// Discrete adjoint of a QSS launch (qss_adjoint.cu): the forward integration
// of every point again (state_out, status as the forward kernel's) with a
// per-CTA tape of at most tape_cap step starts, then the backward pass: ybar_in
// [n][S+2] and, per point, pbar [n][R]; adj_status [n]: 0, the forward status,
// -30 (tape full), -33 (more than 32 attempts in a step).
// With a.tape (a QSS tape of the same points, written by launch_source_qss),
// the step starts come from it for every point whose tape did not overflow;
// fwd_status is then the forward launch's status.
int launch_source_qss_adjoint(const MechView& m, const SourceArgs& a, int tape_cap, int* counter,
                              const int* fwd_status, const double* ybar_out, double* ybar_in, double* pbar,
                              int* adj_status, Scratch& sc, cudaStream_t st);
// Doubles of a QSS tape of n_points with tape_cap step starts each, and the
// largest tape the adjoint paths allocate (beyond it they integrate again).
size_t qss_tape_doubles(const MechView& m, int n_points, int tape_cap);
constexpr size_t kQssTapeBudgetBytes = size_t(2) << 30;
int source_qss_adjoint_run(const MechView& m, const SourceArgs& a, int tape_cap, const double* ybar_out,
                           double* ybar_in, double* lnk_bar, double* lnk_bar_points, int* adj_status, Scratch& sc,
                           cudaStream_t st);
// SourceArgs from the public options (source.cu).
SourceArgs make_source_args(const ember_source_options* o, int n, const double* state_in, const double* split,
                            const double* dt, double t_start, const double* x, double* state_out, int* status,
                            int* stats);
int source_check_options(const ember_source_options* o);
// Rates and thermo of n states into caller buffers (no allocation; capturable).
size_t gas_eval_cache_doubles(const MechView& v, int n);
int launch_gas_eval(const MechView& v, int n, double pressure, int model, int mode, const double* T, const double* Y,
                    double* kcache, double* net, double* hk, double* cp_mass, cudaStream_t st);
// Device bytes a launch above takes from its Scratch (for an arena sized up front).
int source_qss_scratch_bytes(const MechView& m, const SourceArgs& a, size_t* bytes);
// Threads per point of the QSS kernel for these arguments (see threads_per_point).
int source_qss_threads(const MechView& m, const SourceArgs& a);
// Two-pass schedule of the QSS kernel for these arguments (steps 0: one pass).
void source_qss_tail(const MechView& m, const SourceArgs& a, int* steps, int* threads);
int source_bdf_scratch_bytes(const MechView& m, const SourceArgs& a, size_t* bytes);
// Threads per point and matrix layout (1 + BDF_* of bdf.cu) of the BDF kernel for these arguments.
int source_bdf_threads(const MechView& m, const SourceArgs& a);
int source_bdf_layout(const MechView& m, const SourceArgs& a);
// Whether matrix layout 1 + mode fits the BDF kernel's shared memory for this mechanism.
bool source_bdf_layout_fits(const MechView& m, int layout);
// Launch widths of the BDF kernel.
constexpr int kBdfThreadChoices[] = {32, 64, 128, 160, 256};

}  // namespace ember

// A compiled mechanism (ember_mech handle).
struct ember_mech_s {
    int S = 0, R = 0;
    void* blob = nullptr;  // one device allocation holding every table
    ember::MechView view{};
};
