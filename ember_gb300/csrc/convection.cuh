// Convection stage (ConvectionSystemSplit::integrateToTime) for a batch of
// flames: the launch plan shared by ember_convection_integrate and the split
// step. The kernels are in convection.cu.
#pragma once

#include <cstdint>
#include <vector>

#include "common.cuh"

namespace ember {

struct ConvFlame {
    ember_convection_flame f;
    int64_t p0;      // first point of the flame in the concatenated point arrays
    int64_t v0;      // first value of the flame in the variable-major state arrays
    int64_t utw_wk;  // UTW work slice: the integrator's vectors (3N each), then y and per-point scratch
    int64_t hist;    // first recorded time of the flame (max_history per flame)
    int64_t histv;   // first recorded value of the flame (max_history * N per flame)
};

struct ConvArgs {
    int n_flames, S;
    const ConvFlame* flames;
    const double* W;
    const double* x;
    const double* y_left;
    const double* drhodt;
    const double* split;
    double* state;
    double* wk_utw;
    double* wk_spec;     // kWorkVectors * N per (flame, species) system, at spec_off
    const int64_t* spec_off;
    double* hist_t;
    double* hist_v;
    int* n_hist;
    int* status;         // n_flames * (1 + S)
    int* stats;          // n_flames * 4 or null
    double t0, tf, reltol, abstol_u, abstol_t, abstol_y, min_step;
    int max_steps, max_history;
    // allocated sizes (doubles), for the kernels' own checks of their slices
    int64_t wk_utw_n, wk_spec_n, hist_n, histv_n, dyn_n;
    // stage times from a device clock (the split step): t0 = t (f0 == 0) or
    // t + f0 * dt, tf = t + f1 * dt with t = *t_dev; else t0, tf above
    const double* t_dev;
    double f0, f1, dt;
};

struct ConvPlan {
    ConvArgs a{};
    int n_flames = 0, S = 0, max_points = 0;
    int64_t P = 0, V = 0, WU = 0, WS = 0, HS = 0, HV = 0;
    std::vector<ConvFlame> hf;
    std::vector<int64_t> spec_off;
};

// Check the flames and options and lay out every per-flame slice (host only).
int conv_plan_layout(ConvPlan& p, int n_flames, const ember_convection_flame* flames, int S,
                     const ember_convection_options* opts);
// Carve the plan's device buffers (work, record, status, tables) from `sc`,
// upload the tables on `st` and allow the UTW kernel its shared memory.
int conv_plan_alloc(ConvPlan& p, Scratch& sc, bool with_stats, cudaStream_t st);
// Bytes conv_plan_alloc carves, for an arena sized in advance.
size_t conv_plan_bytes(const ConvPlan& p, bool with_stats);
// The three kernels on `st` with arguments `a` (the plan's, inputs and
// times set by the caller).
int conv_launch(const ConvPlan& p, const ConvArgs& a, cudaStream_t st);
// The continuity point of every flame at the start of a split step (after
// the first since *ready was cleared; then sets *ready): state point-major
// with n_vars per point; qdot per point or null (needed for fixedQdot).
// V of the UTW systems' last right-hand side evaluation, point-major across flames.
int conv_velocity_launch(const ConvPlan& p, const ConvArgs& a, double* out, cudaStream_t st);
int conv_continuity_launch(const ConvPlan& p, const ConvArgs& a, const int* ready, const double* state, int n_vars,
                           const double* qdot, cudaStream_t st);

}  // namespace ember
