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
};

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
// SourceArgs from the public options (source.cu).
SourceArgs make_source_args(const ember_source_options* o, int n, const double* state_in, const double* split,
                            const double* dt, double t_start, const double* x, double* state_out, int* status,
                            int* stats);
int source_check_options(const ember_source_options* o);
// Device bytes a launch above takes from its Scratch (for an arena sized up front).
int source_qss_scratch_bytes(const MechView& m, const SourceArgs& a, size_t* bytes);
int source_bdf_scratch_bytes(const MechView& m, const SourceArgs& a, size_t* bytes);

}  // namespace ember

// A compiled mechanism (ember_mech handle).
struct ember_mech_s {
    int S = 0, R = 0;
    void* blob = nullptr;  // one device allocation holding every table
    ember::MechView view{};
};
