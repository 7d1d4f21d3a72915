// Shared declarations of the transport-property kernel (transport.cu), used
// by the split step (split.cu) to refresh B and D on the device.
#pragma once

#include <cstdint>

#include "../../include/ember_gpu.h"
#include "chem.cuh"

namespace ember {

constexpr double kMoleFractionFloor = 1e-20;  // Cantera's Tiny in MixTransport::update_C

struct TransportView {
    int S;
    const double* visc;  // [S][5]
    const double* cond;  // [S][5]
    const double* diff;  // [P][5], P = S(S+1)/2
    const double* w4;    // [P] (W_lo / W_hi)^(1/4)
    const double* s8w1;  // [P] sqrt(8) * sqrt(1 + W_hi / W_lo)
};

__host__ __device__ inline int64_t pair_index(int S, int lo, int hi) {
    return int64_t(lo) * S - int64_t(lo) * (lo - 1) / 2 + (hi - lo);
}

// Properties of n states: T at T[j * tstride], Y_k at Y[j * ystride + k];
// outputs point-major with S values per point (see ember_properties).
int launch_transport(const MechView& m, const TransportView& tv, int n, double p, double thr, const double* T,
                     int64_t tstride, const double* Y, int64_t ystride, const ember_properties& out, cudaStream_t st);

}  // namespace ember

struct ember_transport_s {
    ember_mech mech = nullptr;
    void* blob = nullptr;
    ember::TransportView view{};
};
