// Variable-order BDF source-term integrator (CVODE replacement).
#include "common.cuh"
#include "source.cuh"

namespace ember {

int launch_source_bdf(const MechView& m, const SourceArgs& a, int* counter, Scratch& sc, cudaStream_t st) {
    (void)m; (void)a; (void)counter; (void)sc; (void)st;
    set_error("the BDF source-term integrator is not available in this build");
    return EMBER_EINVAL;
}

}  // namespace ember
