// Arguments shared by the FP64 and mixed-precision flow-map launchers.
#pragma once

#include "nbcs_internal.cuh"

namespace nbcs {

struct FlowmapArgs {
    Params P;
    double ts, te;  // solver-time span params[0] * [t0, t0 + T]
    const double* x;
    const double* y;
    int nx, ny;
    const uint8_t* mask;
    double* out;
    int32_t* status;
    int32_t* stats;
    double rtol, atol;
    int nmax;
    int threads, blocks_per_sm, lanes;
    const void* step_model;
    cudaStream_t stream;
};

int launch_flowmap64(const nbcs_flow* flow, const FlowmapArgs& a);
int launch_flowmap32(const nbcs_flow* flow, const FlowmapArgs& a);
int launch_flowmap32_learned(const nbcs_flow* flow, const FlowmapArgs& a, int mode);
int launch_rhs32(const nbcs_flow* flow, const Params& P, const double* ty, long n, double* dy,
                 cudaStream_t stream);

}  // namespace nbcs
