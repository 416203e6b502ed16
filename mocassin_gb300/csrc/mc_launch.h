// mc_launch.h -- launchers of the transport kernels, one translation unit
// per precision (the FP64 unit is compiled with -fmad=false so its
// arithmetic matches the oracle operation for operation).
#pragma once

#include <cuda_runtime.h>

#include "mc_device.cuh"

namespace mcg {

// Plain form: one thread per packet history, FP64 atomics into the estimators.
cudaError_t launch_plain_fp32(const DevGrid &g, const DevSources &s, const DevReplay &rp,
                              DevCounters *cnt, int num_sms, cudaStream_t stream);
cudaError_t launch_plain_fp64(const DevGrid &g, const DevSources &s, const DevReplay &rp,
                              DevCounters *cnt, int num_sms, cudaStream_t stream);

// Re-layout of the emission CDF rows: [nb][nc+1] (cell fastest) ->
// [nc+1][nb] (one row per cell) with a running maximum along each row.
cudaError_t launch_cdf_transpose(const float *in, float *out, int nc1, int nb, cudaStream_t stream);

}  // namespace mcg
