// mc_launch.h -- launchers of the transport kernels, one translation unit
// per precision (the FP64 unit is compiled with -fmad=false so its
// arithmetic matches the oracle operation for operation).
#pragma once

#include <cuda_runtime.h>

#include "mc_device.cuh"
#include "wave_types.cuh"

namespace mcg {

// Plain form: one thread per packet history, FP64 atomics into the estimators.
cudaError_t launch_plain_fp32(const DevGrid &g, const DevSources &s, const DevReplay &rp,
                              DevCounters *cnt, int num_sms, cudaStream_t stream);
cudaError_t launch_plain_fp64(const DevGrid &g, const DevSources &s, const DevReplay &rp,
                              DevCounters *cnt, int num_sms, cudaStream_t stream);

// Chosen form (wavefront rounds), per precision: the frequency sampling of
// round 0 (stellar) and of later rounds (re-emission), the emission of the
// sorted queue, and the persistent march.
cudaError_t launch_wave_sample_stellar_fp32(const WaveLaunch &L);
cudaError_t launch_wave_sample_stellar_fp64(const WaveLaunch &L);
cudaError_t launch_wave_sample_reemit_fp32(const WaveLaunch &L, unsigned int n_abs);
cudaError_t launch_wave_sample_reemit_fp64(const WaveLaunch &L, unsigned int n_abs);
cudaError_t launch_wave_emit_fp32(const WaveLaunch &L, int round);
cudaError_t launch_wave_emit_fp64(const WaveLaunch &L, int round);
cudaError_t launch_wave_march_fp32(const WaveLaunch &L);
cudaError_t launch_wave_march_fp64(const WaveLaunch &L);

// Scan of the per-bin counts and scatter of the round's n entries into the
// frequency-sorted queue; fold of march-indexed estimators into rows;
// expansion of a cell-fastest array into march order (non-identity grids).
cudaError_t launch_wave_sort(const WaveLaunch &L, unsigned int n);
cudaError_t launch_wave_fold(const double *src, double *dst, const int32_t *lin2cell, long long ncell3, int nc1,
                             int nb, cudaStream_t stream);
cudaError_t launch_wave_expand(const float *src, float *dst, const int32_t *lin2cell, long long ncell3, int nc1,
                               int nb, cudaStream_t stream);

// Opacity contraction: method 0 = FP32 CUDA cores, 1 = tcgen05 split BF16.
cudaError_t launch_opacity(int method, int nc1, int nspecies, int nb, const float *den, const float *xs,
                           const float *ff, float *out, int *error, int num_sms, cudaStream_t stream);

// Jste moments: out[o][cell] = scale * sum_nu J[nu][cell] W[nu][o] (tcgen05).
cudaError_t launch_jmoments(int nc1, int nb, int nout, const double *J, const float *W, double scale, float *out,
                            int *error, int num_sms, cudaStream_t stream);

// Sets the text returned by mc_last_error() on the calling thread.
void set_last_error_text(const char *msg);

// Re-layout of the emission CDF rows: [nb][nc+1] (cell fastest) ->
// [nc+1][nb] (one row per cell) with a running maximum along each row.
cudaError_t launch_cdf_transpose(const float *in, float *out, int nc1, int nb, cudaStream_t stream);

}  // namespace mcg
