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

// ---- the cell update (cellupdate.cu) ----
template <typename Real> struct UpdIonT {  // one of the 33 balance ions
  int z, ion, e, nelec;
  int dr[4], ndr, ar;    // matching dielectronic.dat rows (file order), last aldrovandi.dat row (-1: none)
  int dr8[4], ndr8, ar8; // the same for oxygen at this stage (the fallback of calcAlpha)
  Real chex[4];          // charge exchange with H: chex(:, 1) already x 1e-9
  Real dek, g0g1;        // deltaE/k of the reverse rate and g0/g1 (N0, O0)
};
template <typename Real> struct UpdCelT {  // one ion with forbidden-line data
  int z, ion, e, nlev, nt;
  Real br, zz, ar[4], ad[5];
};
using UpdIonDev = UpdIonT<double>;
using UpdCelDev = UpdCelT<double>;
// the atomic tables at one arithmetic type (the FP32 kernel reads float
// copies: a double-to-float conversion runs at the FP64 rate)
template <typename Real> struct UpdTabs {
  const UpdIonT<Real> *bal;
  const UpdCelT<Real> *cel;
  const Real *rrec, *rnew, *direc, *aldro;
  const Real *logt, *g, *e, *A, *qq, *q2;  // [ncel][32], [ncel][18] x2, [ncel][18][18], [ncel][18][18][32] x2
  const Real *ab;
};
struct UpdStatsDev {
  unsigned long long hit, converged, no_te, no_ion, iters, small, dmax_bits;
};
struct UpdArgs {
  int nc, ncel, ndirec, naldro;
  int bal_z[7], bal_first[7];
  UpdTabs<double> d;
  UpdTabs<float> f;
  const double *hden;
  const float *mom;                          // [67][nc+1]
  long long mstride;
  double *te, *ne, *X;                       // X [nc+1][7][8]
  int *conv, *niter, *flags;
  double *dte;
  double xhi;
  int mat_rows, mat_stride;  // FP32 form: matrix row length (max levels) and odd per-lane stride
};
cudaError_t launch_cell_update(const UpdArgs &a, int fp32, int num_sms, cudaStream_t stream);
cudaError_t launch_cell_update_fp32(const UpdArgs &a, int blocks, cudaStream_t stream);
cudaError_t launch_update_stats(int nc, const int *conv, const int *niter, const int *flags, const double *dte,
                                UpdStatsDev *s, int num_sms, cudaStream_t stream);
cudaError_t launch_species(int nc, int nsp, const int *sp_e, const int *sp_s, const double *X, const double *ab,
                           const double *hden, float *den, int num_sms, cudaStream_t stream);
void spline_natural(const double *x, const double *y, int n, double *y2);

// Sets the text returned by mc_last_error() on the calling thread.
void set_last_error_text(const char *msg);

// Re-layout of the emission CDF rows: [nb][nc+1] (cell fastest) ->
// [nc+1][nb] (one row per cell) with a running maximum along each row.
cudaError_t launch_cdf_transpose(const float *in, float *out, int nc1, int nb, cudaStream_t stream);

}  // namespace mcg
