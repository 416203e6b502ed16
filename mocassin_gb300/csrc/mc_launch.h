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
// resonance-line packets into the absorbed list after round 0
cudaError_t launch_wave_res_inject_fp32(const WaveLaunch &L, const uint32_t *cells, const long long *prefix,
                                        int ncell);
cudaError_t launch_wave_res_inject_fp64(const WaveLaunch &L, const uint32_t *cells, const long long *prefix,
                                        int ncell);
cudaError_t launch_wave_emit_fp32(const WaveLaunch &L, int round);
cudaError_t launch_wave_emit_fp64(const WaveLaunch &L, int round);
cudaError_t launch_wave_march_fp32(const WaveLaunch &L);
cudaError_t launch_wave_march_fp64(const WaveLaunch &L);
// batched march over many models' rounds: the resident grid size first (it
// sets the tasks per pass), then the launch
cudaError_t launch_wave_march_batch_blocks_fp32(bool dust, size_t smem, int num_sms, int *blocks);
cudaError_t launch_wave_march_batch_blocks_fp64(bool dust, size_t smem, int num_sms, int *blocks);
cudaError_t launch_wave_march_batch_fp32(const BatchLaunch &B);
cudaError_t launch_wave_march_batch_fp64(const BatchLaunch &B);
size_t march_batch_smem_fp32(int nx, int ny, int nz);
size_t march_batch_smem_fp64(int nx, int ny, int nz);

// Scan of the per-bin counts and scatter of the round's n entries into the
// frequency-sorted queue; fold of march-indexed estimators into rows;
// expansion of a cell-fastest array into march order (non-identity grids).
cudaError_t launch_wave_sort(const WaveLaunch &L, unsigned int n);
cudaError_t launch_wave_fold(const double *src, double *dst, const int32_t *lin2cell, long long ncell3, int nc1,
                             int nb, cudaStream_t stream);
cudaError_t launch_wave_expand(const float *src, float *dst, const int32_t *lin2cell, long long ncell3, int nc1,
                               int nb, cudaStream_t stream);

// Raises a kernel's dynamic shared-memory limit to at least `bytes` and never
// lowers it: several host threads (one context and stream per model) launch
// the same kernels with their own sizes, and a limit one thread sets must not
// fall below what another thread's launch needs.
cudaError_t raise_smem_limit(const void *func, size_t bytes);

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
  unsigned long long hit, converged, no_te, no_ion, iters, small, dmax_bits, fallback;
};
// The grains of the photoelectric and gas-grain collision terms of the cell
// update (grains.cuh); nsizes = 0: a gas-only update.
struct GrainArgs {
  int nsizes, nb;
  int ivn;                              // first bin above grainVn (0-based)
  double vn, msurf, abundance;          // grainVn [Ryd], MsurfAtom, grainAbun
  const float *nu;                      // [nb] Ryd
  const float *xs;                      // [nsizes][nb] Cabs per grain [cm^2]
  const double *radius_um, *weight;     // [nsizes] grainRadius [um], grainWeight
  const double *ion_nu;                 // [33] threshold of each balance ion [Ryd]
  const double *yn_d, *dnu_d, *qa_d;    // [nb] yield Yn, nu - Vn; [nsizes][nb] Cabs / (1e-8 a^2)
  const float *yn_f, *dnu_f, *qa_f;     // the same in FP32
  const float *idnu_f;                  // [nb] 1 / (nu - Vn) (the FP32 form)
  const double *inv_hnu;                // [nb] 1 / (hcRyd nu) (the FP32 form's photon flux)
  const double *jste;                   // Jste [nb][nc+1] (not normalised)
  double jscale;                        // its normalisation
  const float *ndust;                   // [nc+1] grains per cm^3
  const float *tdust;                   // [nsizes+1][nc+1] grain temperatures (rows 1..), null: 0 K
  double *out;                          // [3][nsizes][nc+1] potential, photoelHeat_d, gasDustColl_d
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
  // warm start: the state before the prediction (null: cold).  At the first
  // T step a prediction whose thermal residual is below accept_res (<= the
  // reference's 1 %) of the heating is accepted; below near_res it is
  // bracketed with small steps; otherwise the cell restarts the cold solve
  // from this state (the plain solve as fallback).
  const double *te_prev, *ne_prev, *x_prev;  // x_prev [nc+1][7][8]
  double accept_res, near_res;
  // the emission's forbidden-line totals, from the populations of each
  // cell's last T step (null: not kept): forb_out [ncel][nc+1], and per cell
  // forb_ok = 1 when they belong to the state the update left
  float *forb_out;
  int *forb_ok;
  double step0;                      // first unbracketed Te step factor (1.2: iterateT's)
  int step_grow;                     // warm start: (factor - 1) doubles per unbracketed step, up to 0.2
  GrainArgs g;                       // grains (g.nsizes = 0: none)
};
cudaError_t launch_cell_update(const UpdArgs &a, int fp32, void *scratch, int num_sms, cudaStream_t stream);
cudaError_t launch_cell_update_fp32(const UpdArgs &a, void *scratch, int num_sms, cudaStream_t stream);
// sets the cache preference of the FP32 form's kernels (before a capture)
cudaError_t cell_update_fp32_prepare(const UpdArgs &a);
size_t cell_update_fp32_scratch(int nc, int ncel, int nsizes, int nb);
cudaError_t launch_update_stats(int nc, const int *conv, const int *niter, const int *flags, const double *dte,
                                UpdStatsDev *s, int num_sms, cudaStream_t stream);
cudaError_t launch_species(int nc, int nsp, const int *sp_e, const int *sp_s, const double *X, const double *ab,
                           const double *hden, float *den, int num_sms, cudaStream_t stream);
// den[k][cell] = weight(k) Ndust(cell) where the grain temperature of size k
// is below t_sub (tdust [nsizes+1][nc1], rows 1..; null: every size), else 0
cudaError_t launch_grain_density(int nc1, int nsizes, const float *weight, const float *ndust, const float *tdust,
                                 float t_sub, float *den, int num_sms, cudaStream_t stream);
void spline_natural(const double *x, const double *y, int n, double *y2);

// ---- the learned warm start (mlp.cu) ----
constexpr int kMlpIn = 80, kMlpHid = 256, kMlpOut = 48, kMlpTargets = 41;
constexpr int kMlpW1 = 0, kMlpB1 = kMlpW1 + kMlpHid * kMlpIn, kMlpW2 = kMlpB1 + kMlpHid,
              kMlpB2 = kMlpW2 + kMlpHid * kMlpHid, kMlpW3 = kMlpB2 + kMlpHid, kMlpB3 = kMlpW3 + kMlpHid * kMlpHid,
              kMlpW4 = kMlpB3 + kMlpHid, kMlpB4 = kMlpW4 + kMlpOut * kMlpHid, kMlpParams = kMlpB4 + kMlpOut;
cudaError_t launch_mlp_gemm(int M, int N, int K, const float *a, int lda, const float *mask, bool round_a,
                            const float *w, bool wt, const float *bias, int act, float *c, int ldc, cudaStream_t s);
// dW += dZ^T bf16(X) and db += column sums of dZ over M rows: per-split
// partial sums in `scratch` (mlp_wgrad_scratch_floats of them), added in a
// fixed order, so that training is reproducible
size_t mlp_wgrad_scratch_floats(int M, int N, int K, int num_sms);
cudaError_t launch_mlp_wgrad(int M, int N, int K, const float *dz, const float *mask, const float *x, float *dW,
                             float *db, float *scratch, size_t scratch_floats, int num_sms, cudaStream_t s);
// the forward layers on the tensor cores (tcgen05, BF16 operands, FP32
// accumulators in TMEM), and the error flag of their bounded mbarrier waits
// (1 when one gave up; reading it clears it)
cudaError_t launch_mlp_forward_tc(int M, int N, int K, const float *a, int lda, const float *w, const float *bias,
                                  int act, float *c, int ldc, int num_sms, cudaStream_t s);
int mlp_tc_take_error();
cudaError_t launch_mlp_loss(int M, int nt, int ld, const float *y, const float *tn, float *dy, double *loss,
                            cudaStream_t s);
cudaError_t launch_mlp_adam(int n, float *w, const float *g, float *m1, float *m2, const int *dstep, int step0,
                            int steps, float lr, cudaStream_t s);
cudaError_t launch_mlp_step(int *dstep, cudaStream_t s);
cudaError_t launch_mlp_gather(int B, long long n, uint32_t seed, const int *dstep, const float *xs, const float *ts,
                              const float *fmean, const float *fstd, const float *tmean, const float *tstd, float *xb,
                              float *tb, cudaStream_t s);
cudaError_t mlp_prepare();
// per-column sums and sums of squares of n rows: kMlpStatBlocks partial
// sums per column (sum[b * cols + col]), for the host to add in order
constexpr int kMlpStatBlocks = 64;
cudaError_t launch_mlp_stats(long long n, int cols, const float *a, double *sum, double *sq, cudaStream_t s);
// appends the rows of the balanced hit cells in cell order; blk_counts holds
// mlp_collect_blocks(num_sms) counts
int mlp_collect_blocks(int num_sms);
cudaError_t launch_mlp_collect(int nc, const float *mom, long long ms, const double *hden, const double *te,
                               const double *X, const int *flags, long long cap, unsigned long long *count, float *xs,
                               float *ts, unsigned int *blk_counts, int num_sms, cudaStream_t s);
cudaError_t launch_mlp_infer_features(int nc, const float *mom, long long ms, const double *hden, const float *fmean,
                                      const float *fstd, float *x, int num_sms, cudaStream_t s);
cudaError_t launch_mlp_apply(int nc, const float *mom, const float *y, const float *tmean, const float *tstd, double *te,
                             double *ne, double *X, double *te_prev, double *ne_prev, double *x_prev, int num_sms,
                             cudaStream_t s);

cudaError_t launch_dust_temperature(int nc1, int nsizes, int nt, const float *A, const float *E, const float *gw,
                                    const float *hit, float *tdust, const double *gcd, const double *gpd, int num_sms,
                                    cudaStream_t stream);

cudaError_t launch_wave_round_control(const WaveLaunch &L, cudaGraphConditionalHandle h);

// Diffuse-emission CDF (emission.cu): the tables derived from the frequency
// grid on the host and the resident cell state they are applied to.
constexpr int kEmiMaxBins = 4096, kEmiMaxLim = 32, kEmiMaxHeavy = 32;
struct EmiArgs {
  int nc, nb;
  const double *te, *ne, *X;      // resident cell state [nc+1], [nc+1][7][8]
  const float *forb;              // [ncel][nc+1] forbidden-line totals
  int ncel;
  const float *ab;                // [7] abundances (H He C N O Ne S)
  const float *nu, *lnu, *wid;    // [nb]: frequency [Ryd], log10, cRyd widFlx / 1e15
  const float *xs_h, *xs_hei, *xs_heii;        // [nb] ground-state cross-sections (Milne relation)
  const float *tp_hi, *tp_hei, *tp_heii;       // [nb] two-photon spectral shapes
  const int *pair;                // [3][nb] gamma edge pair covering each bin (-1: none)
  int nlim[3];
  const float *lg[3];             // [ntk][nlim] log10 gamma (HI, HeI, HeII)
  const int *edge[3];             // [nlim] 0-based bins of the gamma edges
  int ntk;
  const float *tk;                // [ntk]
  int p_from[3], p_milne[3];      // first bin of each Milne range; bin of each threshold
  const float *gaunt_d;           // [8][11] Hummer's Chebyshev coefficients
  int nheavy;
  const int *h_e, *h_stage, *h_ip, *h_hi;      // element index, recombining stage, [ip, hi) bins
  const float *h_g, *h_nuip, *xs_outer;        // g0/g1, nu at ip, [nheavy][nb] outer-shell cross-section
  int j2, ly_bin[4];
  float ly_data[4];
  float hi_rec_sum, heii_rec_sum;
  const float *hei_rec;           // [34][3][4] HeI line fits (first coefficient x 1e25)
  float milne_c;                  // 4 pi h c Ryd (h^2 / 2 pi m k)^1.5 Ryd^2 1e40
  // grains (nsizes 0: none); tdust [nsizes+1][nc+1] (row 0 the mixture), null before the first
  int nsizes, gas;
  const float *xs_abs, *gw, *widflx, *ndust, *tdust;   // [nsizes][nb], [nsizes], [nb], [nc+1]
  const double *hden;
  float t_sub;
  float *rec_cdf, *total_lines;   // out: [nc+1][nb] rows, [nc+1]
  float *dust_cdf;                // out on a dust-only grid: [nc+1][nb]
};
constexpr int kEmiMaxSizes = 16;
// forb / ok: the line totals and their per-cell validity (the cells with ok 0
// are recomputed, through list [nc+1] and count, then marked valid)
cudaError_t launch_emission(const UpdArgs &a, const EmiArgs &E, float *forb, int *ok, int *list, int *count,
                            int num_sms, cudaStream_t s);

// Sets the text returned by mc_last_error() on the calling thread.
void set_last_error_text(const char *msg);

// Re-layout of the emission CDF rows: [nb][nc+1] (cell fastest) ->
// [nc+1][nb] (one row per cell) with a running maximum along each row.
cudaError_t launch_cdf_transpose(const float *in, float *out, int nc1, int nb, cudaStream_t stream);

}  // namespace mcg
