/*
 * mocassin_gpu.h -- C-ABI of the GB300 energy-packet transport library
 * (libmcgpu.so).
 *
 * The library replaces mocassin's Monte Carlo packet loop:
 *   subroutine energyPacketDriver(iStar, n, grid, gpLoc, cellLoc)
 *     source/photon_mod.f90:26-285  (driver loop, re-emission loop :120-125)
 *     source/photon_mod.f90:289-487 (energyPacketRun)
 *     source/photon_mod.f90:768-1059 (newPhotonPacket), :491-684 (initPhotonPacket)
 *     source/photon_mod.f90:720-764 (getNu2), :1061-2872 (pathSegment), :2875-3101 (hg)
 *     source/vector_mod.f90:303-314 (randomUnitVector)
 * called from iterateMC at source/iteration_mod.f90:488-493.
 *
 * Conventions
 *  - Every array crossing this boundary is a plain pointer plus sizes.  Host
 *    arrays keep the layout the Fortran side already has (column-major):
 *      active(nx,ny,nz)          int32, x fastest       (common_mod.f90:258)
 *      opacity(0:Nc,1:Nnu)       float, cell fastest    (common_mod.f90:290)
 *      scaOpac, recPDF, dustPDF  same shape as opacity  (common_mod.f90:264,293,268)
 *      totalLines(0:Nc)          float                  (common_mod.f90:295)
 *      Jste/Jdif(0:Nc,1:Nnu)     double accumulators, cell fastest
 *      escapedPackets(0:Nc,0:Nnu,0:nAngle) double, cell fastest
 *    Grid indices (x,y,z cell indices, nuP) are 1-based as in the Fortran.
 *  - Outputs are caller-allocated and are ACCUMULATED into (the caller zeroes
 *    them once per iteration, as iteration_mod.f90:458-472 does).  The values
 *    are the raw sums of dl*deltaE/dV of photon_mod.f90:1563-1574/1822-1833;
 *    the caller still applies the x1e-9 and /8 of iteration_mod.f90:705-724.
 *  - Every entry point returns an mc_status (0 = MC_OK).  The reference's
 *    fatal "print*; stop" insanity checks become error codes; the text of the
 *    last error of the calling thread is returned by mc_last_error().
 *  - The Fortran driver calls from one host thread (the reference is one
 *    thread per MPI rank).  Several host threads may drive the library at
 *    once, each on its own context (mc_ctx_t; the batch server does so):
 *    calls are not re-entrant on one context, and the drop-in calls
 *    (mc_transport_run / _f32) share one cached context and serialise on it.
 */
#ifndef MOCASSIN_GPU_H
#define MOCASSIN_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MC_ABI_VERSION 2

/* ---- status codes ------------------------------------------------------ */
typedef enum mc_status {
  MC_OK = 0,
  MC_ERR_ARG = 1,          /* bad pointer / size / flag combination          */
  MC_ERR_CUDA = 2,         /* a CUDA runtime call failed                        */
  MC_ERR_BOUNDS = 3,       /* a packet left the index range (pathSegment :1198) */
  MC_ERR_NAN = 4,          /* NaN position/direction/opacity (photon_mod :1143) */
  MC_ERR_REPLAY = 5,       /* replay draw stream exhausted                      */
  MC_ERR_TIMEOUT = 6,      /* device watchdog budget ran out                    */
  MC_ERR_UNSUPPORTED = 7,  /* option outside the built path (sub-grids, 1D ...) */
  MC_ERR_NOMEM = 8,        /* device allocation failed                          */
  MC_ERR_NO_DEVICE = 9     /* no CUDA device visible                            */
} mc_status;

/* ---- grid flags (the common_mod logicals that steer the transport) ----- */
#define MC_FLAG_SYMMETRIC_XYZ (1u << 0) /* lgSymmetricXYZ                     */
#define MC_FLAG_GAS           (1u << 1) /* lgGas                              */
#define MC_FLAG_DUST          (1u << 2) /* lgDust                             */
#define MC_FLAG_ISOTROPIC     (1u << 3) /* lgIsotropic (dust scattering)      */
#define MC_FLAG_DEBUG         (1u << 4) /* lgDebug: diffuse packets go to Jdif */
#define MC_FLAG_MULTISTARS    (1u << 5) /* lgMultistars: no octant folding    */

/* Precision of the march (mc_run_opts_t.precision). */
#define MC_PREC_FP32 0  /* FP32 march, cell-local coordinates, FP64 sums      */
#define MC_PREC_FP64 1  /* FP64 march, reference order of operations (replay) */

/* Random-draw source (mc_run_opts_t.rng). */
#define MC_RNG_PHILOX 0 /* Philox4x32-10 keyed by (seed, iteration, star)    */
#define MC_RNG_REPLAY 1 /* draws read from a caller buffer, one row per packet */

/* Run flags (mc_run_opts_t.run_flags). */
#define MC_RUN_ZERO_FIRST 1 /* zero the device estimators inside the call, before
                               the transport (iteration_mod.f90:458-472); in
                               mc_transport_run: the caller's arrays hold zeros,
                               so they are not uploaded (the result overwrites
                               them)                                          */
#define MC_RUN_FORM_PLAIN 2 /* one thread per packet history (the plain form)
                               instead of the frequency-sorted persistent march */
#define MC_RUN_GRAPH 4      /* the chosen form's rounds inside one CUDA graph (a
                               WHILE node on the device's absorbed count): no
                               host round trip per round; march_ms is then 0 */
#define MC_RUN_HOST_ZEROED 8 /* mc_transport_run / _f32 only: the caller's host
                               estimators hold zeros on entry, as the Fortran
                               driver zeroes Jste and escapedPackets before each
                               iteration (iteration_mod.f90:458-472).  Implies
                               MC_RUN_ZERO_FIRST; the call then writes only the
                               entries the transport made nonzero: the Jste /
                               Jdif rows (frequency bins) that received a
                               deposit, and the escapedPackets entries that
                               received an escape (compacted on the device;
                               scattered by the device straight into pinned
                               host arrays, by the host into pageable ones).
                               Entries it does not write keep the caller's
                               zeros.                                          */

/* Read-only description of one (mother) grid for one iteration.  All
 * pointers are HOST pointers owned by the caller; they are read during the
 * call only. */
typedef struct mc_grid {
  int32_t nx, ny, nz;      /* grid%nx, grid%ny, grid%nz                       */
  int32_t ncells;          /* grid%nCells = Nc; arrays carry rows 0..Nc       */
  int32_t nbins;           /* nbins = Nnu                                     */
  int32_t n_angle;         /* nAngleBins (0..2, set_input_mod.f90:536-541)     */
  const float *x_axis;     /* [nx] cm                                         */
  const float *y_axis;     /* [ny] cm                                         */
  const float *z_axis;     /* [nz] cm                                         */
  const int32_t *active;   /* [nx*ny*nz], x fastest; 0 = inactive (row 0)     */
  const float *opacity;    /* [(Nc+1)*Nnu], cell fastest, 1/cm                */
  const float *sca_opac;   /* [(Nc+1)*Nnu] or NULL when no dust               */
  const float *rec_pdf;    /* [(Nc+1)*Nnu] cumulative, or NULL without gas    */
  const float *total_lines;/* [Nc+1] line fraction, or NULL without gas       */
  const float *dust_pdf;   /* [(Nc+1)*Nnu] cumulative, or NULL                */
  const float *nu_array;   /* [Nnu] Ryd                                       */
  const float *g_sca;      /* [Nnu] HG asymmetry, or NULL                     */
  float geo_corr[3];       /* grid%geoCorrX/Y/Z (grid_mod.f90:807-820)        */
  float r_out;             /* R_out (0 = no outer radius)                     */
  float ion_edge1;         /* ionEdge(1), Ryd                                 */
  uint32_t flags;          /* MC_FLAG_*                                       */
  /* Viewing angles of the escape SED (n_angle > 0 only; grid_mod.f90:416-468):
   * every escape adds deltaE to angle plane 0 of escaped and, when its
   * direction falls in the theta/phi bin of viewpoint i, to plane i too. */
  int32_t n_theta_bins;    /* totAngleBinsTheta, 0 = 10 (common_mod.f90:399)  */
  int32_t n_phi_bins;      /* totAngleBinsPhi, 0 = 20 (common_mod.f90:400)    */
  const float *view_theta; /* viewPointTheta(0:nAngleBins) [rad], or NULL     */
  const float *view_phi;   /* viewPointPhi(0:nAngleBins) [rad]; < 0 = no phi  */
} mc_grid_t;

/* One ionising source: one call of energyPacketDriver(iStar, n, ...). */
typedef struct mc_source {
  int32_t istar;           /* iStar (1-based), keys the random stream         */
  int32_t cell[3];         /* starIndeces(iStar,1:3), 1-based                 */
  int64_t n_packets;       /* n                                               */
  double delta_e;          /* deltaE(iStar) [1e36 erg/s]                      */
  float pos[3];            /* starPosition(iStar) [cm]                        */
  const float *spec_cdf;   /* inSpectrumProbDen(iStar,1:Nnu) (host pointer)   */
} mc_source_t;

/* Per-call options. */
typedef struct mc_run_opts {
  uint64_t seed;           /* Philox key word                                 */
  uint32_t iteration;      /* nIterateMC; second key word with the star index */
  int32_t precision;       /* MC_PREC_*                                       */
  int32_t rng;             /* MC_RNG_*                                        */
  int32_t recursion_limit; /* recursionLimit (constants_mod.f90:56), 0 = 5000 */
  int32_t safe_limit;      /* pathSegment safeLimit (:1190), 0 = 500000       */
  int32_t run_flags;       /* MC_RUN_*                                        */
  const double *replay;    /* MC_RNG_REPLAY: [n_total * replay_stride] draws in
                              [0,1), row p = packet p of the concatenated
                              sources, consumed in the reference draw order   */
  int64_t replay_stride;   /* draws per packet row                            */
} mc_run_opts_t;

/* Counters of one call (read back after the transport). */
typedef struct mc_stats {
  int64_t crossings;       /* pathSegment loop bodies ending in a full crossing
                              (:1817) or an interaction (:1517)               */
  int64_t absorptions;     /* absInt: gas/dust absorptions (:1702, :1803)     */
  int64_t scatterings;     /* scaInt: dust scatterings (:1720)                */
  int64_t escaped;         /* packets that reached escapedPackets             */
  int64_t lines;           /* re-emissions as line packets (:927)             */
  int64_t trapped;         /* histories that hit recursionLimit (:126)        */
  int64_t silent_exits;    /* wall-sitting returns without escape (:1276)     */
  int64_t safe_limit_hits; /* pathSegment safeLimit exhaustion (:2838)        */
  double qphot;            /* Qphot (:859-861)                                */
  double kernel_ms;        /* device time of the call's device work (CUDA events
                              on the library stream: zeroing when requested,
                              the transport kernel, the counter read-back)    */
  int32_t error_code;      /* first device-side error (mc_status), 0 if none  */
  int32_t error_packet;    /* packet index of that error, -1 if none          */
  double march_ms;         /* device time of the march kernel(s) alone        */
  int64_t rounds;          /* march rounds (re-emission generations) run      */
  int64_t h2d_bytes;       /* mc_transport_run / _f32: host-to-device bytes the
                              call copied (grid arrays, sources, estimators);
                              0 for the other entry points                    */
  int64_t d2h_bytes;       /* the same for device-to-host (estimators)         */
} mc_stats_t;

/* ---- library ----------------------------------------------------------- */

/* ABI version (MC_ABI_VERSION). */
int mc_abi_version(void);

/* Text of the last error raised on the calling thread ("" if none). */
const char *mc_last_error(void);

/* Replaces the whole of energyPacketDriver for nsrc sources
 * (photon_mod.f90:26-285, the star loop of iteration_mod.f90:474-496).
 * HOST pointers in, HOST accumulators out: uploads the grid, runs all packets
 * of all sources on the GPU and adds the estimators into jste / jdif /
 * escaped (their current values are copied to the device, the kernels add
 * to them, the sums are copied back).  jdif may be NULL unless
 * MC_FLAG_DEBUG; escaped may be NULL.  The device buffers are kept for the
 * next call with the same grid shape (see mc_transport_release). */
mc_status mc_transport_run(const mc_grid_t *grid, const mc_source_t *src,
                           int32_t nsrc, const mc_run_opts_t *opts,
                           double *jste, double *jdif, double *escaped,
                           mc_stats_t *stats);

/* The same with the estimators in the grid's own 4-byte arrays
 * (grid%Jste, grid%Jdif, grid%escapedPackets are `real` in common_mod.f90:
 * 276-279), so the Fortran passes them without a conversion pass: the sums
 * are still formed in FP64 on the device and rounded to FP32 once, on the
 * device, before the copy back (half the bytes of mc_transport_run). */
mc_status mc_transport_run_f32(const mc_grid_t *grid, const mc_source_t *src,
                               int32_t nsrc, const mc_run_opts_t *opts,
                               float *jste, float *jdif, float *escaped,
                               mc_stats_t *stats);

/* mc_transport_run keeps the device buffers of the last grid shape for the
 * next call (a Lambda iteration calls it with the same grid every time);
 * this frees them.  No counterpart in the reference (it allocates nothing
 * on a device). */
mc_status mc_transport_release(void);

/* ---- resident context: the grid stays in HBM across iterations --------- */
typedef struct mc_ctx mc_ctx_t;

/* Uploads a grid to the current CUDA device and re-lays it out for the
 * kernels.  Replaces nothing in the reference (the reference keeps the grid
 * in host memory); it splits mc_transport_run so a caller that iterates keeps
 * the grid on the device.  The device estimators start at zero. */
mc_status mc_ctx_create(const mc_grid_t *grid, mc_ctx_t **out);

/* Re-uploads the per-iteration arrays (opacity, sca_opac, rec_pdf,
 * total_lines, dust_pdf, g_sca) of an existing context; geometry and sizes
 * must match the grid the context was created with. */
mc_status mc_ctx_update(mc_ctx_t *ctx, const mc_grid_t *grid);

/* Zeroes the device estimators (iteration_mod.f90:458-472). */
mc_status mc_ctx_zero(mc_ctx_t *ctx);

/* Runs the packets of nsrc sources on the resident grid, accumulating into
 * the device estimators.  spec_cdf pointers of src are host pointers. */
mc_status mc_ctx_run(mc_ctx_t *ctx, const mc_source_t *src, int32_t nsrc,
                     const mc_run_opts_t *opts, mc_stats_t *stats);

/* One transport iteration of n resident models (contexts of one device,
 * all gas-only or all dusty): mc_ctx_run of each model, the models' rounds
 * in step, every round's march one persistent launch over all of them
 * (blocks take (model, share) tasks from a global counter).  srcs[i] /
 * nsrcs[i] / opts[i] are model i's arguments of mc_ctx_run; one precision
 * per batch and Philox draws only (MC_ERR_UNSUPPORTED for replay).  Each
 * model consumes the draws of its own mc_ctx_run, so its estimators and
 * counters are those of that call.  stats[i] (may be NULL) is model i's;
 * march_ms is the batched marches' total.  The reference runs one model
 * per process; the call replaces energyPacketDriver (photon_mod.f90:26-285)
 * for many models at once. */
mc_status mc_batch_run(mc_ctx_t *const *ctxs, int32_t n, const mc_source_t *const *srcs,
                       const int32_t *nsrcs, const mc_run_opts_t *opts, mc_stats_t *stats);

/* Copies the device estimators into host arrays (adds into them when
 * accumulate != 0, else overwrites).  Any pointer may be NULL. */
mc_status mc_ctx_download(mc_ctx_t *ctx, double *jste, double *jdif,
                          double *escaped, int32_t accumulate);

/* Device pointers of the estimators (Jste, Jdif, escaped), for callers that
 * consume them on the device (the cell update).  Any out pointer may be NULL. */
mc_status mc_ctx_device_estimators(mc_ctx_t *ctx, double **jste, double **jdif,
                                   double **escaped);

void mc_ctx_destroy(mc_ctx_t *ctx);

/* ---- opacity build ------------------------------------------------------
 * The per-cell opacity of addOpacity (source/ionization_mod.f90:349-484)
 * plus the dust add of iterateMC (source/iteration_mod.f90:166-227), as one
 * dense contraction over K "species" (ions with their shell-summed
 * cross-sections, and grain (species, size) bins):
 *   opacity(cell, nu) = sum_k den(k, cell) * xs(k, nu) + ff(cell) [nu = 1]
 * den: [K][Nc+1] number densities (grain rows: grainAbun * grainWeight * Ndust,
 * zero where sublimated), cell fastest; xs: [K][nbins] cm^2; ff: [Nc+1]
 * free-free opacity of bin 1 (the only bin addOpacity gives it), or NULL;
 * opacity: [nbins][Nc+1] output, cell fastest.  K <= 64. */
#define MC_OPAC_FP32 0    /* CUDA cores, FP32 fused multiply-add             */
#define MC_OPAC_BF16X3 1  /* tensor cores: split BF16 (hi*hi + hi*lo + lo*hi),
                             FP32 accumulate in tensor memory, ~1e-5 relative */

/* Host arrays in and out. */
mc_status mc_opacity_build(int32_t ncells, int32_t nspecies, int32_t nbins, const float *den,
                           const float *xs, const float *ff, int32_t method, float *opacity,
                           double *kernel_ms);

/* Builds the context's resident opacity (total, or the dust scattering
 * opacity scaOpac when sca != 0) from host den/xs/ff: only den crosses the
 * bus, not the (Nc+1) x nbins table. */
mc_status mc_ctx_build_opacity(mc_ctx_t *ctx, int32_t nspecies, const float *den, const float *xs,
                               const float *ff, int32_t method, int32_t sca, double *kernel_ms);

/* ---- moments of the estimator for the cell update -------------------------
 * out(o, cell) = scale * sum_nu Jste(nu, cell) * w(nu, o), o < nout, on
 * the context's device Jste after mc_ctx_run (nout <= 128): the photoionisation sums of
 * updateCell (source/update_mod.f90:175-269, with w = phXSec / (hcRyd nu)
 * and scale the normalisation of iteration_mod.f90:705-724; the reference
 * adds 1e-20 afterwards) and the heating sums of its thermal balance have
 * this form.  w: host [nbins][nout]; out: host [nout][Nc+1] (cell fastest).
 * Tensor cores (tcgen05, split BF16, FP32 accumulate): ~1e-5 relative. */
mc_status mc_ctx_jste_moments(mc_ctx_t *ctx, int32_t nout, const float *w, double scale, float *out,
                              double *kernel_ms);

/* Grain temperatures of getDustT (source/update_mod.f90:1836-1945) on the
 * resident Jste: per size bin k the absorbed integral sum_nu Jste w_abs(nu, k)
 * (w_abs = xSecAbs / pi, host [nbins][nsizes]; scale = the Jste normalisation)
 * located in the emission table em_table [nsizes][ntemps] (T = 1..ntemps K,
 * dust_mod.f90:150-178) as locate does, with a linear step.  tdust: host
 * [nsizes+1][Nc+1]; row 0 = sum_k grain_weight(k) Tdust(k) (Tdust(nS,0) of the
 * reference for one species); cells no packet reached get 0. */
mc_status mc_ctx_dust_temperatures(mc_ctx_t *ctx, int32_t nsizes, const float *w_abs, const float *em_table,
                                   int32_t ntemps, const float *grain_weight, double scale, float *tdust,
                                   double *kernel_ms);

/* ---- the cell update (ionisation and thermal balance) ----------------------
 * updateCell (source/update_mod.f90:15-525) for every active cell of the
 * context, in FP64 on the GPU, after a transport: one warp per cell runs the
 * reference's bracketed secant in Te (iterateT, <= 25 steps) around its
 * ionisation balance (ionBalance, <= 25 passes) and thermal balance
 * (thermBalance with the multi-level forbidden-line cooling of equilibrium,
 * emission_mod.f90:1913-2115), for H, He, C, N, O, Ne, S at nstages = 7.
 * The photoionisation and heating sums come from the resident Jste through
 * the moment kernel (weights w, see mocassin_gb300/balance.py).  The cell
 * state stays on the GPU between calls. */
typedef struct mc_update_tables {
  const double *rrec;        /* [2][31][31] radRecFit power laws (radrec.dat)  */
  const double *rnew;        /* [4][31][31] Verner & Ferland fits              */
  const double *direc;       /* [ndirec][8] dielectronic.dat rows              */
  int32_t ndirec;
  const double *aldro;       /* [naldro][6] aldrovandi.dat rows                */
  int32_t naldro;
  int32_t ncel;              /* ions with forbidden-line data                  */
  const int32_t *cel_key;    /* [ncel][2] (Z, ion stage)                       */
  const int32_t *cel_nlev;   /* levels (<= 17)                                 */
  const int32_t *cel_ntemp;  /* collision-strength temperatures (<= 32)        */
  const double *cel_logt;    /* [ncel][32] log10 T                              */
  const double *cel_qom;     /* [ncel][32][18][18] (T, lower, upper)           */
  const double *cel_a;       /* [ncel][18][18] a[upper][lower] A values [1/s]  */
  const double *cel_g;       /* [ncel][18] statistical weights                 */
  const double *cel_e;       /* [ncel][18] level energies [1/cm]               */
  const double *cel_br, *cel_z;
  const double *cel_ar;      /* [ncel][4]                                      */
  const double *cel_ad;      /* [ncel][5]                                      */
} mc_update_tables_t;

typedef struct mc_update_stats {
  int64_t hit;               /* cells reached by a packet (updated)            */
  int64_t converged;         /* |dX(H0)/X(H0)| <= xhi_limit                    */
  int64_t no_te_balance;     /* noTeBal: 25 T steps without balance            */
  int64_t no_ion_balance;    /* noIonBal                                       */
  int64_t t_iterations;      /* sum of T steps over the hit cells              */
  double dte_max;            /* max |Te_new - Te_old| / Te_old over hit cells  */
  double frac_dte_1pc;       /* fraction of hit cells with |dTe| / Te < 1 %    */
  double moments_ms, update_ms;
  int64_t warm_fallback;     /* warm start: predictions sent back to the cold
                                solve (residual >= near_res x the heating)     */
} mc_update_stats_t;

/* Uploads the atomic tables, the per-cell Hden and the abundances of
 * H, He, C, N, O, Ne, S (number, relative to H). */
mc_status mc_ctx_set_update_tables(mc_ctx_t *ctx, const mc_update_tables_t *tables, const double *hden,
                                   const double *abund);
/* Cell state: te, ne [Nc+1]; ionden [Nc+1][7][8] (element, stage 1..7);
 * flags per cell: 1 = no Te balance, 2 = no ion balance, 4 = the warm start's
 * prediction was sent back to the cold solve. */
mc_status mc_ctx_set_cell_state(mc_ctx_t *ctx, const double *te, const double *ne, const double *ionden);
mc_status mc_ctx_get_cell_state(mc_ctx_t *ctx, double *te, double *ne, double *ionden, int32_t *conv,
                                int32_t *niter, int32_t *flags);
/* One update of every cell from the resident Jste: w [nbins][67] (column 0
 * = 1, then the photoionisation and the heating weights of the 33 balance
 * ions), scale = the Jste normalisation (1e-9, / 8 for a symmetric octant).
 * precision MC_PREC_FP64: the FP64 method (follows the FP64 oracle to
 * ~1e-9); MC_PREC_FP32: the same steps in 4-byte floats, the precision of
 * the reference's own updateCell (`real`), ~64x the FP64 rate on GB300. */
mc_status mc_ctx_update_cells(mc_ctx_t *ctx, const float *w, double scale, double xhi_limit, int32_t precision,
                              mc_update_stats_t *stats);

/* Grains in the gas update (lgDust and lgGas with lgPhotoelectric, the
 * reference's default): every T step of every cell then runs
 * setGrainPotential, setPhotoelHeatCool and setDustGasCollHeatCool
 * (source/update_mod.f90:527-930, called at :367-386) between ionBalance and
 * thermBalance, which adds the photoelectric heating and the collisional
 * cooling of the gas (:1251-1254).  The collision terms use the grain
 * temperatures the last mc_ctx_dust_temperatures left on the device (0 K
 * before the first, as the reference's Tdust starts), and the next
 * mc_ctx_dust_temperatures adds each size's gasDustColl_d - photoelHeat_d of
 * the last update to its absorbed integral (getDustT, :1886-1889).  The cell
 * flag 8 marks a grain potential that did not converge within 100 steps in
 * the cell's last T step.  One grain species in nsizes size bins. */
typedef struct mc_grain_physics {
  int32_t nsizes;            /* 1..32 size bins                                */
  const float *xs_abs;       /* [nsizes][nbins] absorption cross-section per
                                grain [cm^2] (xSecArray at dustAbsXsecP)       */
  const double *radius_um;   /* [nsizes] grainRadius [um]                      */
  const double *weight;      /* [nsizes] grainWeight                           */
  double abundance;          /* grainAbun of the species                       */
  double vn;                 /* grainVn [Ryd] (the species' n,k file header)   */
  double msurf;              /* MsurfAtom (the same header)                    */
  const double *ion_nu;      /* [33] threshold [Ryd] of each balance ion: the
                                IP whose energy a recombining stage above it
                                leaves on the grain (IPerg)                    */
  const float *ndust;        /* [Nc+1] grains per cm^3 (Ndust)                 */
} mc_grain_physics_t;

/* grains NULL: a gas-only update again.  Replaces nothing on the Fortran
 * side: the reference reads the same quantities from its dust module. */
mc_status mc_ctx_set_grain_physics(mc_ctx_t *ctx, const mc_grain_physics_t *grains);
/* The grain block of each cell's last T step in the last update with
 * grains, host arrays [nsizes][Nc+1]: the potential grainPot [Ryd],
 * photoelHeat_d and gasDustColl_d (any pointer may be NULL). */
mc_status mc_ctx_grain_state(mc_ctx_t *ctx, double *potential, double *photoel_cool, double *coll_heat);
/* Rebuilds the resident opacity from the cell state: den[k][cell] =
 * ionden(elem_k, stage_k) * abund(elem_k) * Hden(cell) for the nspecies rows
 * (elem, stage) = species[k], then the contraction with xs [nspecies][nbins]
 * as mc_ctx_build_opacity. */
/* Opacity rows that do not follow the cell state, appended to every
 * mc_ctx_opacity_from_state contraction: den [nrows][Nc+1] (e.g. Ndust) and
 * xs [nrows][nbins] (e.g. the grains' absorption + scattering per grain,
 * the dust add of iteration_mod.f90:166-227); nrows 0 removes them. */
mc_status mc_ctx_set_fixed_opacity(mc_ctx_t *ctx, int32_t nrows, const float *den, const float *xs);
/* The grains' opacity in every mc_ctx_opacity_from_state (the dust add of
 * iteration_mod.f90:166-227): per size bin k and cell, weight(k) Ndust x
 * (xs_ext(k) = abs + sca per grain) joins the opacity and weight(k) Ndust x
 * xs_sca(k) the scattering table (scaOpac), for the sizes whose grain
 * temperature (the last mc_ctx_dust_temperatures; 0 K before the first) is
 * below t_sublime (TdustSublime: sublimated grains drop out).  One species:
 * weight = grainAbun x grainWeight.  nsizes 0 removes them. */
mc_status mc_ctx_set_grain_opacity(mc_ctx_t *ctx, int32_t nsizes, const float *xs_ext, const float *xs_sca,
                                   const float *weight, const float *ndust, float t_sublime);

/* Resonance-line packets (energyPacketDriver, source/photon_mod.f90:180-266,
 * which runs them when lgDust and convPercent >= resLinesTransfer): counts
 * [Nc+1] = resLinePackets of each active cell (initResLinePackets,
 * emission_mod.f90:150-245, stays with the caller).  Every later mc_ctx_run
 * in the wave forms sends, after each star's packets, a block of "diffuse"
 * packets with that star's deltaE: counts[cell] of them from the node
 * (xAxis(ix), yAxis(iy), zAxis(iz)) of each cell, in the reference's loop
 * order (x outer, z inner), each followed through its re-emissions.  Their
 * draws come from Philox streams keyed by star index istar | 0x80.  Not with
 * MC_RUN_FORM_PLAIN, replayed draws or more than 8 sources (MC_ERR_UNSUPPORTED).
 * counts NULL (or all zero) turns them off. */
mc_status mc_ctx_set_res_lines(mc_ctx_t *ctx, const int32_t *counts);
mc_status mc_ctx_opacity_from_state(mc_ctx_t *ctx, int32_t nspecies, const int32_t *species, const float *xs,
                                    int32_t method, double *kernel_ms);

/* ---- the learned warm start of the cell update ----------------------------
 * An MLP (80 -> 256 -> 256 -> 256 -> 48, ReLU; BF16 operands, FP32
 * accumulation and Adam, all on the GPU) from the Jste sums of a cell (log10
 * of sum Jste, of the 33 photoionisation and 33 heating sums, of Hden) to
 * log10 Te and log10 of the 40 ionic fractions.  Trained on cell states the
 * update produced (collect after mc_ctx_update_cells), it warm-starts the
 * update: mc_ctx_update_cells_warm writes the prediction into the state and
 * runs the same solve from there.  At the first T step the solve accepts
 * the prediction when the thermal residual is below 1 % of the heating (or
 * the stricter accept_res of mc_ctx_surrogate_rule); below 30 % (near_res)
 * it brackets the balance from the prediction with steps of 3 %, 6 %, 12 %,
 * then the reference's 20 %, before its secant; otherwise the cell falls
 * back to the plain solve from the state before the prediction (20 % steps,
 * the full 25 T steps; counted in warm_fallback).  Every result
 * meets the reference's 1 % residual test.  No counterpart in the reference
 * (updateCell starts from the previous iteration's state with 20 % steps). */
mc_status mc_ctx_surrogate_init(mc_ctx_t *ctx, uint64_t seed, int64_t capacity);
mc_status mc_ctx_surrogate_collect(mc_ctx_t *ctx, int64_t *rows);
mc_status mc_ctx_surrogate_train(mc_ctx_t *ctx, int32_t steps, int32_t batch, float lr, uint64_t seed, double *loss,
                                 double *train_ms);
mc_status mc_ctx_update_cells_warm(mc_ctx_t *ctx, const float *w, double scale, double xhi_limit, int32_t precision,
                                   mc_update_stats_t *stats);
/* The warm start's rule at the first T step, in units of the heating: a
 * prediction whose thermal residual is below accept_res (0 < accept_res <=
 * 0.01, the reference's own test; default 0.01) is accepted; below near_res
 * (>= accept_res; default 0.3) it is bracketed from the prediction; from
 * near_res up the cell goes back to the plain solve.  accept_res = near_res
 * = 1e-3 is "accept below 1e-3, otherwise the plain solve". */
mc_status mc_ctx_surrogate_rule(mc_ctx_t *ctx, double accept_res, double near_res);

/* ---- diffuse-emission CDF on the GPU ---------------------------------------
 * emissionDriver + setDiffusePDF (emission_mod.f90:32-1311) for a gas grid:
 * from the resident cell state, every cell's recPDF row (the cumulative f-b,
 * f-f, two-photon and heavy-ion continua of HI, HeI and HeII, normalised,
 * entries above 0.999998 set to 1) and totalLines (the fraction of the
 * emitted energy in recombination and forbidden lines), written in place
 * into the transport's CDF rows.  Replaces the per-cell host loop the
 * Fortran runs before each transport (iteration_mod.f90, emissionDriver
 * calls) and the allreduce of recPDF.  The tables are the reference's own
 * module arrays; nu and wid_flx are the grid's nuArray and widFlx. */
typedef struct mc_emission_tables {
  int32_t nbins;             /* must equal the grid's                          */
  const float *nu, *wid_flx; /* [nbins] nuArray [Ryd], widFlx                  */
  const float *xs_h, *xs_hei, *xs_heii; /* [nbins] HI, HeI-singlet, HeII
                                ground-state cross-sections [cm^2] at each bin */
  int32_t ntk;               /* gamma temperature points (tkGamma)             */
  const float *tk;           /* [ntk]                                          */
  int32_t nlim_hi, nlim_hei, nlim_heii; /* nlimGammaHI & co. (even)            */
  const float *nu_gamma_hi, *nu_gamma_hei, *nu_gamma_heii; /* [nlim] edges     */
  const float *lg_hi, *lg_hei, *lg_heii; /* [ntk][nlim] log10 gamma (0: none) */
  const float *y_ay;         /* [41][2] y_dat, Ay_dat (HeI 2^1S two-photon)    */
  const float *hi_rec;       /* [16][9] HIRecLineData (iup, ilow)              */
  const float *heii_rec;     /* [31][17] HeIIRecLineData                       */
  const float *heii_lyman;   /* [4][2] HeIILymanData, HeIILymanNu              */
  const float *hei_rec;      /* [34][3][4] HeIrecLineCoeff, first column x1e25 */
  const double *gaunt_dd;    /* [88] getGauntFF's dd                           */
  int32_t n_heavy;           /* recombining heavy ions (<= 32)                 */
  const int32_t *heavy;      /* [n_heavy][8]: z, ion, nElec, outShell, g0, g1,
                                IPnuP, highNuP (1-based bins)                  */
  const float *xs_outer;     /* [n_heavy][nbins] outer-shell cross-section     */
  /* grains (0 sizes: no dust terms).  The grain temperatures are the ones
   * mc_ctx_dust_temperatures left on the device (none yet: no dust emission). */
  int32_t n_sizes;           /* grain size bins of the one species (<= 16)     */
  const float *xs_abs;       /* [n_sizes][nbins] absorption cross-section per
                                grain [cm^2] (xSecArray at dustAbsXsecP)       */
  const float *grain_weight; /* [n_sizes] grainWeight x grainAbun             */
  float t_sublime;           /* TdustSublime [K]                               */
  const float *ndust;        /* [Nc+1] grains per cm^3 (Ndust)                 */
} mc_emission_tables_t;

mc_status mc_ctx_set_emission_tables(mc_ctx_t *ctx, const mc_emission_tables_t *tables);
/* Builds every cell's emission CDF from the resident Te, Ne and ionic
 * fractions (needs mc_ctx_set_update_tables for the forbidden lines and the
 * abundances, and a cell state); ms = device time, or NULL.  With grains and
 * grain temperatures: on a gas grid the thermal grain emission joins the
 * recPDF rows (sumDiffuseDust, emission_mod.f90:1042-1105); on a dust-only
 * grid the dustPDF rows are built instead (setDustPDF, :1313-1387). */
mc_status mc_ctx_build_emission(mc_ctx_t *ctx, float *ms);
/* Downloads the CDF rows [Nc+1][nbins] and totalLines [Nc+1] (either NULL). */
mc_status mc_ctx_get_emission(mc_ctx_t *ctx, float *rec_rows, float *total_lines);
/* Downloads the dust-emission CDF rows [Nc+1][nbins] (dust-only grids). */
mc_status mc_ctx_get_dust_emission(mc_ctx_t *ctx, float *dust_rows);
/* The collected training rows (features [n][80], targets [n][48], as
 * collect forms them, not normalised): rows gives their count and, with x
 * and t, copies them out; load appends rows (up to the capacity), e.g. the
 * cell states of other models' updates, so one network learns from many. */
mc_status mc_ctx_surrogate_rows(mc_ctx_t *ctx, int64_t *n, float *x, float *t);
mc_status mc_ctx_surrogate_load(mc_ctx_t *ctx, int64_t n, const float *x, const float *t);
/* Parameters (164656 floats: W1[256][80] b1 W2[256][256] b2 W3[256][256] b3
 * W4[48][256] b4). */
mc_status mc_ctx_surrogate_params(mc_ctx_t *ctx, float *get, const float *set);
/* Loss and gradients of one batch (x [m][80], normalised targets t [m][48];
 * the first 41 columns count), and the outputs y [m][48]. */
mc_status mc_ctx_surrogate_grads(mc_ctx_t *ctx, int32_t m, const float *x, const float *t, double *loss, float *grads,
                                 float *y);
/* The network's outputs y [m][48] for m feature rows x [m][80] with the
 * prediction's arithmetic (the four layers on tcgen05: BF16 operands, FP32
 * accumulators in tensor memory), as mc_ctx_update_cells_warm computes them
 * for every cell. */
mc_status mc_ctx_surrogate_forward(mc_ctx_t *ctx, int32_t m, const float *x, float *y);

/* Scheduling parameters of the persistent march (results do not depend on
 * them beyond the order of the FP64 sums): refill_min = free lanes a warp
 * collects before it takes new packets from the queue (1..32, default 8);
 * inner_steps = cell crossings a lane takes between refill checks (1..64,
 * default 4).  mocassin_gb300/autotune.py picks them by timing. */
mc_status mc_ctx_set_tuning(mc_ctx_t *ctx, int32_t refill_min, int32_t inner_steps);
mc_status mc_ctx_get_tuning(mc_ctx_t *ctx, int32_t *refill_min, int32_t *inner_steps);

/* Copies the resident opacity [nbins][Nc+1] (cell fastest) to the host. */
mc_status mc_ctx_get_opacity(mc_ctx_t *ctx, float *opacity);
/* The resident scattering table (scaOpac, the layout of opacity) of a dusty grid. */
mc_status mc_ctx_get_scattering(mc_ctx_t *ctx, float *scattering);

/* ---- allocation-free transport ------------------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc
 * (a code that only hands over device memory it already manages, or a loop
 * where an allocation could block or fail): runs the one-thread-per-history
 * transport on DEVICE arrays the caller owns and allocates nothing.  Every
 * pointer of `grid` (axes, active, opacity, ..., with rec_pdf / dust_pdf in
 * the Fortran layout above), each spec_cdf of `src`, opts->replay and the
 * jste / jdif / escaped accumulators are device pointers; `src`, `opts` and
 * `stats` are host structs.  Its scratch (counters, first error, cell-width
 * tables) is one fixed device array of about 37 KB that every GPU loading
 * the library holds until exit; grids above 1024 cells along an axis or
 * more than 16 sources are rejected with MC_ERR_UNSUPPORTED.  All calls
 * share that array, so calls that overlap on the GPU race: serialise them.
 * Every call looks up the array's device address with the caller's device
 * current (so a cudaDeviceReset, which moves it, is harmless); the first
 * call on a device also loads the module there, so make it before any
 * stream capture.  Every argument is checked before anything is written:
 * the host-side ones first, then the caller's `active` array on the device
 * (a negative entry, a sub-grid pointer, is MC_ERR_UNSUPPORTED; one above
 * ncells is MC_ERR_ARG, as mc_transport_run reports them), and a rejected
 * call returns with the estimators untouched.  `stream` is a cudaStream_t
 * (NULL: default stream); the call returns after the stream has finished
 * its work.  Results equal mc_transport_run with MC_RUN_FORM_PLAIN on the
 * same inputs and draws. */
mc_status mc_transport_run_noalloc(const mc_grid_t *grid, const mc_source_t *src, int32_t nsrc,
                                   const mc_run_opts_t *opts, double *jste, double *jdif,
                                   double *escaped, mc_stats_t *stats, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* MOCASSIN_GPU_H */
