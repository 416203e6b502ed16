// transport_noalloc.cu -- mc_transport_run_noalloc: the packet transport for
// callers that cannot allocate device memory.
//
// Some callers of this library cannot call cudaMalloc at all: a host code
// that hands the library only memory it already owns (a Fortran model whose
// arrays live in a device pool it manages, a framework with its own caching
// allocator that must see every allocation), or a loop that runs where an
// allocation could block or fail at a bad moment.  For them this entry point
// runs the one-thread-per-history transport (the plain form) on device
// arrays the caller passes, and allocates nothing: no cudaMalloc, no
// cudaFree, no allocating library call.  The only scratch it needs -- the
// event counters, the first-error record and the per-axis cell-width tables
// of photon_mod.f90:1469-1512 -- lives in the fixed array below.
//
// Limits: at most kNoAllocMaxAxis cells along each axis and
// mcg::kMaxSources stars per call (larger inputs are rejected with
// MC_ERR_UNSUPPORTED).  The array takes kNoAllocScratchBytes of every GPU
// that loads the library, until the process exits.  All calls share it:
// calls that overlap on the GPU (two streams, two host threads) race on it,
// so serialise them.  Every call looks up the array's device address
// (cudaGetSymbolAddress) with the caller's device current; the first call on
// a device also loads the module there, so make that first call before any
// stream capture begins.  Looking the address up per call keeps it right
// after a cudaDeviceReset, which reloads the module elsewhere.
//
// Order of work: every host-side argument check runs first; then one small
// kernel checks the caller's `active` array on the device (a negative entry
// is a sub-grid pointer, MC_ERR_UNSUPPORTED; one above ncells is MC_ERR_ARG,
// as mc_transport_run reports them) and the call waits for its verdict.  A
// rejected call therefore returns before anything writes the caller's
// estimators, and with nothing of its own left running on the stream.
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "../../include/mocassin_gpu.h"
#include "mc_device.cuh"
#include "mc_launch.h"
#include "transport_plain.cuh"

namespace {

constexpr int kNoAllocMaxAxis = 1024;
// layout: DevCounters (+ the active check's two first indices at
// kCheckOffset) | dx32 dy32 dz32 (floats) | dx64 dy64 dz64 (doubles)
constexpr size_t kCountersBytes = 256;
constexpr size_t kCheckOffset = 128;
constexpr size_t kF32Bytes = 3 * kNoAllocMaxAxis * sizeof(float);
constexpr size_t kF64Bytes = 3 * kNoAllocMaxAxis * sizeof(double);
constexpr size_t kNoAllocScratchBytes = kCountersBytes + kF32Bytes + kF64Bytes;
static_assert(sizeof(mcg::DevCounters) <= kCheckOffset, "counters do not fit their slot");

// Host code must not use this name as an address: it is a host-side stand-in.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// First (lowest) index of a negative `active` entry and of one above ncells;
// INT_MAX when there is none.
struct ActiveCheck {
  int first_negative;
  int first_too_large;
};

mc_status fail(mc_status code, const char *msg) {
  mcg::set_last_error_text(msg);
  return code;
}

// Device address of the scratch array on the current device, looked up with
// that device current.
mc_status scratch_address(unsigned char **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(MC_ERR_NO_DEVICE, "no current CUDA device");
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
    return fail(MC_ERR_CUDA, (std::string("cudaGetSymbolAddress(scratch) failed: ") + cudaGetErrorString(e)).c_str());
  *out = (unsigned char *)p;
  return MC_OK;
}

// The caller's active(nx,ny,nz) against the rows the march may touch.
__global__ void noalloc_active_check_kernel(const int32_t *active, long long n, int ncells, ActiveCheck *out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int a = active[i];
    if (a < 0) atomicMin(&out->first_negative, (int)i);
    if (a > ncells) atomicMin(&out->first_too_large, (int)i);
  }
}

// dV widths / 1e15 of every cell index (photon_mod.f90:1469-1512), from the
// caller's device axes into the scratch tables, in FP32 and FP64.
__global__ void noalloc_widths_kernel(const float *xa, const float *ya, const float *za, int nx, int ny, int nz,
                                      int sym, float *w32, double *w64) {
  const int n[3] = {nx, ny, nz};
  const float *ax[3] = {xa, ya, za};
  for (int k = 0; k < 3; ++k)
    for (int p = 1 + threadIdx.x; p <= n[k]; p += blockDim.x) {
      const float *A = ax[k] - 1;
      const int nn = n[k];
      float d;
      double dd;
      if (p > 1 && p < nn) {
        d = fabsf(A[p + 1] - A[p - 1]) / 2.f;
        dd = fabs((double)A[p + 1] - (double)A[p - 1]) / 2.0;
      } else if (p == 1) {
        d = sym ? fabsf(A[p + 1] - A[p]) / 2.f : fabsf(A[p + 1] - A[p]);
        dd = sym ? fabs((double)A[p + 1] - (double)A[p]) / 2.0 : fabs((double)A[p + 1] - (double)A[p]);
      } else {
        d = fabsf(A[p] - A[p - 1]);
        dd = fabs((double)A[p] - (double)A[p - 1]);
      }
      w32[k * kNoAllocMaxAxis + p - 1] = d / 1.e15f;
      w64[k * kNoAllocMaxAxis + p - 1] = dd / (double)1.e15f;
    }
}

}  // namespace

// See include/mocassin_gpu.h.
extern "C" mc_status mc_transport_run_noalloc(const mc_grid_t *g, const mc_source_t *src,
                                              int32_t nsrc, const mc_run_opts_t *o, double *jste, double *jdif,
                                              double *escaped, mc_stats_t *stats, void *stream_handle) {
  if (!g || !src || !o || !jste) return fail(MC_ERR_ARG, "grid, src, opts and jste are required");
  if (g->nx < 2 || g->ny < 2 || g->nz < 2) return fail(MC_ERR_UNSUPPORTED, "nx, ny, nz must be >= 2");
  if (g->nx > kNoAllocMaxAxis || g->ny > kNoAllocMaxAxis || g->nz > kNoAllocMaxAxis)
    return fail(MC_ERR_UNSUPPORTED, "mc_transport_run_noalloc: more than 1024 cells along an axis");
  if (nsrc < 1 || nsrc > mcg::kMaxSources) return fail(MC_ERR_UNSUPPORTED, "mc_transport_run_noalloc: 1..16 sources");
  if (g->n_angle != 0) return fail(MC_ERR_UNSUPPORTED, "nAngleBins > 0 is not supported");
  if (g->nbins < 3 || g->ncells < 0) return fail(MC_ERR_ARG, "bad nbins / ncells");
  const bool gas = g->flags & MC_FLAG_GAS, dust = g->flags & MC_FLAG_DUST;
  if (!g->x_axis || !g->y_axis || !g->z_axis || !g->active || !g->opacity || !g->nu_array)
    return fail(MC_ERR_ARG, "grid device arrays missing");
  if (!gas && !dust) return fail(MC_ERR_ARG, "grid has neither gas nor dust");
  if (gas && (!g->rec_pdf || !g->total_lines)) return fail(MC_ERR_ARG, "gas grid needs rec_pdf and total_lines");
  if (dust && !g->sca_opac) return fail(MC_ERR_ARG, "dust grid needs sca_opac");
  if (dust && !gas && !g->dust_pdf) return fail(MC_ERR_ARG, "dust-only grid needs dust_pdf");
  if (dust && !(g->flags & MC_FLAG_ISOTROPIC) && !g->g_sca) return fail(MC_ERR_ARG, "HG scattering needs g_sca");
  if ((g->flags & MC_FLAG_DEBUG) && !jdif) return fail(MC_ERR_ARG, "debug grid needs jdif");
  if (o->precision != MC_PREC_FP32 && o->precision != MC_PREC_FP64) return fail(MC_ERR_ARG, "bad precision");
  if (o->rng == MC_RNG_REPLAY && (!o->replay || o->replay_stride <= 0)) return fail(MC_ERR_ARG, "replay needs draws");

  // Sources: every host-side check before any device work is queued.
  mcg::DevSources S{};
  S.nsrc = nsrc;
  long long tot = 0;
  for (int i = 0; i < nsrc; ++i) {
    const mc_source_t &x = src[i];
    if (!x.spec_cdf || x.n_packets < 0) return fail(MC_ERR_ARG, "source needs a device spec_cdf and n >= 0");
    if (x.cell[0] < 1 || x.cell[0] > g->nx || x.cell[1] < 1 || x.cell[1] > g->ny || x.cell[2] < 1 ||
        x.cell[2] > g->nz)
      return fail(MC_ERR_BOUNDS, "source cell outside the grid");
    mcg::DevSource &s = S.s[i];
    s.cdf = x.spec_cdf;  // device pointer, sampled by the linear scan
    for (int k = 0; k < 3; ++k) { s.cell[k] = x.cell[k]; s.pos[k] = x.pos[k]; }
    s.delta_e = x.delta_e;
    s.k0 = (uint32_t)o->seed;
    s.k1 = (uint32_t)(o->seed >> 32) ^ ((o->iteration & 0xFFFFFFu) << 8) ^ ((uint32_t)x.istar & 0xFFu);
    s.n = x.n_packets;
    s.base = tot;
    tot += x.n_packets;
  }
  S.total = tot;

  unsigned char *base = nullptr;
  mc_status st = scratch_address(&base);
  if (st) return st;
  cudaStream_t stream = (cudaStream_t)stream_handle;
  const bool sym = g->flags & MC_FLAG_SYMMETRIC_XYZ;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms < 1) sms = 1;

  // The counters must start at zero every call (they keep the last call's
  // values), and so must the active check.
  mcg::DevCounters h{};
  h.error_packet = -1;
  const char *be = getenv("MC_KERNEL_BUDGET_S");
  double budget = be ? atof(be) : 120.0;
  if (!(budget > 0)) budget = 120.0;
  h.budget_ns = (unsigned long long)(budget * 1e9);
  mcg::DevCounters *dcnt = (mcg::DevCounters *)base;
  ActiveCheck chk{INT_MAX, INT_MAX};
  ActiveCheck *dchk = (ActiveCheck *)(base + kCheckOffset);
  if (cudaMemcpyAsync(dcnt, &h, sizeof h, cudaMemcpyHostToDevice, stream) != cudaSuccess ||
      cudaMemcpyAsync(dchk, &chk, sizeof chk, cudaMemcpyHostToDevice, stream) != cudaSuccess)
    return fail(MC_ERR_CUDA, "counter reset failed");

  // active(x,y,z) on the device: the march indexes opacity and Jste by it, so
  // a row outside 0..ncells must stop the call before the march runs.
  const long long ncell3 = (long long)g->nx * g->ny * g->nz;
  {
    const long long want = (ncell3 + 255) / 256;
    const unsigned blocks = (unsigned)(want < (long long)sms * 4 ? want : (long long)sms * 4);
    noalloc_active_check_kernel<<<blocks, 256, 0, stream>>>(g->active, ncell3, g->ncells, dchk);
    if (cudaGetLastError() != cudaSuccess) return fail(MC_ERR_CUDA, "active-check launch failed");
    if (cudaMemcpyAsync(&chk, dchk, sizeof chk, cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
        cudaStreamSynchronize(stream) != cudaSuccess)
      return fail(MC_ERR_CUDA, "reading the active check back failed");
    const int neg = chk.first_negative, big = chk.first_too_large;
    if (neg != INT_MAX || big != INT_MAX) {
      char buf[96];
      if (neg <= big) {
        snprintf(buf, sizeof buf, "active < 0 (sub-grid pointer) at %d", neg);
        return fail(MC_ERR_UNSUPPORTED, buf);
      }
      snprintf(buf, sizeof buf, "active entry %d exceeds ncells %d", big, g->ncells);
      return fail(MC_ERR_ARG, buf);
    }
  }

  // per-axis widths into the scratch tables (they keep the last call's grid)
  float *d32 = (float *)(base + kCountersBytes);
  double *d64 = (double *)(base + kCountersBytes + kF32Bytes);
  noalloc_widths_kernel<<<1, 256, 0, stream>>>(g->x_axis, g->y_axis, g->z_axis, g->nx, g->ny, g->nz, sym ? 1 : 0,
                                               d32, d64);
  if (cudaGetLastError() != cudaSuccess) return fail(MC_ERR_CUDA, "width-table launch failed");
  if (o->run_flags & MC_RUN_ZERO_FIRST) {
    const size_t nj = (size_t)(g->ncells + 1) * g->nbins, ne = (size_t)(g->ncells + 1) * (g->nbins + 1);
    if (cudaMemsetAsync(jste, 0, nj * sizeof(double), stream) != cudaSuccess ||
        (jdif && cudaMemsetAsync(jdif, 0, nj * sizeof(double), stream) != cudaSuccess) ||
        (escaped && cudaMemsetAsync(escaped, 0, ne * sizeof(double), stream) != cudaSuccess))
      return fail(MC_ERR_CUDA, "zeroing the estimators failed");
  }

  mcg::DevGrid d{};
  d.nx = g->nx; d.ny = g->ny; d.nz = g->nz; d.nc = g->ncells; d.nb = g->nbins;
  d.xa = g->x_axis; d.ya = g->y_axis; d.za = g->z_axis;
  d.active = g->active;
  d.opacity = g->opacity;
  d.sca = g->sca_opac;
  d.rec_cdf = g->rec_pdf;    // Fortran layout, sampled by the linear scan
  d.dust_cdf = g->dust_pdf;
  d.total_lines = g->total_lines;
  d.nu = g->nu_array;
  d.gsca = g->g_sca;
  d.dx32 = d32; d.dy32 = d32 + kNoAllocMaxAxis; d.dz32 = d32 + 2 * kNoAllocMaxAxis;
  d.dx64 = d64; d.dy64 = d64 + kNoAllocMaxAxis; d.dz64 = d64 + 2 * kNoAllocMaxAxis;
  d.gc[0] = g->geo_corr[0]; d.gc[1] = g->geo_corr[1]; d.gc[2] = g->geo_corr[2];
  d.rout = g->r_out;
  d.ion_edge1 = g->ion_edge1;
  d.flags = g->flags;
  d.recursion_limit = o->recursion_limit > 0 ? o->recursion_limit : 5000;
  d.safe_limit = o->safe_limit > 0 ? o->safe_limit : 500000;
  d.jste = jste; d.jdif = jdif; d.esc = escaped;

  mcg::DevReplay rp{o->rng == MC_RNG_REPLAY ? o->replay : nullptr, o->rng == MC_RNG_REPLAY ? o->replay_stride : 0};

  if (tot > 0) {
    const long long want = (tot + 255) / 256;
    const long long blocks = want < (long long)sms * 2 ? want : (long long)sms * 2;
    if (o->precision == MC_PREC_FP64)
      mcg::transport_plain_kernel<double, 1><<<(unsigned)blocks, 256, 0, stream>>>(d, S, rp, dcnt);
    else
      mcg::transport_plain_kernel<float, 1><<<(unsigned)blocks, 256, 0, stream>>>(d, S, rp, dcnt);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(MC_ERR_CUDA, (std::string("transport launch failed: ") + cudaGetErrorString(e)).c_str());
  }
  if (cudaMemcpyAsync(&h, dcnt, sizeof h, cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
      cudaStreamSynchronize(stream) != cudaSuccess)
    return fail(MC_ERR_CUDA, "reading the counters back failed");
  if (stats) {
    memset(stats, 0, sizeof *stats);
    stats->crossings = (int64_t)h.crossings;
    stats->absorptions = (int64_t)h.absorptions;
    stats->scatterings = (int64_t)h.scatterings;
    stats->escaped = (int64_t)h.escaped;
    stats->lines = (int64_t)h.lines;
    stats->trapped = (int64_t)h.trapped;
    stats->silent_exits = (int64_t)h.silent;
    stats->safe_limit_hits = (int64_t)h.safe_hits;
    stats->qphot = h.qphot;
    stats->error_code = h.error_code;
    stats->error_packet = h.error_packet;
    stats->rounds = 1;
  }
  if (h.error_code != 0) {
    char buf[96];
    snprintf(buf, sizeof buf, "device error %d in packet %d", h.error_code, h.error_packet);
    return fail((mc_status)h.error_code, buf);
  }
  return MC_OK;
}
