// mcgpu_api.cu -- the C-ABI of libmcgpu.so (include/mocassin_gpu.h).
//
// Host side of the drop-in for energyPacketDriver (source/photon_mod.f90:26-285):
// validates the Fortran-layout arrays, keeps a resident copy of the grid in
// HBM, launches the transport and hands the estimators back.  All errors are
// returned as mc_status with a message for mc_last_error(); nothing here
// aborts the process (the reference's "print*; stop" sites become codes).
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/mocassin_gpu.h"
#include "mc_device.cuh"
#include "tc_util.cuh"
#include "mc_launch.h"
#include "wave_types.cuh"

namespace {

thread_local std::string g_last_error;

mc_status set_error(mc_status code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

#define MC_CUDA(call)                                                                      \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return set_error(e_ == cudaErrorMemoryAllocation ? MC_ERR_NOMEM : MC_ERR_CUDA,        \
                       "%s failed: %s", #call, cudaGetErrorString(e_));                    \
  } while (0)

// Device buffer owned by a context.
// NVTX range over a C-ABI call, for timeline tools (nsys, ncu's NVTX filter)
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

struct DBuf {
  void *p = nullptr;
  size_t bytes = 0;
  DBuf() = default;
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  ~DBuf() { if (p) cudaFree(p); }
  cudaError_t alloc(size_t b) {
    bytes = b;
    return cudaMalloc(&p, b ? b : 16);
  }
  template <typename T> T *as() const { return (T *)p; }
};

// (re)allocates b to at least `bytes` (contents not kept)
mc_status ensure(DBuf &b, size_t bytes) {
  if (b.p && b.bytes >= bytes) return MC_OK;
  if (b.p) { cudaFree(b.p); b.p = nullptr; b.bytes = 0; }
  MC_CUDA(b.alloc(bytes));
  return MC_OK;
}

}  // namespace

namespace mcg {

void set_last_error_text(const char *msg) { g_last_error = msg; }

// Transposes a [nb][nc1] cell-fastest CDF into [nc1][nb] rows and applies a
// running maximum along each row.  Block: 32 cells; tiles of 32 bins go
// through shared memory so both the read and the write are coalesced.
__global__ void cdf_transpose_kernel(const float *__restrict__ in, float *__restrict__ out, int nc1, int nb) {
  __shared__ float tile[32][33];
  const int c0 = blockIdx.x * 32;
  const int tx = threadIdx.x, ty = threadIdx.y;  // 32 x 8
  float run = -INFINITY;                         // running max of cell c0+tx (owned by ty == 0 lanes)
  for (int v0 = 0; v0 < nb; v0 += 32) {
    for (int k = ty; k < 32; k += 8) {
      const int v = v0 + k, c = c0 + tx;
      tile[k][tx] = (v < nb && c < nc1) ? in[(long long)v * nc1 + c] : 0.f;
    }
    __syncthreads();
    if (ty == 0) {
      for (int k = 0; k < 32; ++k) {
        run = fmaxf(run, tile[k][tx]);
        tile[k][tx] = run;
      }
    }
    __syncthreads();
    for (int k = ty; k < 32; k += 8) {
      const int c = c0 + k, v = v0 + tx;
      if (c < nc1 && v < nb) out[(long long)c * nb + v] = tile[tx][k];
    }
    __syncthreads();
  }
}

#include "wave_util.inc"

cudaError_t launch_cdf_transpose(const float *in, float *out, int nc1, int nb, cudaStream_t stream) {
  dim3 block(32, 8);
  dim3 grid((nc1 + 31) / 32);
  cdf_transpose_kernel<<<grid, block, 0, stream>>>(in, out, nc1, nb);
  return cudaGetLastError();
}

}  // namespace mcg

struct mc_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  int nx = 0, ny = 0, nz = 0, nc = 0, nb = 0;
  uint32_t flags = 0;
  DBuf xa, ya, za, active, opacity, sca, rec_raw, rec_cdf, dust_raw, dust_cdf, tlines, nu, gsca;
  DBuf dx32, dy32, dz32, dx64, dy64, dz64;
  DBuf jste, jdif, esc;
  DBuf stage_j, stage_d, stage_e;  // FP32 staging of the drop-in call's estimators
  // MC_RUN_HOST_ZEROED downloads: per-bin nonzero flags of Jste / Jdif, the
  // compacted escapedPackets entries (indices, values) and their count
  DBuf z_mask, z_idx, z_val, z_cnt;
  // bytes the drop-in call copied host -> device / device -> host
  long long xfer_h2d = 0, xfer_d2h = 0;
  // the drop-in call's last geometry (axes, active, frequencies): a call with
  // the same geometry skips its re-upload and the march-order rebuild
  std::vector<float> geo_f;
  std::vector<int32_t> geo_a;
  // the drop-in call uploads and re-lays out recPDF on a side stream while
  // round 0 (stellar packets only) runs; round 1 waits for ev_cdf
  cudaStream_t side = nullptr;
  cudaEvent_t ev_side0 = nullptr, ev_cdf = nullptr;
  bool cdf_pending = false;
  // MC_RUN_HOST_ZEROED: the last call left the device estimators all zero
  // (it cleared what it had made nonzero after downloading it), so the next
  // one needs no full clear
  bool est_zero = false;
  unsigned long long *h_cnt = nullptr;  // pinned: the compacted escape count
  cudaEvent_t ev_done = nullptr;        // the transport's end, for the side stream
  DBuf view;        // viewing-angle table (n_angle > 0)
  int n_angle = 0;
  // cell update: atomic tables, per-cell state and scratch
  DBuf u_bal, u_cel, u_rrec, u_rnew, u_direc, u_aldro, u_logt, u_g, u_e, u_A, u_qq, u_q2, u_ab, u_hden;
  DBuf f_bal, f_cel, f_rrec, f_rnew, f_direc, f_aldro, f_logt, f_g, f_e, f_A, f_qq, f_q2, f_ab;  // float copies
  DBuf s_te, s_ne, s_X, s_conv, s_niter, s_flags, s_dte, s_mom, s_w, s_ustats, s_err, s_den, s_xs, s_spe, s_sps, s_wave;
  int u_ncel = 0, u_ndirec = 0, u_naldro = 0, u_maxlev = 1;
  int u_bal_z[7] = {}, u_bal_first[7] = {};
  // learned warm start: parameters, Adam state, training buffer, work arrays
  DBuf m_w, m_g, m_m1, m_m2, m_xs, m_ts, m_count, m_fmean, m_fstd, m_tmean, m_tstd, m_loss, m_dstep;
  DBuf m_gscr;  // the weight gradients' per-split partial sums
  DBuf m_ccnt;  // rows per block of the training-row collection
  DBuf m_xb, m_tb, m_a1, m_a2, m_a3, m_y, m_dy, m_d3, m_d2, m_d1, m_xi, m_h1, m_h2, m_h3, m_yi, m_te_prev, m_ne_prev, m_x_prev;
  long long m_cap = 0, m_n = 0;
  int m_step = 0, m_B = 0;
  bool m_ready = false, m_norm = false;
  double m_near_res = 0.3;  // warm start: residual / heating below which a prediction is bracketed
  double m_accept_res = 0.01;  // ... and below which it is accepted
  // diffuse-emission CDF: derived tables (one buffer) and forbidden-line totals
  DBuf e_tab, e_forb;
  DBuf e_ok, e_list, e_cnt;  // per cell: the line totals in e_forb belong to the state (1); stale-cell list
  DBuf d_tdust;      // grain temperatures of the last mc_ctx_dust_temperatures [nsizes+1][nc+1]
  // grains in the gas update (mc_ctx_set_grain_physics): tables and the
  // grain state of the last update with grains [3][nsizes][nc+1]
  DBuf g_nu, g_xs, g_rad, g_w, g_ip, g_ynd, g_dnud, g_qad, g_ynf, g_dnuf, g_qaf, g_nd, g_out, g_ihnu, g_idnuf;
  int g_ns = 0, g_ivn = 0;
  double g_vn = 0., g_msurf = 0., g_abun = 0.;
  bool g_fresh = false;  // g_out belongs to the last update
  DBuf o_fix_den, o_fix_xs;  // opacity rows that do not follow the cell state
  int o_nfix = 0;
  // the grains' opacity rows (mc_ctx_set_grain_opacity): cross-sections
  // [nsizes][nbins] (abs + sca, sca), weights, Ndust, and the scattering
  // table's densities of the last rebuild
  DBuf go_ext, go_sca, go_w, go_nd, go_den;
  int go_n = 0;
  float go_tsub = 0.f;
  int d_nsizes = 0;
  mcg::EmiArgs emi{};
  bool e_ready = false;
  bool u_ready = false, s_ready = false;
  // the FP32 update's launch sequence, captured once per argument set
  cudaGraphExec_t wave_exec = nullptr;
  mcg::UpdArgs wave_args{};
  void *wave_scratch = nullptr;
  DBuf counters, src_cdf, replay;
  // resonance-line packets (mc_ctx_set_res_lines): the cells that emit some,
  // packed, in the reference's loop order, and the packets before each
  DBuf res_cells, res_prefix;
  int res_ncell = 0;
  long long res_per_star = 0;
  // chosen form: march-indexed views and the sorted packet queue
  int identity = 1;
  long long ncell3 = 0;
  DBuf lin2cell, opac_m, sca_m, jste_m, jdif_m, bins;
  DBuf s_nu, s_words, queue, q_id, q_cell, q_words, q_meta, q_origin, q_r, q_v, q_pass;
  DBuf a_id, a_cell, a_words, a_run, a_r;
  size_t queue_cap = 0;
  int refill_min = 8;
  int inner_steps = 4;
  int rounds = 0;
  cudaEvent_t evm0 = nullptr, evm1 = nullptr;
  mcg::DevGrid g{};
  DBuf batch_desc;  // mc_batch_run's model descriptors and task counter (first context of a batch)
};

namespace {

mc_status check_grid(const mc_grid_t *g) {
  if (!g) return set_error(MC_ERR_ARG, "grid is NULL");
  if (g->nx < 2 || g->ny < 2 || g->nz < 2)
    return set_error(MC_ERR_UNSUPPORTED, "nx, ny, nz must be >= 2 (1D grids are not supported): %d %d %d",
                     g->nx, g->ny, g->nz);
  if (g->ncells < 0 || g->nbins < 3) return set_error(MC_ERR_ARG, "bad ncells/nbins %d/%d", g->ncells, g->nbins);
  if (g->n_angle < 0 || g->n_angle > 2)
    return set_error(MC_ERR_ARG, "nAngleBins must be 0..2 (set_input_mod.f90:537), got %d", g->n_angle);
  if (g->n_angle > 0 && (!g->view_theta || !g->view_phi))
    return set_error(MC_ERR_ARG, "nAngleBins > 0 needs view_theta and view_phi");
  if (g->n_theta_bins < 0 || g->n_theta_bins > 254 || g->n_phi_bins < 0 || g->n_phi_bins > 254)
    return set_error(MC_ERR_ARG, "angle bin counts must be 0..254");
  if (!g->x_axis || !g->y_axis || !g->z_axis || !g->active || !g->opacity || !g->nu_array)
    return set_error(MC_ERR_ARG, "grid axes/active/opacity/nu_array must be non-NULL");
  const bool gas = g->flags & MC_FLAG_GAS, dust = g->flags & MC_FLAG_DUST;
  if (!gas && !dust) return set_error(MC_ERR_ARG, "grid has neither gas nor dust");
  if (gas && (!g->rec_pdf || !g->total_lines)) return set_error(MC_ERR_ARG, "gas grid needs rec_pdf and total_lines");
  if (dust && !g->sca_opac) return set_error(MC_ERR_ARG, "dust grid needs sca_opac");
  if (dust && !gas && !g->dust_pdf) return set_error(MC_ERR_ARG, "dust-only grid needs dust_pdf");
  if (dust && !(g->flags & MC_FLAG_ISOTROPIC) && !g->g_sca)
    return set_error(MC_ERR_ARG, "anisotropic dust scattering needs g_sca");
  const int64_t ncell3 = (int64_t)g->nx * g->ny * g->nz;
  for (int64_t i = 0; i < ncell3; ++i) {
    const int a = g->active[i];
    if (a < 0) return set_error(MC_ERR_UNSUPPORTED, "active < 0 (sub-grid pointer) at %lld", (long long)i);
    if (a > g->ncells) return set_error(MC_ERR_ARG, "active %d exceeds ncells %d", a, g->ncells);
  }
  return MC_OK;
}

template <typename T> void widths(const float *ax, int n, bool sym, std::vector<T> &w) {
  // photon_mod.f90:1469-1512, divided by 1e15 (the FP32 literal)
  w.resize(n);
  for (int p = 1; p <= n; ++p) {
    T d;
    auto A = [&](int i) { return (T)ax[i - 1]; };
    if (p > 1 && p < n) d = std::fabs(A(p + 1) - A(p - 1)) / (T)2;
    else if (p == 1) d = sym ? std::fabs(A(p + 1) - A(p)) / (T)2 : std::fabs(A(p + 1) - A(p));
    else d = std::fabs(A(p) - A(p - 1));
    w[p - 1] = d / (T)1.e15f;
  }
}

mc_status upload(DBuf &b, const void *host, size_t bytes, cudaStream_t s) {
  MC_CUDA(b.alloc(bytes));
  if (host && bytes) MC_CUDA(cudaMemcpyAsync(b.p, host, bytes, cudaMemcpyHostToDevice, s));
  return MC_OK;
}

// The viewpoint of every (theta, phi) escape bin, as initCartesianGrid sets
// up viewPointPtheta / viewPointPphi (grid_mod.f90:416-468) and the escape
// sites test them (photon_mod.f90:414-447): entry [it][ip] is the angle
// plane that receives deltaE besides plane 0 (0 = none).
mc_status view_table(const mc_grid_t *g, mcg::DevGrid &d, std::vector<uint8_t> &tab) {
  const float pi = 3.141592654f, two_pi = 2.f * pi;  // constants_mod.f90:32-33
  const int na = g->n_angle;
  int nt = g->n_theta_bins > 0 ? g->n_theta_bins : 10;
  int np = g->n_phi_bins > 0 ? g->n_phi_bins : 20;
  std::vector<float> vth(g->view_theta, g->view_theta + na + 1), vph(g->view_phi, g->view_phi + na + 1);
  const float dth = pi / (float)nt;
  for (int i = 1; i <= na; ++i)
    if (vph[i] < 0.f) {  // phi dependence off
      np = 1;
      for (float &v : vph) v = -1.f;
      break;
    }
  const float dph = two_pi / (float)np;
  std::vector<int> pt(nt + 1, 0), pp(np + 1, 0);
  for (int i = 1; i <= na; ++i) {
    if (vth[i] > pi / 2.f && (g->flags & MC_FLAG_SYMMETRIC_XYZ))
      return set_error(MC_ERR_ARG, "viewing angle theta > pi/2 is not available for a symmetric grid");
    const int it = (int)(vth[i] / dth) + 1, ip = (int)(vph[i] / dph) + 1;
    if (it < 0 || it > nt || ip < 0 || ip > np)
      return set_error(MC_ERR_ARG, "viewing angle %d (%g, %g) outside the angle bins", i, vth[i], vph[i]);
    pt[it] = i;
    pp[ip] = i;
  }
  tab.assign((size_t)(nt + 1) * (np + 1), 0);
  for (int it = 1; it <= nt; ++it)
    for (int ip = 1; ip <= np; ++ip) {
      const int vt = pt[it], vp = pp[ip];
      int v = 0;
      if (vt > 0 && vph[vt] < 0.f) v = vt;
      else if (vt == vp || vth[vp] == vth[vt] || vph[vt] == vph[vp]) v = vt;
      tab[(size_t)it * (np + 1) + ip] = (uint8_t)v;
    }
  d.n_angle = na;
  d.n_theta = nt;
  d.n_phi = np;
  d.dtheta = dth;
  d.dphi = dph;
  return MC_OK;
}

// opac_row0 > 0: the opacity rows (frequency bins) below it are not copied:
// the caller guarantees no packet marches there (the non-ionising bins of a
// gas-only grid escape before any march).
// Device view of a pinned (page-locked, mapped) host pointer, or nullptr
// for pageable memory.
void *pinned_view(const void *h) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, h) != cudaSuccess) { cudaGetLastError(); return nullptr; }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

mc_status upload_arrays(mc_ctx *c, const mc_grid_t *g, bool first, cudaStream_t cdf_stream = nullptr,
                        int opac_row0 = 0) {
  const int nc1 = g->ncells + 1, nb = g->nbins;
  const size_t plane = (size_t)nc1 * nb * sizeof(float);
  cudaStream_t s = c->stream;
  mc_status st;
  auto put = [&](DBuf &b, const void *h, size_t bytes) -> mc_status {
    if (h) c->xfer_h2d += (long long)bytes;
    if (first || !b.p) return upload(b, h, bytes, s);
    if (h) {
      cudaError_t e = cudaMemcpyAsync(b.p, h, bytes, cudaMemcpyHostToDevice, s);
      if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "H2D copy failed: %s", cudaGetErrorString(e));
    }
    return MC_OK;
  };
  if (!first && c->opacity.p && opac_row0 > 0 && opac_row0 < nb) {
    const size_t off = (size_t)opac_row0 * nc1 * sizeof(float);
    c->xfer_h2d += (long long)(plane - off);
    cudaError_t e = cudaMemcpyAsync((char *)c->opacity.p + off, (const char *)g->opacity + off, plane - off,
                                    cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "H2D copy failed: %s", cudaGetErrorString(e));
  } else if ((st = put(c->opacity, g->opacity, plane))) {
    return st;
  }
  if (g->sca_opac && (st = put(c->sca, g->sca_opac, plane))) return st;
  if (!c->identity) {
    const size_t mplane = (size_t)c->ncell3 * nb * sizeof(float);
    if (!c->opac_m.p) MC_CUDA(c->opac_m.alloc(mplane));
    MC_CUDA(mcg::launch_wave_expand(c->opacity.as<float>(), c->opac_m.as<float>(), c->lin2cell.as<int32_t>(),
                                    c->ncell3, nc1, nb, s));
    if (g->sca_opac) {
      if (!c->sca_m.p) MC_CUDA(c->sca_m.alloc(mplane));
      MC_CUDA(mcg::launch_wave_expand(c->sca.as<float>(), c->sca_m.as<float>(), c->lin2cell.as<int32_t>(),
                                      c->ncell3, nc1, nb, s));
    }
  }
  if (g->total_lines && (st = put(c->tlines, g->total_lines, (size_t)nc1 * sizeof(float)))) return st;
  if (g->g_sca && (st = put(c->gsca, g->g_sca, (size_t)nb * sizeof(float)))) return st;
  if (g->rec_pdf) {
    const cudaStream_t cs = cdf_stream ? cdf_stream : s;
    if (cs != s && c->ev_side0) {
      // the recPDF copy starts once the opacity rows are up: round 0 needs
      // them, and the two copies would share the host link
      MC_CUDA(cudaEventRecord(c->ev_side0, s));
      MC_CUDA(cudaStreamWaitEvent(cs, c->ev_side0, 0));
    }
    c->xfer_h2d += (long long)plane;
    if (first || !c->rec_raw.p) {
      if ((st = upload(c->rec_raw, g->rec_pdf, plane, cs))) return st;
    } else {
      cudaError_t e = cudaMemcpyAsync(c->rec_raw.p, g->rec_pdf, plane, cudaMemcpyHostToDevice, cs);
      if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "H2D copy failed: %s", cudaGetErrorString(e));
    }
    if (!c->rec_cdf.p) MC_CUDA(c->rec_cdf.alloc(plane));
    MC_CUDA(mcg::launch_cdf_transpose(c->rec_raw.as<float>(), c->rec_cdf.as<float>(), nc1, nb, cs));
  }
  if (g->dust_pdf) {
    if ((st = put(c->dust_raw, g->dust_pdf, plane))) return st;
    if (!c->dust_cdf.p) MC_CUDA(c->dust_cdf.alloc(plane));
    MC_CUDA(mcg::launch_cdf_transpose(c->dust_raw.as<float>(), c->dust_cdf.as<float>(), nc1, nb, s));
  }
  if (g->n_angle > 0) {
    std::vector<uint8_t> tab;
    if ((st = view_table(g, c->g, tab))) return st;
    if (c->view.bytes != tab.size()) {
      if (c->view.p) { cudaFree(c->view.p); c->view.p = nullptr; c->view.bytes = 0; }
      MC_CUDA(c->view.alloc(tab.size()));
    }
    MC_CUDA(cudaMemcpyAsync(c->view.p, tab.data(), tab.size(), cudaMemcpyHostToDevice, s));
    MC_CUDA(cudaStreamSynchronize(s));  // the host table goes out of scope
    c->g.view = c->view.as<uint8_t>();
  } else {
    c->g.n_angle = 0;
  }
  return MC_OK;
}

mc_status make_sources(mc_ctx *c, const mc_source_t *src, int32_t nsrc, const mc_run_opts_t *o,
                       mcg::DevSources &S) {
  if (nsrc < 1 || nsrc > mcg::kMaxSources)
    return set_error(MC_ERR_ARG, "nsrc must be 1..%d (got %d)", mcg::kMaxSources, nsrc);
  std::vector<float> cdfs((size_t)nsrc * c->nb);
  S.nsrc = nsrc;
  S.nres = 0;
  long long base = 0;
  for (int i = 0; i < nsrc; ++i) {
    const mc_source_t &x = src[i];
    if (!x.spec_cdf) return set_error(MC_ERR_ARG, "source %d has no spec_cdf", i);
    if (x.n_packets < 0) return set_error(MC_ERR_ARG, "source %d has negative n_packets", i);
    if (x.cell[0] < 1 || x.cell[0] > c->nx || x.cell[1] < 1 || x.cell[1] > c->ny || x.cell[2] < 1 ||
        x.cell[2] > c->nz)
      return set_error(MC_ERR_BOUNDS, "source %d cell (%d,%d,%d) outside the grid", i, x.cell[0], x.cell[1],
                       x.cell[2]);
    float run = -INFINITY;  // running max: binary search == getNu2's scan
    for (int k = 0; k < c->nb; ++k) {
      run = std::fmax(run, x.spec_cdf[k]);
      cdfs[(size_t)i * c->nb + k] = run;
    }
    mcg::DevSource &d = S.s[i];
    d.cell[0] = x.cell[0]; d.cell[1] = x.cell[1]; d.cell[2] = x.cell[2];
    d.pos[0] = x.pos[0]; d.pos[1] = x.pos[1]; d.pos[2] = x.pos[2];
    d.delta_e = x.delta_e;
    d.k0 = (uint32_t)o->seed;
    d.k1 = (uint32_t)(o->seed >> 32) ^ ((o->iteration & 0xFFFFFFu) << 8) ^ ((uint32_t)x.istar & 0xFFu);
    d.n = x.n_packets;
    d.base = base;
    base += x.n_packets;
  }
  S.total = base;
  const size_t bytes = cdfs.size() * sizeof(float);
  if (c->src_cdf.bytes < bytes) {
    if (c->src_cdf.p) { cudaFree(c->src_cdf.p); c->src_cdf.p = nullptr; }
    MC_CUDA(c->src_cdf.alloc(bytes));
  }
  MC_CUDA(cudaMemcpyAsync(c->src_cdf.p, cdfs.data(), bytes, cudaMemcpyHostToDevice, c->stream));
  for (int i = 0; i < nsrc; ++i) S.s[i].cdf = c->src_cdf.as<float>() + (size_t)i * c->nb;
  return MC_OK;
}

double kernel_budget_ns() {
  const char *e = getenv("MC_KERNEL_BUDGET_S");
  double s = e ? atof(e) : 120.0;
  if (!(s > 0)) s = 120.0;
  return s * 1e9;
}

}  // namespace

extern "C" {

int mc_abi_version(void) { return MC_ABI_VERSION; }

const char *mc_last_error(void) { return g_last_error.c_str(); }

mc_status mc_ctx_create(const mc_grid_t *g, mc_ctx_t **out) {
  if (!out) return set_error(MC_ERR_ARG, "out is NULL");
  *out = nullptr;
  mc_status st = check_grid(g);
  if (st) return st;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return set_error(MC_ERR_NO_DEVICE, "no CUDA device");
  mc_ctx *c = new mc_ctx();
  auto fail = [&](mc_status s) { delete c; return s; };
  if (cudaGetDevice(&c->device) != cudaSuccess) return fail(set_error(MC_ERR_CUDA, "cudaGetDevice failed"));
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
  if (const char *rm = getenv("MC_REFILL_MIN")) c->refill_min = atoi(rm) > 0 ? atoi(rm) : 8;
  if (const char *is = getenv("MC_INNER_STEPS")) c->inner_steps = atoi(is) > 0 ? atoi(is) : 4;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess)
    return fail(set_error(MC_ERR_CUDA, "stream/event creation failed"));
  c->nx = g->nx; c->ny = g->ny; c->nz = g->nz; c->nc = g->ncells; c->nb = g->nbins; c->flags = g->flags;
  const bool sym = g->flags & MC_FLAG_SYMMETRIC_XYZ;
  const size_t n3 = (size_t)g->nx * g->ny * g->nz;
  if ((st = upload(c->xa, g->x_axis, g->nx * sizeof(float), c->stream)) ||
      (st = upload(c->ya, g->y_axis, g->ny * sizeof(float), c->stream)) ||
      (st = upload(c->za, g->z_axis, g->nz * sizeof(float), c->stream)) ||
      (st = upload(c->active, g->active, n3 * sizeof(int32_t), c->stream)) ||
      (st = upload(c->nu, g->nu_array, g->nbins * sizeof(float), c->stream)))
    return fail(st);
  std::vector<float> w32;
  std::vector<double> w64;
  const float *ax[3] = {g->x_axis, g->y_axis, g->z_axis};
  const int na[3] = {g->nx, g->ny, g->nz};
  DBuf *b32[3] = {&c->dx32, &c->dy32, &c->dz32};
  DBuf *b64[3] = {&c->dx64, &c->dy64, &c->dz64};
  for (int k = 0; k < 3; ++k) {
    widths<float>(ax[k], na[k], sym, w32);
    widths<double>(ax[k], na[k], sym, w64);
    if ((st = upload(*b32[k], w32.data(), w32.size() * sizeof(float), c->stream))) return fail(st);
    if ((st = upload(*b64[k], w64.data(), w64.size() * sizeof(double), c->stream))) return fail(st);
    // the host vectors are reused: finish the copy first
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return fail(set_error(MC_ERR_CUDA, "sync failed"));
  }
  {
    // march order lin = (z-1) + nz*((y-1) + ny*(x-1)) -> active value
    c->ncell3 = (long long)g->nx * g->ny * g->nz;
    std::vector<int32_t> l2c((size_t)c->ncell3);
    c->identity = 1;
    for (int x = 1; x <= g->nx; ++x)
      for (int y = 1; y <= g->ny; ++y)
        for (int z = 1; z <= g->nz; ++z) {
          const long long lin = (z - 1) + (long long)g->nz * ((y - 1) + (long long)g->ny * (x - 1));
          const int a = g->active[(x - 1) + (long long)g->nx * ((y - 1) + (long long)g->ny * (z - 1))];
          l2c[lin] = a;
          if (a != lin + 1) c->identity = 0;
        }
    if ((st = upload(c->lin2cell, l2c.data(), l2c.size() * sizeof(int32_t), c->stream))) return fail(st);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return fail(set_error(MC_ERR_CUDA, "sync failed"));
    if (cudaEventCreate(&c->evm0) != cudaSuccess || cudaEventCreate(&c->evm1) != cudaSuccess)
      return fail(set_error(MC_ERR_CUDA, "event creation failed"));
    if (c->bins.alloc((size_t)g->nbins * 2 * sizeof(unsigned int) + 32) != cudaSuccess)
      return fail(set_error(MC_ERR_NOMEM, "bins"));
  }
  if ((st = upload_arrays(c, g, true))) return fail(st);
  c->n_angle = g->n_angle;
  const size_t nj = (size_t)(g->ncells + 1) * g->nbins;
  const size_t ne = (size_t)(g->ncells + 1) * (g->nbins + 1) * (g->n_angle + 1);
  if (c->jste.alloc(nj * sizeof(double)) != cudaSuccess) return fail(set_error(MC_ERR_NOMEM, "Jste alloc"));
  if ((g->flags & MC_FLAG_DEBUG) && c->jdif.alloc(nj * sizeof(double)) != cudaSuccess)
    return fail(set_error(MC_ERR_NOMEM, "Jdif alloc"));
  if (c->esc.alloc(ne * sizeof(double)) != cudaSuccess) return fail(set_error(MC_ERR_NOMEM, "escaped alloc"));
  if (!c->identity) {
    const size_t nm = (size_t)c->ncell3 * g->nbins * sizeof(double);
    if (c->jste_m.alloc(nm) != cudaSuccess) return fail(set_error(MC_ERR_NOMEM, "march Jste alloc"));
    if ((g->flags & MC_FLAG_DEBUG) && c->jdif_m.alloc(nm) != cudaSuccess)
      return fail(set_error(MC_ERR_NOMEM, "march Jdif alloc"));
  }
  if (c->counters.alloc(sizeof(mcg::DevCounters)) != cudaSuccess) return fail(set_error(MC_ERR_NOMEM, "counters"));

  mcg::DevGrid &d = c->g;
  d.nx = g->nx; d.ny = g->ny; d.nz = g->nz; d.nc = g->ncells; d.nb = g->nbins;
  d.xa = c->xa.as<float>(); d.ya = c->ya.as<float>(); d.za = c->za.as<float>();
  d.active = c->active.as<int32_t>();
  d.opacity = c->opacity.as<float>();
  d.sca = c->sca.as<float>();
  d.rec_cdf = c->rec_cdf.as<float>();
  d.dust_cdf = c->dust_cdf.as<float>();
  d.total_lines = c->tlines.as<float>();
  d.nu = c->nu.as<float>();
  d.gsca = c->gsca.as<float>();
  d.dx32 = c->dx32.as<float>(); d.dy32 = c->dy32.as<float>(); d.dz32 = c->dz32.as<float>();
  d.dx64 = c->dx64.as<double>(); d.dy64 = c->dy64.as<double>(); d.dz64 = c->dz64.as<double>();
  d.gc[0] = g->geo_corr[0]; d.gc[1] = g->geo_corr[1]; d.gc[2] = g->geo_corr[2];
  d.rout = g->r_out;
  d.ion_edge1 = g->ion_edge1;
  d.flags = g->flags;
  d.jste = c->jste.as<double>();
  d.jdif = c->jdif.as<double>();
  d.esc = c->esc.as<double>();
  mc_status z = mc_ctx_zero(c);
  if (z) return fail(z);
  if (cudaStreamSynchronize(c->stream) != cudaSuccess)
    return fail(set_error(MC_ERR_CUDA, "upload failed: %s", cudaGetErrorString(cudaGetLastError())));
  *out = c;
  return MC_OK;
}


namespace {

// Re-uploads the geometry of a grid of the context's shape (axes, active,
// frequencies, cell widths, march order).  Returns MC_ERR_ARG when the
// active map changes which cells are active in a way that changes the march
// layout (the caller then builds a new context).
// true when g's axes, active map and frequencies equal the ones the last
// drop-in call left in the context (and records them otherwise)
bool same_geometry(mc_ctx *c, const mc_grid_t *g) {
  const size_t nf = (size_t)g->nx + g->ny + g->nz + g->nbins;
  const size_t n3 = (size_t)g->nx * g->ny * g->nz;
  bool same = c->geo_f.size() == nf && c->geo_a.size() == n3;
  const float *parts[4] = {g->x_axis, g->y_axis, g->z_axis, g->nu_array};
  const size_t lens[4] = {(size_t)g->nx, (size_t)g->ny, (size_t)g->nz, (size_t)g->nbins};
  if (same) {
    size_t o = 0;
    for (int k = 0; k < 4 && same; o += lens[k], ++k)
      same = memcmp(c->geo_f.data() + o, parts[k], lens[k] * sizeof(float)) == 0;
    same = same && memcmp(c->geo_a.data(), g->active, n3 * sizeof(int32_t)) == 0;
  }
  if (!same) {
    c->geo_f.resize(nf);
    size_t o = 0;
    for (int k = 0; k < 4; o += lens[k], ++k) memcpy(c->geo_f.data() + o, parts[k], lens[k] * sizeof(float));
    c->geo_a.assign(g->active, g->active + n3);
  }
  return same;
}

mc_status refresh_geometry(mc_ctx *c, const mc_grid_t *g) {
  const bool sym = g->flags & MC_FLAG_SYMMETRIC_XYZ;
  const size_t n3 = (size_t)g->nx * g->ny * g->nz;
  std::vector<int32_t> l2c(n3);
  int identity = 1;
  for (int x = 1; x <= g->nx; ++x)
    for (int y = 1; y <= g->ny; ++y)
      for (int z = 1; z <= g->nz; ++z) {
        const long long lin = (z - 1) + (long long)g->nz * ((y - 1) + (long long)g->ny * (x - 1));
        const int a = g->active[(x - 1) + (long long)g->nx * ((y - 1) + (long long)g->ny * (z - 1))];
        l2c[lin] = a;
        if (a != lin + 1) identity = 0;
      }
  if (identity != c->identity) return set_error(MC_ERR_ARG, "march layout changed");
  cudaStream_t s = c->stream;
  MC_CUDA(cudaMemcpyAsync(c->xa.p, g->x_axis, g->nx * sizeof(float), cudaMemcpyHostToDevice, s));
  MC_CUDA(cudaMemcpyAsync(c->ya.p, g->y_axis, g->ny * sizeof(float), cudaMemcpyHostToDevice, s));
  MC_CUDA(cudaMemcpyAsync(c->za.p, g->z_axis, g->nz * sizeof(float), cudaMemcpyHostToDevice, s));
  MC_CUDA(cudaMemcpyAsync(c->active.p, g->active, n3 * sizeof(int32_t), cudaMemcpyHostToDevice, s));
  MC_CUDA(cudaMemcpyAsync(c->nu.p, g->nu_array, g->nbins * sizeof(float), cudaMemcpyHostToDevice, s));
  MC_CUDA(cudaMemcpyAsync(c->lin2cell.p, l2c.data(), n3 * sizeof(int32_t), cudaMemcpyHostToDevice, s));
  c->xfer_h2d += (long long)((g->nx + g->ny + g->nz) * (sizeof(float) * 2 + sizeof(double)) + 2 * n3 * sizeof(int32_t) +
                             g->nbins * sizeof(float));
  std::vector<float> w32[3];
  std::vector<double> w64[3];
  const float *ax[3] = {g->x_axis, g->y_axis, g->z_axis};
  const int na[3] = {g->nx, g->ny, g->nz};
  DBuf *b32[3] = {&c->dx32, &c->dy32, &c->dz32};
  DBuf *b64[3] = {&c->dx64, &c->dy64, &c->dz64};
  for (int k = 0; k < 3; ++k) {
    widths<float>(ax[k], na[k], sym, w32[k]);
    widths<double>(ax[k], na[k], sym, w64[k]);
    MC_CUDA(cudaMemcpyAsync(b32[k]->p, w32[k].data(), na[k] * sizeof(float), cudaMemcpyHostToDevice, s));
    MC_CUDA(cudaMemcpyAsync(b64[k]->p, w64[k].data(), na[k] * sizeof(double), cudaMemcpyHostToDevice, s));
  }
  MC_CUDA(cudaStreamSynchronize(s));  // the host vectors go out of scope
  c->g.gc[0] = g->geo_corr[0]; c->g.gc[1] = g->geo_corr[1]; c->g.gc[2] = g->geo_corr[2];
  c->g.rout = g->r_out;
  c->g.ion_edge1 = g->ion_edge1;
  return MC_OK;
}

// The context kept by mc_transport_run between calls (one host thread drives
// the library, so a single cache suffices).
std::mutex g_cache_mutex;
mc_ctx *g_cached = nullptr;

}  // namespace

mc_status mc_ctx_update(mc_ctx_t *c, const mc_grid_t *g) {
  if (!c) return set_error(MC_ERR_ARG, "ctx is NULL");
  mc_status st = check_grid(g);
  if (st) return st;
  if (g->nx != c->nx || g->ny != c->ny || g->nz != c->nz || g->ncells != c->nc || g->nbins != c->nb ||
      g->flags != c->flags || g->n_angle != c->n_angle)
    return set_error(MC_ERR_ARG, "grid shape/flags differ from the context's");
  if ((st = upload_arrays(c, g, false))) return st;
  MC_CUDA(cudaStreamSynchronize(c->stream));
  return MC_OK;
}

mc_status mc_ctx_zero(mc_ctx_t *c) {
  if (!c) return set_error(MC_ERR_ARG, "ctx is NULL");
  MC_CUDA(cudaMemsetAsync(c->jste.p, 0, c->jste.bytes, c->stream));
  if (c->jdif.p) MC_CUDA(cudaMemsetAsync(c->jdif.p, 0, c->jdif.bytes, c->stream));
  MC_CUDA(cudaMemsetAsync(c->esc.p, 0, c->esc.bytes, c->stream));
  return MC_OK;
}

namespace {

mc_status wave_buffers(mc_ctx_t *c, size_t n) {
  if (n <= c->queue_cap) return MC_OK;
  struct B { DBuf *b; size_t per; } bs[] = {
      {&c->s_nu, 2},     {&c->s_words, 4}, {&c->queue, 4},   {&c->q_id, 4},     {&c->q_cell, 4},
      {&c->q_words, 4},  {&c->q_meta, 4},  {&c->q_origin, 4}, {&c->q_r, 24},    {&c->q_v, 24},
      {&c->q_pass, 8},   {&c->a_id, 4},    {&c->a_cell, 4},  {&c->a_words, 4},  {&c->a_run, 2},
      {&c->a_r, 24}};
  for (auto &x : bs)
    if (x.b->p) { cudaFree(x.b->p); x.b->p = nullptr; x.b->bytes = 0; }
  for (auto &x : bs) MC_CUDA(x.b->alloc(n * x.per));
  c->queue_cap = n;
  return MC_OK;
}

mc_status wave_setup(mc_ctx_t *c, const mcg::DevGrid &g, const mcg::DevSources &S, const mcg::DevReplay &rp,
                     mcg::WaveLaunch &L) {
  if (S.total >= 0xFFFFFFFFll) return set_error(MC_ERR_ARG, "2^32-1 or more packets in one call");
  if (g.nb > 0xFFFF) return set_error(MC_ERR_UNSUPPORTED, "nbins above 65535");
  if (c->nx > 1023 || c->ny > 1023 || c->nz > 1023) return set_error(MC_ERR_UNSUPPORTED, "grid axes above 1023");
  const long long all = S.total + (S.nres > 0 ? (long long)S.nres * S.s[S.nsrc].n : 0);
  if (all >= 0xFFFFFFFFll) return set_error(MC_ERR_ARG, "2^32-1 or more packets in one call");
  mc_status st = wave_buffers(c, (size_t)all);
  if (st) return st;
  L.g = g;
  L.S = S;
  L.rp = rp;
  L.cnt = c->counters.as<mcg::DevCounters>();
  L.num_sms = c->num_sms;
  L.stream = c->stream;
  mcg::WaveGrid &w = L.w;
  w.identity = c->identity;
  if (c->identity) {
    w.opac = c->opacity.as<float>();
    w.sca = c->sca.as<float>();
    w.jste = c->jste.as<double>();
    w.jdif = c->jdif.as<double>();
    w.S = c->nc + 1;
    w.off = 1;
  } else {
    w.opac = c->opac_m.as<float>();
    w.sca = c->sca_m.as<float>();
    w.jste = c->jste_m.as<double>();
    w.jdif = c->jdif_m.as<double>();
    w.S = c->ncell3;
    w.off = 0;
    MC_CUDA(cudaMemsetAsync(c->jste_m.p, 0, c->jste_m.bytes, c->stream));
    if (c->jdif_m.p) MC_CUDA(cudaMemsetAsync(c->jdif_m.p, 0, c->jdif_m.bytes, c->stream));
  }
  w.lin2cell = c->lin2cell.as<int32_t>();
  w.refill_min = c->refill_min;
  w.inner_steps = c->inner_steps;
  w.s_nu = c->s_nu.as<uint16_t>();
  w.s_words = c->s_words.as<uint32_t>();
  w.bin_count = c->bins.as<unsigned int>();
  w.bin_cursor = w.bin_count + c->nb;
  w.qhead = (unsigned long long *)(((uintptr_t)(w.bin_cursor + c->nb) + 7) & ~(uintptr_t)7);
  w.a_count = (unsigned int *)(w.qhead + 1);
  w.queue = c->queue.as<uint32_t>();
  w.q_id = c->q_id.as<uint32_t>();
  w.q_cell = c->q_cell.as<uint32_t>();
  w.q_words = c->q_words.as<uint32_t>();
  w.q_meta = c->q_meta.as<uint32_t>();
  w.q_origin = c->q_origin.as<int32_t>();
  w.q_r = c->q_r.p;
  w.q_v = c->q_v.p;
  w.q_pass = c->q_pass.p;
  w.a_id = c->a_id.as<uint32_t>();
  w.a_cell = c->a_cell.as<uint32_t>();
  w.a_words = c->a_words.as<uint32_t>();
  w.a_run = c->a_run.as<uint16_t>();
  w.a_r = c->a_r.p;
  w.n_round = w.a_count + 1;
  w.round_ctr = (int *)(w.a_count + 2);
  return MC_OK;
}

// The chosen form with every round inside one CUDA graph: round 0 (stellar
// packets), then a WHILE node whose body is one re-emission round (sample,
// sort, emit, march) ending in wave_round_control_kernel, which sets the
// loop condition from the device's own absorbed count.  No host round trip
// between rounds.  The march is not timed on its own here.
mc_status run_wave_graph(mc_ctx_t *c, const mcg::DevGrid &g, const mcg::DevSources &S, const mcg::DevReplay &rp,
                         int precision, int *rounds_out) {
  mcg::WaveLaunch L{};
  mc_status st = wave_setup(c, g, S, rp, L);
  if (st) return st;
  const bool f64 = precision == MC_PREC_FP64;
  cudaStream_t s = c->stream;
  MC_CUDA(cudaMemsetAsync(L.w.round_ctr, 0, sizeof(int), s));
  // two graphs: round 0 (stellar packets only), then the round control and a
  // WHILE node over the re-emission rounds; a pending recPDF upload of the
  // drop-in call is waited for between them
  cudaGraph_t g0 = nullptr, graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  auto fail = [&](cudaError_t e, const char *what) {
    if (g0) cudaGraphDestroy(g0);
    if (graph) cudaGraphDestroy(graph);
    return set_error(MC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  };
  cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return fail(e, "capture failed");
  auto round0 = [&]() -> cudaError_t {
    cudaError_t r = cudaMemsetAsync(c->bins.p, 0, (size_t)c->nb * 2 * sizeof(unsigned int), s);
    if (r == cudaSuccess) r = f64 ? mcg::launch_wave_sample_stellar_fp64(L) : mcg::launch_wave_sample_stellar_fp32(L);
    if (r == cudaSuccess) r = mcg::launch_wave_sort(L, (unsigned int)S.total);
    if (r == cudaSuccess) r = f64 ? mcg::launch_wave_emit_fp64(L, 0) : mcg::launch_wave_emit_fp32(L, 0);
    if (r == cudaSuccess) r = f64 ? mcg::launch_wave_march_fp64(L) : mcg::launch_wave_march_fp32(L);
    if (r == cudaSuccess && S.nres > 0)
      r = f64 ? mcg::launch_wave_res_inject_fp64(L, c->res_cells.as<uint32_t>(), c->res_prefix.as<long long>(),
                                                 c->res_ncell)
              : mcg::launch_wave_res_inject_fp32(L, c->res_cells.as<uint32_t>(), c->res_prefix.as<long long>(),
                                                 c->res_ncell);
    return r;
  };
  cudaError_t ce = round0();
  e = cudaStreamEndCapture(s, &g0);
  if (ce != cudaSuccess) return fail(ce, "round 0 capture failed");
  if (e != cudaSuccess) return fail(e, "round 0 capture failed");
  e = cudaGraphCreate(&graph, 0);
  if (e != cudaSuccess) return fail(e, "graph creation failed");
  cudaGraphConditionalHandle handle;
  e = cudaGraphConditionalHandleCreate(&handle, graph, 0, cudaGraphCondAssignDefault);
  if (e != cudaSuccess) return fail(e, "conditional handle creation failed");
  // the condition for round 1, from round 0's absorbed count
  e = cudaStreamBeginCaptureToGraph(s, graph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return fail(e, "capture failed");
  ce = mcg::launch_wave_round_control(L, handle);
  cudaGraph_t captured = nullptr;
  e = cudaStreamEndCapture(s, &captured);
  if (ce != cudaSuccess) return fail(ce, "round control capture failed");
  if (e != cudaSuccess) return fail(e, "round control capture failed");
  cudaGraphNode_t last = nullptr;
  size_t nsink = 0;
  e = cudaGraphGetNodes(graph, nullptr, &nsink);
  std::vector<cudaGraphNode_t> nodes(nsink);
  if (e == cudaSuccess && nsink) e = cudaGraphGetNodes(graph, nodes.data(), &nsink);
  if (e != cudaSuccess || nsink != 1) return fail(e != cudaSuccess ? e : cudaErrorUnknown, "graph inspection failed");
  last = nodes[0];
  cudaGraphNodeParams cp{};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = handle;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t cond = nullptr;
  e = cudaGraphAddNode(&cond, graph, &last, nullptr, 1, &cp);
  if (e != cudaSuccess) return fail(e, "conditional node failed");
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  e = cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return fail(e, "body capture failed");
  auto round_k = [&]() -> cudaError_t {
    cudaError_t r = cudaMemsetAsync(c->bins.p, 0, (size_t)c->nb * 2 * sizeof(unsigned int), s);
    if (r == cudaSuccess)
      r = f64 ? mcg::launch_wave_sample_reemit_fp64(L, mcg::kDeviceCount)
              : mcg::launch_wave_sample_reemit_fp32(L, mcg::kDeviceCount);
    if (r == cudaSuccess) r = mcg::launch_wave_sort(L, mcg::kDeviceCount);
    if (r == cudaSuccess) r = f64 ? mcg::launch_wave_emit_fp64(L, 1) : mcg::launch_wave_emit_fp32(L, 1);
    if (r == cudaSuccess) r = f64 ? mcg::launch_wave_march_fp64(L) : mcg::launch_wave_march_fp32(L);
    if (r == cudaSuccess) r = mcg::launch_wave_round_control(L, handle);
    return r;
  };
  ce = round_k();
  cudaGraph_t cbody = nullptr;
  e = cudaStreamEndCapture(s, &cbody);
  if (ce != cudaSuccess) return fail(ce, "round capture failed");
  if (e != cudaSuccess) return fail(e, "round capture failed");
  cudaGraphExec_t exec0 = nullptr;
  e = cudaGraphInstantiate(&exec0, g0, 0);
  if (e != cudaSuccess) return fail(e, "graph instantiation failed");
  e = cudaGraphLaunch(exec0, s);
  cudaGraphExecDestroy(exec0);
  if (e != cudaSuccess) return fail(e, "graph launch failed");
  if (c->cdf_pending) {
    e = cudaStreamWaitEvent(s, c->ev_cdf, 0);
    c->cdf_pending = false;
    if (e != cudaSuccess) return fail(e, "event wait failed");
  }
  e = cudaGraphInstantiate(&exec, graph, 0);
  if (e != cudaSuccess) return fail(e, "graph instantiation failed");
  e = cudaGraphLaunch(exec, s);
  cudaGraphExecDestroy(exec);
  if (e != cudaSuccess) return fail(e, "graph launch failed");
  if (!c->identity) {
    MC_CUDA(mcg::launch_wave_fold(c->jste_m.as<double>(), c->jste.as<double>(), L.w.lin2cell, c->ncell3, c->nc + 1,
                                  c->nb, s));
    if (c->jdif_m.p)
      MC_CUDA(mcg::launch_wave_fold(c->jdif_m.as<double>(), c->jdif.as<double>(), L.w.lin2cell, c->ncell3,
                                    c->nc + 1, c->nb, s));
  }
  int rounds = 0;
  MC_CUDA(cudaMemcpyAsync(&rounds, L.w.round_ctr, sizeof(int), cudaMemcpyDeviceToHost, s));
  MC_CUDA(cudaStreamSynchronize(s));
  cudaGraphDestroy(g0);
  cudaGraphDestroy(graph);
  *rounds_out = rounds;
  return MC_OK;
}

mc_status run_wave(mc_ctx_t *c, const mcg::DevGrid &g, const mcg::DevSources &S, const mcg::DevReplay &rp,
                   int precision, float *march_ms, int *rounds_out) {
  mcg::WaveLaunch L{};
  mc_status st = wave_setup(c, g, S, rp, L);
  if (st) return st;
  mcg::WaveGrid &w = L.w;
  const bool f64 = precision == MC_PREC_FP64;
  unsigned int n_abs = 0;
  float total_ms = 0.f;
  int round = 0;
  for (;; ++round) {
    MC_CUDA(cudaMemsetAsync(c->bins.p, 0, (size_t)c->nb * 2 * sizeof(unsigned int), c->stream));
    cudaError_t e;
    if (round == 0) e = f64 ? mcg::launch_wave_sample_stellar_fp64(L) : mcg::launch_wave_sample_stellar_fp32(L);
    else e = f64 ? mcg::launch_wave_sample_reemit_fp64(L, n_abs) : mcg::launch_wave_sample_reemit_fp32(L, n_abs);
    if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "sample launch failed: %s", cudaGetErrorString(e));
    MC_CUDA(mcg::launch_wave_sort(L, round == 0 ? (unsigned int)S.total : n_abs));
    e = f64 ? mcg::launch_wave_emit_fp64(L, round) : mcg::launch_wave_emit_fp32(L, round);
    if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "emit launch failed: %s", cudaGetErrorString(e));
    MC_CUDA(cudaEventRecord(c->evm0, c->stream));
    e = f64 ? mcg::launch_wave_march_fp64(L) : mcg::launch_wave_march_fp32(L);
    if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "march launch failed: %s", cudaGetErrorString(e));
    MC_CUDA(cudaEventRecord(c->evm1, c->stream));
    if (round == 0 && S.nres > 0) {
      e = f64 ? mcg::launch_wave_res_inject_fp64(L, c->res_cells.as<uint32_t>(), c->res_prefix.as<long long>(),
                                                 c->res_ncell)
              : mcg::launch_wave_res_inject_fp32(L, c->res_cells.as<uint32_t>(), c->res_prefix.as<long long>(),
                                                 c->res_ncell);
      if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "resonance-line launch failed: %s", cudaGetErrorString(e));
    }
    struct { unsigned int a_count; int err; } hb{};
    MC_CUDA(cudaMemcpyAsync(&hb.a_count, w.a_count, sizeof(unsigned int), cudaMemcpyDeviceToHost, c->stream));
    MC_CUDA(cudaMemcpyAsync(&hb.err, &L.cnt->error_code, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    MC_CUDA(cudaStreamSynchronize(c->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->evm0, c->evm1);
    total_ms += ms;
    n_abs = hb.a_count;
    if (n_abs == 0 || hb.err != 0) break;
    if (round > g.recursion_limit + 1) return set_error(MC_ERR_BOUNDS, "re-emission rounds exceeded recursionLimit");
  }
  if (!c->identity) {
    MC_CUDA(mcg::launch_wave_fold(c->jste_m.as<double>(), c->jste.as<double>(), w.lin2cell, c->ncell3, c->nc + 1,
                                  c->nb, c->stream));
    if (c->jdif_m.p)
      MC_CUDA(mcg::launch_wave_fold(c->jdif_m.as<double>(), c->jdif.as<double>(), w.lin2cell, c->ncell3,
                                    c->nc + 1, c->nb, c->stream));
  }
  *march_ms = total_ms;
  *rounds_out = round + 1;
  return MC_OK;
}

}  // namespace

mc_status mc_ctx_run(mc_ctx_t *c, const mc_source_t *src, int32_t nsrc, const mc_run_opts_t *o,
                     mc_stats_t *stats) {
  NvtxRange nvtx_range("mc transport");
  if (!c || !src || !o) return set_error(MC_ERR_ARG, "ctx/src/opts is NULL");
  if (o->precision != MC_PREC_FP32 && o->precision != MC_PREC_FP64)
    return set_error(MC_ERR_ARG, "precision must be MC_PREC_FP32 or MC_PREC_FP64");
  if (o->rng != MC_RNG_PHILOX && o->rng != MC_RNG_REPLAY) return set_error(MC_ERR_ARG, "unknown rng");
  mcg::DevSources S{};
  mc_status st = make_sources(c, src, nsrc, o, S);
  if (st) return st;
  if (c->res_per_star > 0) {
    // a block of resonance-line packets after each star's (energyPacketDriver
    // :180-266), with the star's deltaE and its own draw stream
    if (o->rng != MC_RNG_PHILOX) return set_error(MC_ERR_UNSUPPORTED, "resonance-line packets draw from Philox only");
    if (o->run_flags & MC_RUN_FORM_PLAIN)
      return set_error(MC_ERR_UNSUPPORTED, "resonance-line packets need the wave form, not MC_RUN_FORM_PLAIN");
    if (2 * nsrc > mcg::kMaxSources)
      return set_error(MC_ERR_UNSUPPORTED, "resonance-line packets: at most %d sources", mcg::kMaxSources / 2);
    if (S.total < 1) return set_error(MC_ERR_ARG, "resonance-line packets need stellar packets in the call");
    S.nres = nsrc;
    for (int i = 0; i < nsrc; ++i) {
      mcg::DevSource &d = S.s[nsrc + i];
      d = S.s[i];
      d.k1 = (uint32_t)(o->seed >> 32) ^ ((o->iteration & 0xFFFFFFu) << 8) ^ ((uint32_t)(src[i].istar | 0x80) & 0xFFu);
      d.n = c->res_per_star;
      d.base = S.total + (long long)i * c->res_per_star;
    }
  }
  mcg::DevReplay rp{nullptr, 0};
  if (o->rng == MC_RNG_REPLAY) {
    if (!o->replay || o->replay_stride <= 0) return set_error(MC_ERR_ARG, "replay needs draws and a stride");
    const size_t bytes = (size_t)S.total * o->replay_stride * sizeof(double);
    if (c->replay.bytes < bytes) {
      if (c->replay.p) { cudaFree(c->replay.p); c->replay.p = nullptr; }
      MC_CUDA(c->replay.alloc(bytes));
    }
    MC_CUDA(cudaMemcpyAsync(c->replay.p, o->replay, bytes, cudaMemcpyHostToDevice, c->stream));
    rp.draws = c->replay.as<double>();
    rp.stride = o->replay_stride;
  }
  mcg::DevGrid g = c->g;
  g.recursion_limit = o->recursion_limit > 0 ? o->recursion_limit : 5000;
  g.safe_limit = o->safe_limit > 0 ? o->safe_limit : 500000;
  mcg::DevCounters h{};
  h.error_packet = -1;
  h.budget_ns = (unsigned long long)kernel_budget_ns();
  MC_CUDA(cudaEventRecord(c->ev0, c->stream));
  if (o->run_flags & MC_RUN_ZERO_FIRST) {
    mc_status z = mc_ctx_zero(c);
    if (z) return z;
  }
  MC_CUDA(cudaMemcpyAsync(c->counters.p, &h, sizeof h, cudaMemcpyHostToDevice, c->stream));
  const bool plain = o->run_flags & MC_RUN_FORM_PLAIN;
  float wave_ms = 0.f;
  // the graph form waits for a pending recPDF upload between round 0 and
  // round 1; the other forms before they start
  if (c->cdf_pending && !(S.total > 0 && !plain && (o->run_flags & MC_RUN_GRAPH))) {
    MC_CUDA(cudaStreamWaitEvent(c->stream, c->ev_cdf, 0));
    c->cdf_pending = false;
  }
  if (S.total > 0) {
    if (plain) {
      MC_CUDA(cudaEventRecord(c->evm0, c->stream));
      cudaError_t e = o->precision == MC_PREC_FP64
                          ? mcg::launch_plain_fp64(g, S, rp, c->counters.as<mcg::DevCounters>(), c->num_sms, c->stream)
                          : mcg::launch_plain_fp32(g, S, rp, c->counters.as<mcg::DevCounters>(), c->num_sms, c->stream);
      if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "transport launch failed: %s", cudaGetErrorString(e));
      MC_CUDA(cudaEventRecord(c->evm1, c->stream));
    } else {
      mc_status ws = (o->run_flags & MC_RUN_GRAPH) ? run_wave_graph(c, g, S, rp, o->precision, &c->rounds)
                                                    : run_wave(c, g, S, rp, o->precision, &wave_ms, &c->rounds);
      if (ws) return ws;
    }
  } else {
    MC_CUDA(cudaEventRecord(c->evm0, c->stream));
    MC_CUDA(cudaEventRecord(c->evm1, c->stream));
  }
  MC_CUDA(cudaEventRecord(c->ev1, c->stream));
  MC_CUDA(cudaMemcpyAsync(&h, c->counters.p, sizeof h, cudaMemcpyDeviceToHost, c->stream));

  MC_CUDA(cudaStreamSynchronize(c->stream));
  float ms = 0.f, mms = 0.f;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  if (plain || S.total == 0) cudaEventElapsedTime(&mms, c->evm0, c->evm1);
  else mms = wave_ms;
  if (stats) {
    stats->crossings = (int64_t)h.crossings;
    stats->absorptions = (int64_t)h.absorptions;
    stats->scatterings = (int64_t)h.scatterings;
    stats->escaped = (int64_t)h.escaped;
    stats->lines = (int64_t)h.lines;
    stats->trapped = (int64_t)h.trapped;
    stats->silent_exits = (int64_t)h.silent;
    stats->safe_limit_hits = (int64_t)h.safe_hits;
    stats->qphot = h.qphot;
    stats->kernel_ms = ms;
    stats->error_code = h.error_code;
    stats->error_packet = h.error_packet;
    stats->march_ms = mms;
    stats->rounds = plain ? 1 : c->rounds;
    stats->h2d_bytes = 0;
    stats->d2h_bytes = 0;
  }
  if (h.error_code != 0)
    return set_error((mc_status)h.error_code, "device error %d in packet %d", h.error_code, h.error_packet);
  return MC_OK;
}

mc_status mc_batch_run(mc_ctx_t *const *ctxs, int32_t n, const mc_source_t *const *srcs, const int32_t *nsrcs,
                       const mc_run_opts_t *opts, mc_stats_t *stats) {
  NvtxRange nvtx_range("mc batch transport");
  if (!ctxs || !srcs || !nsrcs || !opts) return set_error(MC_ERR_ARG, "ctxs/srcs/nsrcs/opts is NULL");
  if (n < 1 || n > 4096) return set_error(MC_ERR_ARG, "1..4096 models per batch");
  const int prec = opts[0].precision;
  if (prec != MC_PREC_FP32 && prec != MC_PREC_FP64) return set_error(MC_ERR_ARG, "precision must be MC_PREC_FP32 or MC_PREC_FP64");
  const bool f64 = prec == MC_PREC_FP64;
  mc_ctx_t *c0 = ctxs[0];
  if (!c0) return set_error(MC_ERR_ARG, "ctxs[0] is NULL");
  struct Model {
    mc_ctx_t *c;
    mcg::WaveLaunch L;
    mcg::DevCounters h;
    unsigned int n_round;
    bool live;
    int rounds;
  };
  std::vector<Model> M((size_t)n);
  const bool dust = c0->flags & MC_FLAG_DUST;
  for (int i = 0; i < n; ++i) {  // every argument is checked before any model is touched
    mc_ctx_t *c = ctxs[i];
    const mc_run_opts_t *o = opts + i;
    if (!c || !srcs[i]) return set_error(MC_ERR_ARG, "model %d: ctx/src is NULL", i);
    if (o->precision != prec) return set_error(MC_ERR_ARG, "model %d: one precision per batch", i);
    if (o->rng != MC_RNG_PHILOX) return set_error(MC_ERR_UNSUPPORTED, "model %d: a batch draws from Philox only", i);
    if (c->device != c0->device) return set_error(MC_ERR_ARG, "model %d: contexts of one device only", i);
    if ((bool)(c->flags & MC_FLAG_DUST) != dust) return set_error(MC_ERR_UNSUPPORTED, "model %d: gas and dusty grids in one batch", i);
    for (int j = 0; j < i; ++j)
      if (ctxs[j] == c) return set_error(MC_ERR_ARG, "model %d: context given twice", i);
  }
  for (int i = 0; i < n; ++i) {
    mc_ctx_t *c = ctxs[i];
    const mc_run_opts_t *o = opts + i;
    mcg::DevSources S{};
    mc_status st = make_sources(c, srcs[i], nsrcs[i], o, S);
    if (st) return st;
    mcg::DevGrid g = c->g;
    g.recursion_limit = o->recursion_limit > 0 ? o->recursion_limit : 5000;
    g.safe_limit = o->safe_limit > 0 ? o->safe_limit : 500000;
    Model &m = M[(size_t)i];
    m.c = c;
    m.h = mcg::DevCounters{};
    m.h.error_packet = -1;
    m.h.budget_ns = (unsigned long long)kernel_budget_ns();
    MC_CUDA(cudaEventRecord(c->ev0, c->stream));
    if (o->run_flags & MC_RUN_ZERO_FIRST) {
      mc_status z = mc_ctx_zero(c);
      if (z) return z;
    }
    MC_CUDA(cudaMemcpyAsync(c->counters.p, &m.h, sizeof m.h, cudaMemcpyHostToDevice, c->stream));
    if (c->cdf_pending) {
      MC_CUDA(cudaStreamWaitEvent(c->stream, c->ev_cdf, 0));
      c->cdf_pending = false;
    }
    st = wave_setup(c, g, S, mcg::DevReplay{nullptr, 0}, m.L);
    if (st) return st;
    m.n_round = (unsigned int)S.total;
    m.live = S.total > 0;
    m.rounds = 0;
  }
  // descriptors of the round's live models, then the task counter
  const size_t desc_bytes = ((size_t)n * sizeof(mcg::BatchModel) + 15) & ~(size_t)15;
  if (c0->batch_desc.bytes < desc_bytes + 16) {
    if (c0->batch_desc.p) { cudaFree(c0->batch_desc.p); c0->batch_desc.p = nullptr; c0->batch_desc.bytes = 0; }
    MC_CUDA(c0->batch_desc.alloc(desc_bytes + 16));
  }
  mcg::BatchModel *d_models = c0->batch_desc.as<mcg::BatchModel>();
  unsigned int *d_task = (unsigned int *)((char *)c0->batch_desc.p + desc_bytes);
  std::vector<mcg::BatchModel> hm;
  float march_ms = 0.f;
  for (int round = 0;; ++round) {
    unsigned long long total = 0;
    size_t smem = 0;
    hm.clear();
    for (auto &m : M) {
      if (!m.live) continue;
      mc_ctx_t *c = m.c;
      MC_CUDA(cudaMemsetAsync(c->bins.p, 0, (size_t)c->nb * 2 * sizeof(unsigned int), c->stream));
      cudaError_t e;
      if (round == 0) e = f64 ? mcg::launch_wave_sample_stellar_fp64(m.L) : mcg::launch_wave_sample_stellar_fp32(m.L);
      else e = f64 ? mcg::launch_wave_sample_reemit_fp64(m.L, m.n_round) : mcg::launch_wave_sample_reemit_fp32(m.L, m.n_round);
      if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "sample launch failed: %s", cudaGetErrorString(e));
      MC_CUDA(mcg::launch_wave_sort(m.L, m.n_round));
      e = f64 ? mcg::launch_wave_emit_fp64(m.L, round) : mcg::launch_wave_emit_fp32(m.L, round);
      if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "emit launch failed: %s", cudaGetErrorString(e));
      if (c != c0) {
        MC_CUDA(cudaEventRecord(c->evm0, c->stream));
        MC_CUDA(cudaStreamWaitEvent(c0->stream, c->evm0, 0));
      }
      total += m.n_round;
      const size_t sh = f64 ? mcg::march_batch_smem_fp64(c->nx, c->ny, c->nz) : mcg::march_batch_smem_fp32(c->nx, c->ny, c->nz);
      smem = sh > smem ? sh : smem;
      mcg::BatchModel b{};
      b.g = m.L.g;
      b.S = m.L.S;
      b.w = m.L.w;
      b.cnt = m.L.cnt;
      hm.push_back(b);
      ++m.rounds;
    }
    if (hm.empty()) break;
    int blocks = 0;
    MC_CUDA(f64 ? mcg::launch_wave_march_batch_blocks_fp64(dust, smem, c0->num_sms, &blocks)
                : mcg::launch_wave_march_batch_blocks_fp32(dust, smem, c0->num_sms, &blocks));
    // each model's share of one pass of tasks follows its packets
    unsigned int end = 0;
    size_t k = 0;
    for (auto &m : M) {
      if (!m.live) continue;
      const double share = (double)blocks * (double)m.n_round / (double)(total ? total : 1);
      const unsigned int t = share < 1.0 ? 1u : (unsigned int)(share + 0.5);
      end += t;
      hm[k++].task_end = end;
    }
    MC_CUDA(cudaMemcpyAsync(d_models, hm.data(), hm.size() * sizeof(mcg::BatchModel), cudaMemcpyHostToDevice, c0->stream));
    MC_CUDA(cudaMemsetAsync(d_task, 0, sizeof(unsigned int), c0->stream));
    mcg::BatchLaunch B{d_models, (int)hm.size(), end, d_task, smem, blocks, dust, c0->stream};
    MC_CUDA(cudaEventRecord(c0->evm0, c0->stream));
    cudaError_t e = f64 ? mcg::launch_wave_march_batch_fp64(B) : mcg::launch_wave_march_batch_fp32(B);
    if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "batched march launch failed: %s", cudaGetErrorString(e));
    MC_CUDA(cudaEventRecord(c0->evm1, c0->stream));
    std::vector<unsigned int> hcount(M.size(), 0u);
    std::vector<int> herr(M.size(), 0);
    for (size_t i = 0; i < M.size(); ++i) {
      Model &m = M[i];
      if (!m.live) continue;
      if (m.c != c0) MC_CUDA(cudaStreamWaitEvent(m.c->stream, c0->evm1, 0));
      MC_CUDA(cudaMemcpyAsync(&hcount[i], m.L.w.a_count, sizeof(unsigned int), cudaMemcpyDeviceToHost, m.c->stream));
      MC_CUDA(cudaMemcpyAsync(&herr[i], &m.L.cnt->error_code, sizeof(int), cudaMemcpyDeviceToHost, m.c->stream));
    }
    for (auto &m : M)
      if (m.live) MC_CUDA(cudaStreamSynchronize(m.c->stream));
    MC_CUDA(cudaStreamSynchronize(c0->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c0->evm0, c0->evm1);
    march_ms += ms;
    for (size_t i = 0; i < M.size(); ++i) {
      Model &m = M[i];
      if (!m.live) continue;
      m.n_round = hcount[i];
      if (m.n_round == 0 || herr[i] != 0) m.live = false;
      else if (round > m.L.g.recursion_limit + 1)
        return set_error(MC_ERR_BOUNDS, "model %d: re-emission rounds exceeded recursionLimit", (int)i);
    }
  }
  mc_status first = MC_OK;
  for (size_t i = 0; i < M.size(); ++i) {
    Model &m = M[i];
    mc_ctx_t *c = m.c;
    if (!c->identity && m.rounds > 0) {
      MC_CUDA(mcg::launch_wave_fold(c->jste_m.as<double>(), c->jste.as<double>(), m.L.w.lin2cell, c->ncell3, c->nc + 1,
                                    c->nb, c->stream));
      if (c->jdif_m.p)
        MC_CUDA(mcg::launch_wave_fold(c->jdif_m.as<double>(), c->jdif.as<double>(), m.L.w.lin2cell, c->ncell3,
                                      c->nc + 1, c->nb, c->stream));
    }
    MC_CUDA(cudaEventRecord(c->ev1, c->stream));
    MC_CUDA(cudaMemcpyAsync(&m.h, c->counters.p, sizeof m.h, cudaMemcpyDeviceToHost, c->stream));
    MC_CUDA(cudaStreamSynchronize(c->stream));
    c->rounds = m.rounds;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev0, c->ev1);
    if (stats) {
      mc_stats_t &t = stats[i];
      t.crossings = (int64_t)m.h.crossings;
      t.absorptions = (int64_t)m.h.absorptions;
      t.scatterings = (int64_t)m.h.scatterings;
      t.escaped = (int64_t)m.h.escaped;
      t.lines = (int64_t)m.h.lines;
      t.trapped = (int64_t)m.h.trapped;
      t.silent_exits = (int64_t)m.h.silent;
      t.safe_limit_hits = (int64_t)m.h.safe_hits;
      t.qphot = m.h.qphot;
      t.kernel_ms = ms;
      t.error_code = m.h.error_code;
      t.error_packet = m.h.error_packet;
      t.march_ms = march_ms;
      t.rounds = m.rounds;
      t.h2d_bytes = 0;
      t.d2h_bytes = 0;
    }
    if (m.h.error_code != 0 && first == MC_OK)
      first = set_error((mc_status)m.h.error_code, "model %d: device error %d in packet %d", (int)i, m.h.error_code,
                        m.h.error_packet);
  }
  return first;
}

mc_status mc_ctx_download(mc_ctx_t *c, double *jste, double *jdif, double *escaped, int32_t accumulate) {
  if (!c) return set_error(MC_ERR_ARG, "ctx is NULL");
  struct Item { double *h; DBuf *d; } items[3] = {{jste, &c->jste}, {jdif, &c->jdif}, {escaped, &c->esc}};
  for (auto &it : items) {
    if (!it.h || !it.d->p) continue;
    const size_t n = it.d->bytes / sizeof(double);
    if (!accumulate) {
      MC_CUDA(cudaMemcpyAsync(it.h, it.d->p, it.d->bytes, cudaMemcpyDeviceToHost, c->stream));
      MC_CUDA(cudaStreamSynchronize(c->stream));
    } else {
      std::vector<double> tmp(n);
      MC_CUDA(cudaMemcpyAsync(tmp.data(), it.d->p, it.d->bytes, cudaMemcpyDeviceToHost, c->stream));
      MC_CUDA(cudaStreamSynchronize(c->stream));
      for (size_t i = 0; i < n; ++i) it.h[i] += tmp[i];
    }
  }
  return MC_OK;
}

mc_status mc_ctx_device_estimators(mc_ctx_t *c, double **jste, double **jdif, double **escaped) {
  if (!c) return set_error(MC_ERR_ARG, "ctx is NULL");
  if (jste) *jste = c->jste.as<double>();
  if (jdif) *jdif = c->jdif.as<double>();
  if (escaped) *escaped = c->esc.as<double>();
  return MC_OK;
}

void mc_ctx_destroy(mc_ctx_t *c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->evm0) cudaEventDestroy(c->evm0);
  if (c->evm1) cudaEventDestroy(c->evm1);
  if (c->wave_exec) cudaGraphExecDestroy(c->wave_exec);
  if (c->side) cudaStreamSynchronize(c->side);
  if (c->ev_side0) cudaEventDestroy(c->ev_side0);
  if (c->ev_cdf) cudaEventDestroy(c->ev_cdf);
  if (c->ev_done) cudaEventDestroy(c->ev_done);
  if (c->side) cudaStreamDestroy(c->side);
  if (c->h_cnt) cudaFreeHost(c->h_cnt);
  cudaStream_t s = c->stream;
  delete c;  // frees the device buffers
  if (s) cudaStreamDestroy(s);
}

namespace {

mc_status opacity_device(int method, int nc1, int nspecies, int nb, const float *hden, const float *hxs,
                         const float *hff, float *dout, int num_sms, cudaStream_t s, double *kernel_ms) {
  if (nspecies < 1 || nspecies > 64) return set_error(MC_ERR_ARG, "nspecies must be 1..64 (got %d)", nspecies);
  if (method != MC_OPAC_FP32 && method != MC_OPAC_BF16X3) return set_error(MC_ERR_ARG, "unknown opacity method");
  if (!hden || !hxs || !dout || nc1 < 1 || nb < 1) return set_error(MC_ERR_ARG, "opacity: bad arguments");
  DBuf den, xs, ff, err;
  MC_CUDA(den.alloc((size_t)nspecies * nc1 * sizeof(float)));
  MC_CUDA(xs.alloc((size_t)nspecies * nb * sizeof(float)));
  MC_CUDA(err.alloc(sizeof(int)));
  MC_CUDA(cudaMemcpyAsync(den.p, hden, den.bytes, cudaMemcpyHostToDevice, s));
  MC_CUDA(cudaMemcpyAsync(xs.p, hxs, xs.bytes, cudaMemcpyHostToDevice, s));
  MC_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), s));
  if (hff) {
    MC_CUDA(ff.alloc((size_t)nc1 * sizeof(float)));
    MC_CUDA(cudaMemcpyAsync(ff.p, hff, ff.bytes, cudaMemcpyHostToDevice, s));
  }
  cudaEvent_t e0, e1;
  MC_CUDA(cudaEventCreate(&e0));
  MC_CUDA(cudaEventCreate(&e1));
  MC_CUDA(cudaEventRecord(e0, s));
  cudaError_t e = mcg::launch_opacity(method, nc1, nspecies, nb, den.as<float>(), xs.as<float>(),
                                      hff ? ff.as<float>() : nullptr, dout, err.as<int>(), num_sms, s);
  if (e != cudaSuccess) {
    cudaEventDestroy(e0); cudaEventDestroy(e1);
    return set_error(MC_ERR_CUDA, "opacity launch failed: %s", cudaGetErrorString(e));
  }
  MC_CUDA(cudaEventRecord(e1, s));
  int herr = 0;
  MC_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  MC_CUDA(cudaStreamSynchronize(s));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (kernel_ms) *kernel_ms = ms;
  if (herr) return set_error((mc_status)herr, "opacity kernel: tensor-core wait timed out");
  return MC_OK;
}

}  // namespace

extern "C" mc_status mc_opacity_build(int32_t ncells, int32_t nspecies, int32_t nbins, const float *den,
                                      const float *xs, const float *ff, int32_t method, float *opacity,
                                      double *kernel_ms) {
  if (!opacity) return set_error(MC_ERR_ARG, "opacity is NULL");
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return set_error(MC_ERR_NO_DEVICE, "no CUDA device");
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int nc1 = ncells + 1;
  DBuf out;
  MC_CUDA(out.alloc((size_t)nc1 * nbins * sizeof(float)));
  mc_status st = opacity_device(method, nc1, nspecies, nbins, den, xs, ff, out.as<float>(), sms, 0, kernel_ms);
  if (st) return st;
  MC_CUDA(cudaMemcpy(opacity, out.p, out.bytes, cudaMemcpyDeviceToHost));
  return MC_OK;
}

extern "C" mc_status mc_ctx_jste_moments(mc_ctx_t *c, int32_t nout, const float *w, double scale, float *out,
                                          double *kernel_ms) {
  NvtxRange nvtx_range("mc Jste moments");
  if (!c || !w || !out) return set_error(MC_ERR_ARG, "ctx, w and out are required");
  if (nout < 1 || nout > 128) return set_error(MC_ERR_ARG, "nout must be 1..128 (got %d)", nout);
  const int nc1 = c->nc + 1, nb = c->nb;
  DBuf dw, dout, err;
  MC_CUDA(dw.alloc((size_t)nb * nout * sizeof(float)));
  MC_CUDA(dout.alloc((size_t)nout * nc1 * sizeof(float)));
  MC_CUDA(err.alloc(sizeof(int)));
  cudaStream_t s = c->stream;
  MC_CUDA(cudaMemcpyAsync(dw.p, w, dw.bytes, cudaMemcpyHostToDevice, s));
  MC_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), s));
  MC_CUDA(cudaEventRecord(c->evm0, s));
  cudaError_t e = mcg::launch_jmoments(nc1, nb, nout, c->jste.as<double>(), dw.as<float>(), scale, dout.as<float>(),
                                       err.as<int>(), c->num_sms, s);
  if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "moment launch failed: %s", cudaGetErrorString(e));
  MC_CUDA(cudaEventRecord(c->evm1, s));
  int herr = 0;
  MC_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  MC_CUDA(cudaMemcpyAsync(out, dout.p, dout.bytes, cudaMemcpyDeviceToHost, s));
  MC_CUDA(cudaStreamSynchronize(s));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, c->evm0, c->evm1);
  if (kernel_ms) *kernel_ms = ms;
  if (herr) return set_error((mc_status)herr, "moment kernel: tensor-core wait timed out");
  return MC_OK;
}

extern "C" mc_status mc_ctx_dust_temperatures(mc_ctx_t *c, int32_t nsizes, const float *w_abs,
                                              const float *em_table, int32_t ntemps, const float *grain_weight,
                                              double scale, float *tdust, double *kernel_ms) {
  NvtxRange nvtx_range("mc grain temperatures");
  if (!c || !w_abs || !em_table || !grain_weight || !tdust)
    return set_error(MC_ERR_ARG, "ctx, w_abs, em_table, grain_weight and tdust are required");
  if (nsizes < 1 || nsizes > 127) return set_error(MC_ERR_ARG, "nsizes must be 1..127 (got %d)", nsizes);
  if (ntemps < 2) return set_error(MC_ERR_ARG, "ntemps must be >= 2");
  const int nc1 = c->nc + 1, nb = c->nb, nout = nsizes + 1;
  // gas and grains: the grain terms of the last update join the absorbed integrals
  const bool grains = c->g_ns > 0 && c->g_fresh && c->g_ns == nsizes;
  // column 0 = 1: the hit test of updateCell (any Jste > 0)
  std::vector<float> w((size_t)nb * nout);
  for (int i = 0; i < nb; ++i) {
    w[(size_t)i * nout] = 1.f;
    for (int k = 0; k < nsizes; ++k) w[(size_t)i * nout + 1 + k] = w_abs[(size_t)i * nsizes + k];
  }
  DBuf dw, dm, de, dg, err;
  DBuf &dt = c->d_tdust;
  if (dt.p && dt.bytes != (size_t)nout * nc1 * sizeof(float)) { cudaFree(dt.p); dt.p = nullptr; dt.bytes = 0; }
  MC_CUDA(dw.alloc(w.size() * sizeof(float)));
  MC_CUDA(dm.alloc((size_t)nout * nc1 * sizeof(float)));
  MC_CUDA(de.alloc((size_t)nsizes * ntemps * sizeof(float)));
  MC_CUDA(dg.alloc((size_t)nsizes * sizeof(float)));
  if (!dt.p) MC_CUDA(dt.alloc((size_t)nout * nc1 * sizeof(float)));
  c->d_nsizes = nsizes;
  // cell 0 (outside the grid) is never written by the kernel: it stays 0
  MC_CUDA(cudaMemsetAsync(dt.p, 0, dt.bytes, c->stream));
  MC_CUDA(err.alloc(sizeof(int)));
  cudaStream_t s = c->stream;
  MC_CUDA(cudaMemcpyAsync(dw.p, w.data(), dw.bytes, cudaMemcpyHostToDevice, s));
  MC_CUDA(cudaMemcpyAsync(de.p, em_table, de.bytes, cudaMemcpyHostToDevice, s));
  MC_CUDA(cudaMemcpyAsync(dg.p, grain_weight, dg.bytes, cudaMemcpyHostToDevice, s));
  MC_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), s));
  MC_CUDA(cudaEventRecord(c->evm0, s));
  cudaError_t e = mcg::launch_jmoments(nc1, nb, nout, c->jste.as<double>(), dw.as<float>(), scale, dm.as<float>(),
                                       err.as<int>(), c->num_sms, s);
  if (e == cudaSuccess)
    e = mcg::launch_dust_temperature(
        nc1, nsizes, ntemps, dm.as<float>() + nc1, de.as<float>(), dg.as<float>(), dm.as<float>(), dt.as<float>(),
        grains ? c->g_out.as<double>() + (size_t)2 * nsizes * nc1 : nullptr,
        grains ? c->g_out.as<double>() + (size_t)nsizes * nc1 : nullptr, c->num_sms, s);
  if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "dust temperature launch failed: %s", cudaGetErrorString(e));
  MC_CUDA(cudaEventRecord(c->evm1, s));
  int herr = 0;
  MC_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  MC_CUDA(cudaMemcpyAsync(tdust, dt.p, dt.bytes, cudaMemcpyDeviceToHost, s));
  MC_CUDA(cudaStreamSynchronize(s));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, c->evm0, c->evm1);
  if (kernel_ms) *kernel_ms = ms;
  if (herr) return set_error((mc_status)herr, "moment kernel: tensor-core wait timed out");
  return MC_OK;
}

extern "C" mc_status mc_ctx_build_opacity(mc_ctx_t *c, int32_t nspecies, const float *den, const float *xs,
                                          const float *ff, int32_t method, int32_t sca, double *kernel_ms) {
  if (!c) return set_error(MC_ERR_ARG, "ctx is NULL");
  DBuf &target = sca ? c->sca : c->opacity;
  if (!target.p) return set_error(MC_ERR_ARG, "the context has no %s table", sca ? "scaOpac" : "opacity");
  const int nc1 = c->nc + 1, nb = c->nb;
  mc_status st = opacity_device(method, nc1, nspecies, nb, den, xs, ff, target.as<float>(), c->num_sms, c->stream,
                                kernel_ms);
  if (st) return st;
  if (!c->identity) {
    DBuf &m = sca ? c->sca_m : c->opac_m;
    MC_CUDA(mcg::launch_wave_expand(target.as<float>(), m.as<float>(), c->lin2cell.as<int32_t>(), c->ncell3, nc1, nb,
                                    c->stream));
    MC_CUDA(cudaStreamSynchronize(c->stream));
  }
  return MC_OK;
}

// ---------------------------------------------------------------- cell update
namespace {

constexpr int kUZ[7] = {1, 2, 6, 7, 8, 10, 16};
constexpr int kUNL = 18, kUNT = 32;

mc_status put_buf(DBuf &b, const void *h, size_t bytes, cudaStream_t s) {
  if (b.p && b.bytes != bytes) { cudaFree(b.p); b.p = nullptr; b.bytes = 0; }
  if (!b.p) MC_CUDA(b.alloc(bytes));
  if (h && bytes) MC_CUDA(cudaMemcpyAsync(b.p, h, bytes, cudaMemcpyHostToDevice, s));
  return MC_OK;
}

// chex(elem, ion, 1:4) of ionBalance (update_mod.f90:1400-1460) for the
// benchmark elements
void chex_coeff(int z, int ion, double c[4]) {
  c[0] = c[1] = c[2] = c[3] = 0.;
  auto set = [&](double a, double b, double d, double e) { c[0] = a; c[1] = b; c[2] = d; c[3] = e; };
  switch (z * 100 + ion) {
    case 201: set(7.47e-6, 2.06, 9.93, -3.89); break;
    case 202: set(1.e-5, 0., 0., 0.); break;
    case 601: set(1.76e-9, 8.33, 4278.78, -6.41); break;
    case 602: set(1.67e-4, 2.79, 304.72, -4.07); break;
    case 603: set(3.25, 0.21, 0.19, -3.29); break;
    case 604: set(332.46, -0.11, -0.995, -1.58e-3); break;
    case 701: set(1.01e-3, -0.29, -0.92, -8.38); break;
    case 702: set(3.05e-1, 0.60, 2.65, -0.93); break;
    case 703: set(4.54, 0.57, -0.65, -0.89); break;
    case 704: set(3.28, 0.52, -0.52, -0.19); break;
    case 801: set(1.04, 3.15e-2, -0.61, -9.73); break;
    case 802: set(1.04, 0.27, 2.02, -5.92); break;
    case 803: set(3.98, 0.26, 0.56, -2.62); break;
    case 804: set(2.52e-1, 0.63, 2.08, -4.16); break;
    case 1002: set(1.e-5, 0., 0., 0.); break;
    case 1003: set(14.73, 4.52e-2, -0.84, -0.31); break;
    case 1004: set(6.47, 0.54, 3.59, -5.22); break;
    case 1601: set(3.82e-7, 11.10, 2.57e4, -8.22); break;
    case 1602: set(1.e-5, 0., 0., 0.); break;
    case 1603: set(2.29, 4.02e-2, 1.59, -6.06); break;
    case 1604: set(6.44, 0.13, 2.69, -5.69); break;
    default: break;
  }
  c[0] *= 1.e-9;
}

// g0 / g1 of getOuterShell (hydro_mod.f90:89-182) for z <= 20
double g0g1_of(int nElec) {
  static const int gl[30] = {2, 1, 2, 1, 6, 9, 4, 9, 6, 1, 2, 1, 6, 9, 4, 9, 6, 1, 2, 1,
                             10, 21, 28, 7, 6, 25, 28, 21, 2, 1};
  const int g0 = gl[nElec - 1], g1 = nElec == 1 ? 1 : gl[nElec - 2];
  return (double)g0 / (double)g1;
}

int elem_index(int z) {
  for (int e = 0; e < 7; ++e)
    if (kUZ[e] == z) return e;
  return -1;
}

}  // namespace

extern "C" mc_status mc_ctx_set_update_tables(mc_ctx_t *c, const mc_update_tables_t *t, const double *hden,
                                              const double *abund) {
  if (!c || !t || !hden || !abund) return set_error(MC_ERR_ARG, "ctx, tables, hden and abund are required");
  if (!t->rrec || !t->rnew || !t->direc || !t->aldro || t->ndirec < 0 || t->naldro < 0)
    return set_error(MC_ERR_ARG, "update tables: recombination data missing");
  if (t->ncel < 0 || t->ncel > 32) return set_error(MC_ERR_ARG, "update tables: ncel must be 0..32 (got %d)", t->ncel);
  cudaStream_t s = c->stream;
  std::vector<mcg::UpdIonDev> bal;
  int b = 0;
  for (int e = 0; e < 7; ++e) {
    const int z = kUZ[e], ni = std::min(z, 6);
    c->u_bal_z[e] = z;
    c->u_bal_first[e] = b;
    for (int ion = 1; ion <= ni; ++ion, ++b) {
      mcg::UpdIonDev d{};
      d.z = z; d.ion = ion; d.e = e; d.nelec = z - ion + 1;
      chex_coeff(z, ion, d.chex);
      d.dek = (z == 7 && ion == 1) ? 10863. : (z == 8 && ion == 1) ? 2205. : 0.;
      d.g0g1 = g0g1_of(d.nelec);
      // the dielectronic rows of (z, ion) and of (O, ion), in file order
      auto rows_for = [&](int zz, int *dr, int &ndr, int &ar) -> bool {
        ndr = 0;
        ar = -1;
        for (int i = 0; i < t->ndirec; ++i) {
          const int el = (int)t->direc[8 * i], n = (int)t->direc[8 * i + 1];
          if (el != zz || el + 1 - n != ion) continue;
          if (ndr == 4) return false;
          dr[ndr++] = i;
        }
        for (int i = 0; i < t->naldro; ++i) {
          const int el = (int)t->aldro[6 * i], n = (int)t->aldro[6 * i + 1];
          if (el == zz && el + 1 - n == ion) ar = i;
        }
        return true;
      };
      if (!rows_for(z, d.dr, d.ndr, d.ar) || !rows_for(8, d.dr8, d.ndr8, d.ar8))
        return set_error(MC_ERR_ARG, "update tables: more than 4 dielectronic rows for one ion");
      bal.push_back(d);
    }
  }
  const int ncel = t->ncel;
  std::vector<mcg::UpdCelDev> cel(ncel);
  std::vector<double> q2((size_t)std::max(ncel, 1) * kUNL * kUNL * kUNT, 0.);
  for (int k = 0; k < ncel; ++k) {
    mcg::UpdCelDev &d = cel[k];
    d.z = t->cel_key[2 * k];
    d.ion = t->cel_key[2 * k + 1];
    d.e = elem_index(d.z);
    d.nlev = t->cel_nlev[k];
    d.nt = t->cel_ntemp[k];
    if (d.e < 0 || d.ion < 1 || d.ion > std::min(d.z + 1, 7) || d.nlev < 1 || d.nlev > 17 || d.nt < 1 || d.nt > kUNT)
      return set_error(MC_ERR_ARG, "update tables: line ion %d (Z %d, ion %d, %d levels, %d temperatures) unusable", k,
                       d.z, d.ion, d.nlev, d.nt);
    d.br = t->cel_br[k];
    d.zz = t->cel_z[k];
    for (int i = 0; i < 4; ++i) d.ar[i] = t->cel_ar[4 * k + i];
    for (int i = 0; i < 5; ++i) d.ad[i] = t->cel_ad[5 * k + i];
    if (d.nt > 2) {
      const double *lt = t->cel_logt + (size_t)k * kUNT;
      for (int lo = 1; lo < d.nlev; ++lo)
        for (int hi = lo + 1; hi <= d.nlev; ++hi) {
          double y[kUNT];
          for (int it = 0; it < d.nt; ++it) y[it] = t->cel_qom[(((size_t)k * kUNT + it) * kUNL + lo) * kUNL + hi];
          mcg::spline_natural(lt, y, d.nt, &q2[(((size_t)k * kUNL + lo) * kUNL + hi) * kUNT]);
        }
    }
  }
  // collision strengths re-laid out [ion][lower][upper][T]
  std::vector<double> qq((size_t)std::max(ncel, 1) * kUNL * kUNL * kUNT, 0.);
  for (int k = 0; k < ncel; ++k)
    for (int it = 0; it < kUNT; ++it)
      for (int lo = 0; lo < kUNL; ++lo)
        for (int hi = 0; hi < kUNL; ++hi)
          qq[(((size_t)k * kUNL + lo) * kUNL + hi) * kUNT + it] = t->cel_qom[(((size_t)k * kUNT + it) * kUNL + lo) * kUNL + hi];
  const size_t nk = (size_t)std::max(ncel, 1);
  // float copies for the FP32 form
  auto tof = [](const double *p, size_t n) {
    std::vector<float> v(n);
    for (size_t i = 0; i < n; ++i) v[i] = p ? (float)p[i] : 0.f;
    return v;
  };
  std::vector<mcg::UpdIonT<float>> balf(bal.size());
  for (size_t i = 0; i < bal.size(); ++i) {
    const mcg::UpdIonDev &d = bal[i];
    mcg::UpdIonT<float> &f = balf[i];
    f.z = d.z; f.ion = d.ion; f.e = d.e; f.nelec = d.nelec;
    for (int j = 0; j < 4; ++j) { f.dr[j] = d.dr[j]; f.dr8[j] = d.dr8[j]; f.chex[j] = (float)d.chex[j]; }
    f.ndr = d.ndr; f.ar = d.ar; f.ndr8 = d.ndr8; f.ar8 = d.ar8;
    f.dek = (float)d.dek; f.g0g1 = (float)d.g0g1;
  }
  std::vector<mcg::UpdCelT<float>> celf(nk);
  for (int k = 0; k < ncel; ++k) {
    const mcg::UpdCelDev &d = cel[k];
    mcg::UpdCelT<float> &f = celf[k];
    f.z = d.z; f.ion = d.ion; f.e = d.e; f.nlev = d.nlev; f.nt = d.nt;
    f.br = (float)d.br; f.zz = (float)d.zz;
    for (int j = 0; j < 4; ++j) f.ar[j] = (float)d.ar[j];
    for (int j = 0; j < 5; ++j) f.ad[j] = (float)d.ad[j];
  }
  const std::vector<float> rrecf = tof(t->rrec, 2 * 31 * 31), rnewf = tof(t->rnew, 4 * 31 * 31),
                           direcf = tof(t->direc, (size_t)t->ndirec * 8), aldrof = tof(t->aldro, (size_t)t->naldro * 6),
                           logtf = tof(ncel ? t->cel_logt : nullptr, nk * kUNT),
                           gf = tof(ncel ? t->cel_g : nullptr, nk * kUNL), ef = tof(ncel ? t->cel_e : nullptr, nk * kUNL),
                           Af = tof(ncel ? t->cel_a : nullptr, nk * kUNL * kUNL), qqf = tof(qq.data(), qq.size()),
                           q2f = tof(q2.data(), q2.size()), abf = tof(abund, 7);
  mc_status st;
  if ((st = put_buf(c->f_bal, balf.data(), balf.size() * sizeof(balf[0]), s)) ||
      (st = put_buf(c->f_cel, celf.data(), nk * sizeof(celf[0]), s)) ||
      (st = put_buf(c->f_rrec, rrecf.data(), rrecf.size() * 4, s)) ||
      (st = put_buf(c->f_rnew, rnewf.data(), rnewf.size() * 4, s)) ||
      (st = put_buf(c->f_direc, direcf.data(), std::max<size_t>(direcf.size(), 1) * 4, s)) ||
      (st = put_buf(c->f_aldro, aldrof.data(), std::max<size_t>(aldrof.size(), 1) * 4, s)) ||
      (st = put_buf(c->f_logt, logtf.data(), logtf.size() * 4, s)) || (st = put_buf(c->f_g, gf.data(), gf.size() * 4, s)) ||
      (st = put_buf(c->f_e, ef.data(), ef.size() * 4, s)) || (st = put_buf(c->f_A, Af.data(), Af.size() * 4, s)) ||
      (st = put_buf(c->f_qq, qqf.data(), qqf.size() * 4, s)) || (st = put_buf(c->f_q2, q2f.data(), q2f.size() * 4, s)) ||
      (st = put_buf(c->f_ab, abf.data(), abf.size() * 4, s)))
    return st;
  if ((st = put_buf(c->u_bal, bal.data(), bal.size() * sizeof(mcg::UpdIonDev), s)) ||
      (st = put_buf(c->u_cel, cel.data(), nk * sizeof(mcg::UpdCelDev), s)) ||
      (st = put_buf(c->u_rrec, t->rrec, 2 * 31 * 31 * sizeof(double), s)) ||
      (st = put_buf(c->u_rnew, t->rnew, 4 * 31 * 31 * sizeof(double), s)) ||
      (st = put_buf(c->u_direc, t->direc, (size_t)std::max(t->ndirec, 1) * 8 * sizeof(double), s)) ||
      (st = put_buf(c->u_aldro, t->aldro, (size_t)std::max(t->naldro, 1) * 6 * sizeof(double), s)) ||
      (st = put_buf(c->u_logt, ncel ? t->cel_logt : nullptr, nk * kUNT * sizeof(double), s)) ||
      (st = put_buf(c->u_g, ncel ? t->cel_g : nullptr, nk * kUNL * sizeof(double), s)) ||
      (st = put_buf(c->u_e, ncel ? t->cel_e : nullptr, nk * kUNL * sizeof(double), s)) ||
      (st = put_buf(c->u_A, ncel ? t->cel_a : nullptr, nk * kUNL * kUNL * sizeof(double), s)) ||
      (st = put_buf(c->u_qq, qq.data(), qq.size() * sizeof(double), s)) ||
      (st = put_buf(c->u_q2, q2.data(), q2.size() * sizeof(double), s)) ||
      (st = put_buf(c->u_ab, abund, 7 * sizeof(double), s)) ||
      (st = put_buf(c->u_hden, hden, (size_t)(c->nc + 1) * sizeof(double), s)))
    return st;
  MC_CUDA(cudaStreamSynchronize(s));  // the host vectors go out of scope
  c->u_ncel = ncel;
  if (c->e_ok.p) MC_CUDA(cudaMemsetAsync(c->e_ok.p, 0, c->e_ok.bytes, s));  // other line ions
  c->u_maxlev = 1;
  for (int k = 0; k < ncel; ++k) c->u_maxlev = std::max(c->u_maxlev, (int)t->cel_nlev[k]);
  c->u_ndirec = t->ndirec;
  c->u_naldro = t->naldro;
  c->u_ready = true;
  return MC_OK;
}

extern "C" mc_status mc_ctx_set_cell_state(mc_ctx_t *c, const double *te, const double *ne, const double *X) {
  if (!c || !te || !ne || !X) return set_error(MC_ERR_ARG, "ctx, te, ne and ionden are required");
  const size_t nc1 = (size_t)c->nc + 1;
  cudaStream_t s = c->stream;
  mc_status st;
  if ((st = put_buf(c->s_te, te, nc1 * sizeof(double), s)) || (st = put_buf(c->s_ne, ne, nc1 * sizeof(double), s)) ||
      (st = put_buf(c->s_X, X, nc1 * 56 * sizeof(double), s)) || (st = put_buf(c->s_conv, nullptr, nc1 * 4, s)) ||
      (st = put_buf(c->s_niter, nullptr, nc1 * 4, s)) || (st = put_buf(c->s_flags, nullptr, nc1 * 4, s)) ||
      (st = put_buf(c->s_dte, nullptr, nc1 * sizeof(double), s)))
    return st;
  MC_CUDA(cudaMemsetAsync(c->s_conv.p, 0, c->s_conv.bytes, s));
  MC_CUDA(cudaMemsetAsync(c->s_niter.p, 0, c->s_niter.bytes, s));
  MC_CUDA(cudaMemsetAsync(c->s_flags.p, 0, c->s_flags.bytes, s));
  if (c->e_ok.p) MC_CUDA(cudaMemsetAsync(c->e_ok.p, 0, c->e_ok.bytes, s));  // line totals of another state
  MC_CUDA(cudaStreamSynchronize(s));
  c->s_ready = true;
  return MC_OK;
}

extern "C" mc_status mc_ctx_get_cell_state(mc_ctx_t *c, double *te, double *ne, double *X, int32_t *conv,
                                          int32_t *niter, int32_t *flags) {
  if (!c || !c->s_ready) return set_error(MC_ERR_ARG, "no cell state on the context");
  cudaStream_t s = c->stream;
  struct Item { void *h; DBuf *d; } items[6] = {{te, &c->s_te}, {ne, &c->s_ne}, {X, &c->s_X},
                                                {conv, &c->s_conv}, {niter, &c->s_niter}, {flags, &c->s_flags}};
  for (auto &it : items)
    if (it.h) MC_CUDA(cudaMemcpyAsync(it.h, it.d->p, it.d->bytes, cudaMemcpyDeviceToHost, s));
  MC_CUDA(cudaStreamSynchronize(s));
  return MC_OK;
}

namespace {
mc_status surrogate_predict_state(mc_ctx_t *c);
}

// The atomic tables and the resident cell state in the update's arguments.
static void fill_update_tables(mc_ctx_t *c, mcg::UpdArgs &a) {
  a.nc = c->nc;
  a.ncel = c->u_ncel;
  a.ndirec = c->u_ndirec;
  a.naldro = c->u_naldro;
  for (int i = 0; i < 7; ++i) { a.bal_z[i] = c->u_bal_z[i]; a.bal_first[i] = c->u_bal_first[i]; }
  a.d.bal = c->u_bal.as<mcg::UpdIonDev>();
  a.d.cel = c->u_cel.as<mcg::UpdCelDev>();
  a.d.rrec = c->u_rrec.as<double>(); a.d.rnew = c->u_rnew.as<double>();
  a.d.direc = c->u_direc.as<double>(); a.d.aldro = c->u_aldro.as<double>();
  a.d.logt = c->u_logt.as<double>(); a.d.g = c->u_g.as<double>(); a.d.e = c->u_e.as<double>();
  a.d.A = c->u_A.as<double>(); a.d.qq = c->u_qq.as<double>(); a.d.q2 = c->u_q2.as<double>();
  a.d.ab = c->u_ab.as<double>();
  a.f.bal = c->f_bal.as<mcg::UpdIonT<float>>();
  a.f.cel = c->f_cel.as<mcg::UpdCelT<float>>();
  a.f.rrec = c->f_rrec.as<float>(); a.f.rnew = c->f_rnew.as<float>();
  a.f.direc = c->f_direc.as<float>(); a.f.aldro = c->f_aldro.as<float>();
  a.f.logt = c->f_logt.as<float>(); a.f.g = c->f_g.as<float>(); a.f.e = c->f_e.as<float>();
  a.f.A = c->f_A.as<float>(); a.f.qq = c->f_qq.as<float>(); a.f.q2 = c->f_q2.as<float>();
  a.f.ab = c->f_ab.as<float>();
  a.hden = c->u_hden.as<double>();
  a.te = c->s_te.as<double>(); a.ne = c->s_ne.as<double>(); a.X = c->s_X.as<double>();
  a.mat_rows = c->u_maxlev;
  a.mat_stride = (c->u_maxlev * c->u_maxlev) | 1;
}

static mc_status ensure_line_totals(mc_ctx_t *c);

static mc_status update_cells_impl(mc_ctx_t *c, const float *w, double scale, double xhi_limit, int32_t precision,
                                   bool warm, mc_update_stats_t *stats) {
  NvtxRange nvtx_range("mc cell update");
  if (!c || !w) return set_error(MC_ERR_ARG, "ctx and w are required");
  if (warm && !(c->m_ready && c->m_norm)) return set_error(MC_ERR_ARG, "the surrogate is not trained");
  if (precision != MC_PREC_FP32 && precision != MC_PREC_FP64) return set_error(MC_ERR_ARG, "unknown precision");
  if (!c->u_ready) return set_error(MC_ERR_ARG, "mc_ctx_set_update_tables has not been called");
  if (!c->s_ready) return set_error(MC_ERR_ARG, "mc_ctx_set_cell_state has not been called");
  const int nout = 67, nc1 = c->nc + 1, nb = c->nb;
  cudaStream_t s = c->stream;
  mc_status st;
  if ((st = put_buf(c->s_w, w, (size_t)nb * nout * sizeof(float), s)) ||
      (st = put_buf(c->s_mom, nullptr, (size_t)nout * nc1 * sizeof(float), s)) ||
      (st = put_buf(c->s_err, nullptr, sizeof(int), s)) ||
      (st = put_buf(c->s_ustats, nullptr, sizeof(mcg::UpdStatsDev), s)))
    return st;
  MC_CUDA(cudaMemsetAsync(c->s_err.p, 0, sizeof(int), s));
  MC_CUDA(cudaMemsetAsync(c->s_ustats.p, 0, sizeof(mcg::UpdStatsDev), s));
  cudaEvent_t e0, e1, e2;
  MC_CUDA(cudaEventCreate(&e0));
  MC_CUDA(cudaEventCreate(&e1));
  MC_CUDA(cudaEventCreate(&e2));
  MC_CUDA(cudaEventRecord(e0, s));
  cudaError_t e = mcg::launch_jmoments(nc1, nb, nout, c->jste.as<double>(), c->s_w.as<float>(), scale,
                                       c->s_mom.as<float>(), c->s_err.as<int>(), c->num_sms, s);
  if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "moment launch failed: %s", cudaGetErrorString(e));
  MC_CUDA(cudaEventRecord(e1, s));
  if (warm) {
    mc_status ws = surrogate_predict_state(c);
    if (ws) return ws;
  }
  mcg::UpdArgs a{};
  a.nc = c->nc;
  a.te_prev = warm ? c->m_te_prev.as<double>() : nullptr;
  a.ne_prev = warm ? c->m_ne_prev.as<double>() : nullptr;
  a.x_prev = warm ? c->m_x_prev.as<double>() : nullptr;
  a.near_res = c->m_near_res;
  a.accept_res = c->m_accept_res;
  // a predicted Te is near the balance: bracket it with small steps first
  a.step0 = warm ? 1.03 : 1.2;
  a.step_grow = warm ? 1 : 0;
  fill_update_tables(c, a);
  a.mom = c->s_mom.as<float>();
  a.mstride = nc1;
  a.te = c->s_te.as<double>(); a.ne = c->s_ne.as<double>(); a.X = c->s_X.as<double>();
  a.conv = c->s_conv.as<int>(); a.niter = c->s_niter.as<int>(); a.flags = c->s_flags.as<int>();
  a.dte = c->s_dte.as<double>();
  a.xhi = xhi_limit;
  a.mat_rows = c->u_maxlev;
  a.mat_stride = (c->u_maxlev * c->u_maxlev) | 1;
  // with emission tables the FP32 form keeps each cell's last line totals for
  // the next emission build; the FP64 form marks the cells it updated stale
  if (c->e_ready && c->u_ncel > 0) {
    mc_status es = ensure_line_totals(c);
    if (es) return es;
    a.forb_out = precision == MC_PREC_FP32 ? c->e_forb.as<float>() : nullptr;
    a.forb_ok = c->e_ok.as<int>();
  }
  if (c->g_ns > 0) {
    mcg::GrainArgs &g = a.g;
    g.nsizes = c->g_ns;
    g.nb = nb;
    g.ivn = c->g_ivn;
    g.vn = c->g_vn; g.msurf = c->g_msurf; g.abundance = c->g_abun;
    g.nu = c->g_nu.as<float>(); g.xs = c->g_xs.as<float>();
    g.radius_um = c->g_rad.as<double>(); g.weight = c->g_w.as<double>(); g.ion_nu = c->g_ip.as<double>();
    g.yn_d = c->g_ynd.as<double>(); g.dnu_d = c->g_dnud.as<double>(); g.qa_d = c->g_qad.as<double>();
    g.yn_f = c->g_ynf.as<float>(); g.dnu_f = c->g_dnuf.as<float>(); g.qa_f = c->g_qaf.as<float>();
    g.idnu_f = c->g_idnuf.as<float>();
    g.inv_hnu = c->g_ihnu.as<double>();
    g.jste = c->jste.as<double>();
    g.jscale = scale;
    g.ndust = c->g_nd.as<float>();
    g.tdust = (c->d_tdust.p && c->d_nsizes == c->g_ns) ? c->d_tdust.as<float>() : nullptr;
    mc_status gs = c->g_out.bytes == (size_t)3 * c->g_ns * nc1 * sizeof(double)
                       ? MC_OK
                       : put_buf(c->g_out, nullptr, (size_t)3 * c->g_ns * nc1 * sizeof(double), s);
    if (gs) return gs;
    MC_CUDA(cudaMemsetAsync(c->g_out.p, 0, c->g_out.bytes, s));
    g.out = c->g_out.as<double>();
    c->g_fresh = true;
  }
  if (precision == MC_PREC_FP32) {
    const size_t need = mcg::cell_update_fp32_scratch(c->nc, c->u_ncel, c->g_ns, nb);
    mc_status ss = c->s_wave.bytes == need ? MC_OK : put_buf(c->s_wave, nullptr, need, s);
    if (ss) return ss;
  }
  if (precision == MC_PREC_FP32) {
    // the 101 launches of the T-step wavefronts replay as one graph; it is
    // captured again only when the arguments (state, tables, warm start) change
    const bool same = c->wave_exec && c->wave_scratch == c->s_wave.p &&
                      std::memcmp(&c->wave_args, &a, sizeof a) == 0;
    if (!same) {
      if (c->wave_exec) { cudaGraphExecDestroy(c->wave_exec); c->wave_exec = nullptr; }
      MC_CUDA(mcg::cell_update_fp32_prepare(a));
      cudaGraph_t graph = nullptr;
      MC_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      cudaError_t ce = mcg::launch_cell_update(a, 1, c->s_wave.p, c->num_sms, s);
      cudaError_t ee = cudaStreamEndCapture(s, &graph);
      if (ce == cudaSuccess) ce = ee;
      if (ce == cudaSuccess) ce = cudaGraphInstantiate(&c->wave_exec, graph, 0);
      if (graph) cudaGraphDestroy(graph);
      if (ce != cudaSuccess) {
        c->wave_exec = nullptr;
        return set_error(MC_ERR_CUDA, "cell update capture failed: %s", cudaGetErrorString(ce));
      }
      c->wave_args = a;
      c->wave_scratch = c->s_wave.p;
    }
    e = cudaGraphLaunch(c->wave_exec, s);
  } else {
    e = mcg::launch_cell_update(a, 0, c->s_wave.p, c->num_sms, s);
  }
  if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "cell update launch failed: %s", cudaGetErrorString(e));
  MC_CUDA(cudaEventRecord(e2, s));
  e = mcg::launch_update_stats(c->nc, a.conv, a.niter, a.flags, a.dte, c->s_ustats.as<mcg::UpdStatsDev>(),
                               c->num_sms, s);
  if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "update stats launch failed: %s", cudaGetErrorString(e));
  mcg::UpdStatsDev hs{};
  int herr = 0;
  MC_CUDA(cudaMemcpyAsync(&hs, c->s_ustats.p, sizeof hs, cudaMemcpyDeviceToHost, s));
  MC_CUDA(cudaMemcpyAsync(&herr, c->s_err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  MC_CUDA(cudaStreamSynchronize(s));
  if (warm && mcg::mlp_tc_take_error() > 0)
    return set_error(MC_ERR_TIMEOUT, "a tensor-core wait of the surrogate gave up");
  float m1 = 0.f, m2 = 0.f;
  cudaEventElapsedTime(&m1, e0, e1);
  cudaEventElapsedTime(&m2, e1, e2);
  cudaEventDestroy(e0); cudaEventDestroy(e1); cudaEventDestroy(e2);
  if (herr) return set_error((mc_status)herr, "moment kernel: tensor-core wait timed out");
  if (stats) {
    stats->hit = (int64_t)hs.hit;
    stats->converged = (int64_t)hs.converged;
    stats->no_te_balance = (int64_t)hs.no_te;
    stats->no_ion_balance = (int64_t)hs.no_ion;
    stats->warm_fallback = (int64_t)hs.fallback;
    stats->t_iterations = (int64_t)hs.iters;
    double dmax;
    std::memcpy(&dmax, &hs.dmax_bits, sizeof dmax);
    stats->dte_max = dmax;
    stats->frac_dte_1pc = hs.hit ? (double)hs.small / (double)hs.hit : 0.;
    stats->moments_ms = m1;
    stats->update_ms = m2;
  }
  return MC_OK;
}

extern "C" mc_status mc_ctx_update_cells(mc_ctx_t *c, const float *w, double scale, double xhi_limit,
                                        int32_t precision, mc_update_stats_t *stats) {
  return update_cells_impl(c, w, scale, xhi_limit, precision, false, stats);
}

extern "C" mc_status mc_ctx_update_cells_warm(mc_ctx_t *c, const float *w, double scale, double xhi_limit,
                                             int32_t precision, mc_update_stats_t *stats) {
  return update_cells_impl(c, w, scale, xhi_limit, precision, true, stats);
}

extern "C" mc_status mc_ctx_set_grain_physics(mc_ctx_t *c, const mc_grain_physics_t *gp) {
  if (!c) return set_error(MC_ERR_ARG, "ctx is NULL");
  c->g_fresh = false;
  if (!gp) { c->g_ns = 0; return MC_OK; }
  const int ns = gp->nsizes, nb = c->nb, nc1 = c->nc + 1;
  if (ns < 1 || ns > 32) return set_error(MC_ERR_ARG, "grain nsizes must be 1..32 (got %d)", ns);
  if (!gp->xs_abs || !gp->radius_um || !gp->weight || !gp->ion_nu || !gp->ndust)
    return set_error(MC_ERR_ARG, "grains: xs_abs, radius_um, weight, ion_nu and ndust are required");
  if (!(gp->vn >= 0.) || !(gp->msurf > 0.)) return set_error(MC_ERR_ARG, "grains: vn >= 0 and msurf > 0 required");
  for (int k = 0; k < ns; ++k)
    if (!(gp->radius_um[k] > 0.)) return set_error(MC_ERR_ARG, "grains: radius %d must be > 0", k);
  if (!c->nu.p) return set_error(MC_ERR_ARG, "the context has no frequency grid");
  std::vector<float> nu(nb);
  MC_CUDA(cudaMemcpy(nu.data(), c->nu.p, (size_t)nb * sizeof(float), cudaMemcpyDeviceToHost));
  // the per-bin factors of the grain sums that do not depend on the
  // potential: yield Yn = min(Y0 (1 - Vn/nu), Y1) (Y0 = 0.5, Y1 = 0.2,
  // update_mod.f90:20), nu - Vn, and Qa = Cabs / (1e-8 a^2) per size
  std::vector<double> ynd(nb), dnud(nb), qad((size_t)ns * nb), ihnu(nb);
  std::vector<float> ynf(nb), dnuf(nb), qaf((size_t)ns * nb), idnuf(nb);
  const double vn = gp->vn;
  for (int i = 0; i < nb; ++i) {
    const double v = (double)nu[i];
    ynd[i] = std::min(0.5 * (1. - vn / v), 0.2);
    dnud[i] = v - vn;
    ihnu[i] = 1. / (2.1799153e-11 * v);
    ynf[i] = (float)ynd[i];
    dnuf[i] = (float)dnud[i];
    idnuf[i] = 1.f / dnuf[i];
  }
  for (int k = 0; k < ns; ++k) {
    const double r = gp->radius_um[k], qden = 1.e-8 * (r * r);
    for (int i = 0; i < nb; ++i) {
      qad[(size_t)k * nb + i] = (double)gp->xs_abs[(size_t)k * nb + i] / qden;
      qaf[(size_t)k * nb + i] = (float)qad[(size_t)k * nb + i];
    }
  }
  cudaStream_t s = c->stream;
  mc_status st;
  if ((st = put_buf(c->g_nu, nu.data(), (size_t)nb * 4, s)) ||
      (st = put_buf(c->g_xs, gp->xs_abs, (size_t)ns * nb * 4, s)) ||
      (st = put_buf(c->g_rad, gp->radius_um, (size_t)ns * 8, s)) ||
      (st = put_buf(c->g_w, gp->weight, (size_t)ns * 8, s)) ||
      (st = put_buf(c->g_ip, gp->ion_nu, 33 * 8, s)) ||
      (st = put_buf(c->g_ynd, ynd.data(), (size_t)nb * 8, s)) ||
      (st = put_buf(c->g_dnud, dnud.data(), (size_t)nb * 8, s)) ||
      (st = put_buf(c->g_qad, qad.data(), qad.size() * 8, s)) ||
      (st = put_buf(c->g_ynf, ynf.data(), (size_t)nb * 4, s)) ||
      (st = put_buf(c->g_dnuf, dnuf.data(), (size_t)nb * 4, s)) ||
      (st = put_buf(c->g_qaf, qaf.data(), qaf.size() * 4, s)) ||
      (st = put_buf(c->g_nd, gp->ndust, (size_t)nc1 * 4, s)) ||
      (st = put_buf(c->g_ihnu, ihnu.data(), (size_t)nb * 8, s)) ||
      (st = put_buf(c->g_idnuf, idnuf.data(), (size_t)nb * 4, s)))
    return st;
  MC_CUDA(cudaStreamSynchronize(s));
  // the first bin above Vn (locate's 1-based index of the last bin <= Vn)
  int ivn = 0;
  if (vn > (double)nu[nb - 1]) ivn = nb;
  else if (vn >= (double)nu[0])
    while (ivn < nb && !((double)nu[ivn] > vn)) ++ivn;
  c->g_ivn = ivn;
  c->g_ns = ns;
  c->g_vn = vn;
  c->g_msurf = gp->msurf;
  c->g_abun = gp->abundance;
  return MC_OK;
}

extern "C" mc_status mc_ctx_grain_state(mc_ctx_t *c, double *potential, double *photoel_cool, double *coll_heat) {
  if (!c) return set_error(MC_ERR_ARG, "ctx is NULL");
  if (c->g_ns <= 0 || !c->g_fresh) return set_error(MC_ERR_ARG, "no update with grains has run");
  const size_t n = (size_t)c->g_ns * (c->nc + 1);
  double *dst[3] = {potential, photoel_cool, coll_heat};
  for (int q = 0; q < 3; ++q)
    if (dst[q]) MC_CUDA(cudaMemcpyAsync(dst[q], c->g_out.as<double>() + q * n, n * 8, cudaMemcpyDeviceToHost, c->stream));
  MC_CUDA(cudaStreamSynchronize(c->stream));
  return MC_OK;
}

// ------------------------------------------------------------ surrogate
namespace {

using mcg::kMlpIn;
using mcg::kMlpHid;
using mcg::kMlpOut;
using mcg::kMlpParams;


// forward pass of M rows: x [M][80] -> a1, a2, a3 [M][256] -> y [M][48]
// the four layers of M rows; tensor: on tcgen05 (the prediction over a
// grid), else on the CUDA cores (training, whose steps of a few thousand
// rows gain nothing from the tensor cores and keep the arithmetic the
// measured networks were trained with)
mc_status mlp_forward(mc_ctx_t *c, int M, const float *x, float *a1, float *a2, float *a3, float *y,
                      bool tensor = false) {
  const float *W = c->m_w.as<float>();
  cudaStream_t s = c->stream;
  const int sm = c->num_sms;
  auto layer = [&](int N, int K, const float *a, const float *w, const float *b, int act, float *o) {
    return tensor ? mcg::launch_mlp_forward_tc(M, N, K, a, K, w, b, act, o, N, sm, s)
                  : mcg::launch_mlp_gemm(M, N, K, a, K, nullptr, true, w, true, b, act, o, N, s);
  };
  cudaError_t e = layer(kMlpHid, kMlpIn, x, W + mcg::kMlpW1, W + mcg::kMlpB1, 1, a1);
  if (e == cudaSuccess) e = layer(kMlpHid, kMlpHid, a1, W + mcg::kMlpW2, W + mcg::kMlpB2, 1, a2);
  if (e == cudaSuccess) e = layer(kMlpHid, kMlpHid, a2, W + mcg::kMlpW3, W + mcg::kMlpB3, 1, a3);
  if (e == cudaSuccess) e = layer(kMlpOut, kMlpHid, a3, W + mcg::kMlpW4, W + mcg::kMlpB4, 0, y);
  if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "mlp forward failed: %s", cudaGetErrorString(e));
  return MC_OK;
}

// loss and gradients of M rows (x, normalised targets t) into m_g
mc_status mlp_backward(mc_ctx_t *c, int M, const float *x, const float *t) {
  cudaStream_t s = c->stream;
  mc_status st;
  const size_t h = (size_t)M * kMlpHid * 4, o = (size_t)M * kMlpOut * 4;
  if ((st = ensure(c->m_a1, h)) || (st = ensure(c->m_a2, h)) || (st = ensure(c->m_a3, h)) ||
      (st = ensure(c->m_y, o)) || (st = ensure(c->m_dy, o)) || (st = ensure(c->m_d3, h)) ||
      (st = ensure(c->m_d2, h)) || (st = ensure(c->m_d1, h)))
    return st;
  float *a1 = c->m_a1.as<float>(), *a2 = c->m_a2.as<float>(), *a3 = c->m_a3.as<float>();
  float *y = c->m_y.as<float>(), *dy = c->m_dy.as<float>();
  float *d3 = c->m_d3.as<float>(), *d2 = c->m_d2.as<float>(), *d1 = c->m_d1.as<float>();
  if ((st = mlp_forward(c, M, x, a1, a2, a3, y))) return st;
  const float *W = c->m_w.as<float>();
  float *G = c->m_g.as<float>();
  const int sm = c->num_sms;
  const size_t nscr = std::max({mcg::mlp_wgrad_scratch_floats(M, kMlpOut, kMlpHid, sm),
                                mcg::mlp_wgrad_scratch_floats(M, kMlpHid, kMlpHid, sm),
                                mcg::mlp_wgrad_scratch_floats(M, kMlpHid, kMlpIn, sm)});
  if ((st = ensure(c->m_gscr, nscr * sizeof(float)))) return st;
  float *scr = c->m_gscr.as<float>();
  MC_CUDA(cudaMemsetAsync(G, 0, kMlpParams * sizeof(float), s));
  cudaError_t e = mcg::launch_mlp_loss(M, mcg::kMlpTargets, kMlpOut, y, t, dy, c->m_loss.as<double>(), s);
  // layer 4 (linear): dW4 = dY^T a3, dA3 = dY W4
  if (e == cudaSuccess)
    e = mcg::launch_mlp_wgrad(M, kMlpOut, kMlpHid, dy, nullptr, a3, G + mcg::kMlpW4, G + mcg::kMlpB4, scr, nscr, sm, s);
  if (e == cudaSuccess)
    e = mcg::launch_mlp_gemm(M, kMlpHid, kMlpOut, dy, kMlpOut, nullptr, false, W + mcg::kMlpW4, false, nullptr, 0, d3,
                             kMlpHid, s);
  // layer 3 (ReLU): dZ3 = dA3 (a3 > 0)
  if (e == cudaSuccess)
    e = mcg::launch_mlp_wgrad(M, kMlpHid, kMlpHid, d3, a3, a2, G + mcg::kMlpW3, G + mcg::kMlpB3, scr, nscr, sm, s);
  if (e == cudaSuccess)
    e = mcg::launch_mlp_gemm(M, kMlpHid, kMlpHid, d3, kMlpHid, a3, false, W + mcg::kMlpW3, false, nullptr, 0, d2,
                             kMlpHid, s);
  // layer 2 (ReLU): dZ2 = dA2 (a2 > 0)
  if (e == cudaSuccess)
    e = mcg::launch_mlp_wgrad(M, kMlpHid, kMlpHid, d2, a2, a1, G + mcg::kMlpW2, G + mcg::kMlpB2, scr, nscr, sm, s);
  if (e == cudaSuccess)
    e = mcg::launch_mlp_gemm(M, kMlpHid, kMlpHid, d2, kMlpHid, a2, false, W + mcg::kMlpW2, false, nullptr, 0, d1,
                             kMlpHid, s);
  // layer 1 (ReLU): dZ1 = dA1 (a1 > 0)
  if (e == cudaSuccess)
    e = mcg::launch_mlp_wgrad(M, kMlpHid, kMlpIn, d1, a1, x, G + mcg::kMlpW1, G + mcg::kMlpB1, scr, nscr, sm, s);
  if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "mlp backward failed: %s", cudaGetErrorString(e));
  return MC_OK;
}

mc_status surrogate_predict_state(mc_ctx_t *c) {
  const int nc1 = c->nc + 1;
  cudaStream_t s = c->stream;
  mc_status st;
  if ((st = ensure(c->m_xi, (size_t)nc1 * kMlpIn * 4)) || (st = ensure(c->m_h1, (size_t)nc1 * kMlpHid * 4)) ||
      (st = ensure(c->m_h2, (size_t)nc1 * kMlpHid * 4)) || (st = ensure(c->m_h3, (size_t)nc1 * kMlpHid * 4)) ||
      (st = ensure(c->m_yi, (size_t)nc1 * kMlpOut * 4)) ||
      (st = ensure(c->m_te_prev, (size_t)nc1 * 8)) || (st = ensure(c->m_ne_prev, (size_t)nc1 * 8)) ||
      (st = ensure(c->m_x_prev, (size_t)nc1 * 56 * 8)))
    return st;
  cudaError_t e = mcg::launch_mlp_infer_features(c->nc, c->s_mom.as<float>(), nc1, c->u_hden.as<double>(),
                                                 c->m_fmean.as<float>(), c->m_fstd.as<float>(), c->m_xi.as<float>(),
                                                 c->num_sms, s);
  if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "features failed: %s", cudaGetErrorString(e));
  if ((st = mlp_forward(c, nc1, c->m_xi.as<float>(), c->m_h1.as<float>(), c->m_h2.as<float>(), c->m_h3.as<float>(),
                        c->m_yi.as<float>(), true)))
    return st;
  e = mcg::launch_mlp_apply(c->nc, c->s_mom.as<float>(), c->m_yi.as<float>(), c->m_tmean.as<float>(),
                            c->m_tstd.as<float>(), c->s_te.as<double>(), c->s_ne.as<double>(), c->s_X.as<double>(),
                            c->m_te_prev.as<double>(), c->m_ne_prev.as<double>(), c->m_x_prev.as<double>(),
                            c->num_sms, s);
  if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "apply failed: %s", cudaGetErrorString(e));
  return MC_OK;
}

mc_status surrogate_normalise(mc_ctx_t *c) {
  const long long n = std::min(c->m_n, c->m_cap);
  if (n < 2) return set_error(MC_ERR_ARG, "the surrogate has fewer than 2 training rows");
  cudaStream_t s = c->stream;
  // per-block partial sums, added here in block order (reproducible)
  const size_t B = mcg::kMlpStatBlocks, ox = 0, qx = B * kMlpIn, ot = 2 * B * kMlpIn, qt = ot + B * kMlpOut;
  DBuf sums;
  MC_CUDA(sums.alloc((qt + B * kMlpOut) * sizeof(double)));
  double *d = sums.as<double>();
  cudaError_t e = mcg::launch_mlp_stats(n, kMlpIn, c->m_xs.as<float>(), d + ox, d + qx, s);
  if (e == cudaSuccess) e = mcg::launch_mlp_stats(n, kMlpOut, c->m_ts.as<float>(), d + ot, d + qt, s);
  if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "stats failed: %s", cudaGetErrorString(e));
  std::vector<double> part(qt + B * kMlpOut), h(4 * 128, 0.0);
  MC_CUDA(cudaMemcpyAsync(part.data(), d, sums.bytes, cudaMemcpyDeviceToHost, s));
  MC_CUDA(cudaStreamSynchronize(s));
  for (size_t b = 0; b < B; ++b) {
    for (int i = 0; i < kMlpIn; ++i) { h[i] += part[ox + b * kMlpIn + i]; h[128 + i] += part[qx + b * kMlpIn + i]; }
    for (int o = 0; o < kMlpOut; ++o) { h[256 + o] += part[ot + b * kMlpOut + o]; h[384 + o] += part[qt + b * kMlpOut + o]; }
  }
  std::vector<float> fm(kMlpIn), fs(kMlpIn), tm(kMlpOut), ts(kMlpOut);
  auto ms = [&](double sum, double sq, float &mean, float &sd) {
    const double m = sum / (double)n, v = std::max(sq / (double)n - m * m, 0.);
    mean = (float)m;
    sd = (float)std::max(std::sqrt(v), 1e-3);
  };
  for (int i = 0; i < kMlpIn; ++i) ms(h[i], h[128 + i], fm[i], fs[i]);
  for (int o = 0; o < kMlpOut; ++o) ms(h[256 + o], h[384 + o], tm[o], ts[o]);
  mc_status st;
  if ((st = put_buf(c->m_fmean, fm.data(), kMlpIn * 4, s)) || (st = put_buf(c->m_fstd, fs.data(), kMlpIn * 4, s)) ||
      (st = put_buf(c->m_tmean, tm.data(), kMlpOut * 4, s)) || (st = put_buf(c->m_tstd, ts.data(), kMlpOut * 4, s)))
    return st;
  MC_CUDA(cudaStreamSynchronize(s));
  c->m_norm = true;
  return MC_OK;
}

}  // namespace

extern "C" mc_status mc_ctx_surrogate_rule(mc_ctx_t *c, double accept_res, double near_res) {
  if (!c || !(accept_res > 0. && accept_res <= 0.01) || !(near_res >= accept_res))
    return set_error(MC_ERR_ARG, "ctx, 0 < accept_res <= 0.01 and near_res >= accept_res are required");
  c->m_accept_res = accept_res;
  c->m_near_res = near_res;
  return MC_OK;
}

extern "C" mc_status mc_ctx_surrogate_init(mc_ctx_t *c, uint64_t seed, int64_t capacity) {
  if (!c || capacity < 1) return set_error(MC_ERR_ARG, "ctx and a positive capacity are required");
  cudaStream_t s = c->stream;
  // He-uniform initial weights, zero biases
  std::vector<float> w(kMlpParams, 0.f);
  uint64_t x = seed ? seed : 0x9E3779B97F4A7C15ull;
  auto uni = [&]() {
    x ^= x << 13; x ^= x >> 7; x ^= x << 17;  // xorshift64
    return (double)(x >> 11) * (1.0 / 9007199254740992.0);
  };
  auto fill = [&](int off, int nout, int nin) {
    const double lim = std::sqrt(6.0 / nin);
    for (int i = 0; i < nout * nin; ++i) w[off + i] = (float)((2. * uni() - 1.) * lim);
  };
  fill(mcg::kMlpW1, kMlpHid, 68);
  fill(mcg::kMlpW2, kMlpHid, kMlpHid);
  fill(mcg::kMlpW3, kMlpHid, kMlpHid);
  fill(mcg::kMlpW4, kMlpOut, kMlpHid);
  for (int o = 0; o < kMlpHid; ++o)
    for (int i = 68; i < kMlpIn; ++i) w[mcg::kMlpW1 + o * kMlpIn + i] = 0.f;
  mc_status st;
  if ((st = put_buf(c->m_w, w.data(), kMlpParams * 4, s)) || (st = put_buf(c->m_g, nullptr, kMlpParams * 4, s)) ||
      (st = put_buf(c->m_m1, nullptr, kMlpParams * 4, s)) || (st = put_buf(c->m_m2, nullptr, kMlpParams * 4, s)) ||
      (st = put_buf(c->m_xs, nullptr, (size_t)capacity * kMlpIn * 4, s)) ||
      (st = put_buf(c->m_ts, nullptr, (size_t)capacity * kMlpOut * 4, s)) ||
      (st = put_buf(c->m_count, nullptr, 8, s)) || (st = put_buf(c->m_loss, nullptr, 8, s)) ||
      (st = put_buf(c->m_dstep, nullptr, sizeof(int), s)))
    return st;
  MC_CUDA(mcg::mlp_prepare());
  MC_CUDA(cudaMemsetAsync(c->m_dstep.p, 0, sizeof(int), s));
  MC_CUDA(cudaMemsetAsync(c->m_m1.p, 0, c->m_m1.bytes, s));
  MC_CUDA(cudaMemsetAsync(c->m_m2.p, 0, c->m_m2.bytes, s));
  MC_CUDA(cudaMemsetAsync(c->m_count.p, 0, 8, s));
  MC_CUDA(cudaStreamSynchronize(s));
  c->m_cap = capacity;
  c->m_n = 0;
  c->m_step = 0;
  c->m_ready = true;
  c->m_norm = false;
  return MC_OK;
}

extern "C" mc_status mc_ctx_surrogate_collect(mc_ctx_t *c, int64_t *rows) {
  if (!c || !c->m_ready) return set_error(MC_ERR_ARG, "mc_ctx_surrogate_init has not been called");
  if (!c->s_mom.p || !c->s_ready) return set_error(MC_ERR_ARG, "no cell update to learn from");
  cudaStream_t s = c->stream;
  mc_status st0;
  if ((st0 = ensure(c->m_ccnt, (size_t)mcg::mlp_collect_blocks(c->num_sms) * sizeof(unsigned int)))) return st0;
  cudaError_t e = mcg::launch_mlp_collect(c->nc, c->s_mom.as<float>(), c->nc + 1, c->u_hden.as<double>(),
                                          c->s_te.as<double>(), c->s_X.as<double>(), c->s_flags.as<int>(), c->m_cap,
                                          c->m_count.as<unsigned long long>(), c->m_xs.as<float>(),
                                          c->m_ts.as<float>(), c->m_ccnt.as<unsigned int>(), c->num_sms, s);
  if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "collect failed: %s", cudaGetErrorString(e));
  unsigned long long n = 0;
  MC_CUDA(cudaMemcpyAsync(&n, c->m_count.p, 8, cudaMemcpyDeviceToHost, s));
  MC_CUDA(cudaStreamSynchronize(s));
  c->m_n = (long long)n;
  // the normalisation is fixed by the first training: the network's
  // weights depend on it, so later rows are scaled the same way
  if (rows) *rows = std::min((long long)n, c->m_cap);
  return MC_OK;
}

extern "C" mc_status mc_ctx_surrogate_train(mc_ctx_t *c, int32_t steps, int32_t batch, float lr, uint64_t seed,
                                           double *loss, double *train_ms) {
  NvtxRange nvtx_range("mc surrogate training");
  if (!c || !c->m_ready) return set_error(MC_ERR_ARG, "mc_ctx_surrogate_init has not been called");
  if (steps < 0 || batch < 1) return set_error(MC_ERR_ARG, "steps >= 0 and batch >= 1 required");
  mc_status st;
  if (!c->m_norm && (st = surrogate_normalise(c))) return st;
  cudaStream_t s = c->stream;
  if ((st = ensure(c->m_xb, (size_t)batch * kMlpIn * 4)) || (st = ensure(c->m_tb, (size_t)batch * kMlpOut * 4)))
    return st;
  cudaEvent_t e0, e1;
  MC_CUDA(cudaEventCreate(&e0));
  MC_CUDA(cudaEventCreate(&e1));
  MC_CUDA(cudaEventRecord(e0, s));
  const long long n = std::min(c->m_n, c->m_cap);
  double last = 0.;
  const int step0 = c->m_step;
  // one training step: minibatch, forward, loss, backward, Adam, t += 1
  auto one_step = [&]() -> mc_status {
    MC_CUDA(cudaMemsetAsync(c->m_loss.p, 0, 8, s));
    cudaError_t e = mcg::launch_mlp_gather(batch, n, (uint32_t)seed, c->m_dstep.as<int>(), c->m_xs.as<float>(),
                                           c->m_ts.as<float>(), c->m_fmean.as<float>(), c->m_fstd.as<float>(),
                                           c->m_tmean.as<float>(), c->m_tstd.as<float>(), c->m_xb.as<float>(),
                                           c->m_tb.as<float>(), s);
    if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "gather failed: %s", cudaGetErrorString(e));
    mc_status bs = mlp_backward(c, batch, c->m_xb.as<float>(), c->m_tb.as<float>());
    if (bs) return bs;
    e = mcg::launch_mlp_adam(kMlpParams, c->m_w.as<float>(), c->m_g.as<float>(), c->m_m1.as<float>(),
                             c->m_m2.as<float>(), c->m_dstep.as<int>(), step0, steps, lr, s);
    if (e == cudaSuccess) e = mcg::launch_mlp_step(c->m_dstep.as<int>(), s);
    if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "adam failed: %s", cudaGetErrorString(e));
    return MC_OK;
  };
  // the first step runs eagerly (it sizes the work arrays); the rest replay
  // a captured graph of one step
  if (steps > 0 && (st = one_step())) return st;
  if (steps > 1) {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    MC_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    mc_status cs = one_step();
    cudaError_t ce = cudaStreamEndCapture(s, &graph);
    if (cs) { if (graph) cudaGraphDestroy(graph); return cs; }
    if (ce != cudaSuccess) return set_error(MC_ERR_CUDA, "training capture failed: %s", cudaGetErrorString(ce));
    ce = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (ce != cudaSuccess) return set_error(MC_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(ce));
    for (int k = 1; k < steps && ce == cudaSuccess; ++k) ce = cudaGraphLaunch(exec, s);
    cudaGraphExecDestroy(exec);
    if (ce != cudaSuccess) return set_error(MC_ERR_CUDA, "graph launch failed: %s", cudaGetErrorString(ce));
  }
  c->m_step += steps;
  MC_CUDA(cudaEventRecord(e1, s));
  if (steps > 0) MC_CUDA(cudaMemcpyAsync(&last, c->m_loss.p, 8, cudaMemcpyDeviceToHost, s));
  MC_CUDA(cudaStreamSynchronize(s));
  if (mcg::mlp_tc_take_error() > 0) return set_error(MC_ERR_TIMEOUT, "a tensor-core wait of the surrogate gave up");
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (loss) *loss = steps > 0 ? last / ((double)batch * mcg::kMlpTargets) : 0.;
  if (train_ms) *train_ms = ms;
  return MC_OK;
}

extern "C" mc_status mc_ctx_surrogate_rows(mc_ctx_t *c, int64_t *n, float *x, float *t) {
  if (!c || !c->m_ready || !n) return set_error(MC_ERR_ARG, "mc_ctx_surrogate_init has not been called");
  const long long rows = std::min(c->m_n, c->m_cap);
  *n = rows;
  if (x) MC_CUDA(cudaMemcpyAsync(x, c->m_xs.p, (size_t)rows * kMlpIn * 4, cudaMemcpyDeviceToHost, c->stream));
  if (t) MC_CUDA(cudaMemcpyAsync(t, c->m_ts.p, (size_t)rows * kMlpOut * 4, cudaMemcpyDeviceToHost, c->stream));
  MC_CUDA(cudaStreamSynchronize(c->stream));
  return MC_OK;
}

extern "C" mc_status mc_ctx_surrogate_load(mc_ctx_t *c, int64_t n, const float *x, const float *t) {
  if (!c || !c->m_ready) return set_error(MC_ERR_ARG, "mc_ctx_surrogate_init has not been called");
  if (n < 0 || (n > 0 && (!x || !t))) return set_error(MC_ERR_ARG, "n >= 0 rows with x and t required");
  const long long have = std::min(c->m_n, c->m_cap), take = std::min((long long)n, c->m_cap - have);
  if (take > 0) {
    MC_CUDA(cudaMemcpyAsync(c->m_xs.as<float>() + (size_t)have * kMlpIn, x, (size_t)take * kMlpIn * 4,
                            cudaMemcpyHostToDevice, c->stream));
    MC_CUDA(cudaMemcpyAsync(c->m_ts.as<float>() + (size_t)have * kMlpOut, t, (size_t)take * kMlpOut * 4,
                            cudaMemcpyHostToDevice, c->stream));
  }
  const unsigned long long total = (unsigned long long)(have + std::max(take, 0ll));
  MC_CUDA(cudaMemcpyAsync(c->m_count.p, &total, 8, cudaMemcpyHostToDevice, c->stream));
  MC_CUDA(cudaStreamSynchronize(c->stream));
  c->m_n = (long long)total;
  return MC_OK;
}

extern "C" mc_status mc_ctx_surrogate_params(mc_ctx_t *c, float *get, const float *set) {
  if (!c || !c->m_ready) return set_error(MC_ERR_ARG, "mc_ctx_surrogate_init has not been called");
  if (set) MC_CUDA(cudaMemcpyAsync(c->m_w.p, set, kMlpParams * 4, cudaMemcpyHostToDevice, c->stream));
  if (get) MC_CUDA(cudaMemcpyAsync(get, c->m_w.p, kMlpParams * 4, cudaMemcpyDeviceToHost, c->stream));
  MC_CUDA(cudaStreamSynchronize(c->stream));
  return MC_OK;
}

extern "C" mc_status mc_ctx_surrogate_grads(mc_ctx_t *c, int32_t m, const float *x, const float *t, double *loss,
                                           float *grads, float *y) {
  if (!c || !c->m_ready || m < 1 || !x || !t) return set_error(MC_ERR_ARG, "bad surrogate gradient arguments");
  cudaStream_t s = c->stream;
  DBuf dx, dt;
  MC_CUDA(dx.alloc((size_t)m * kMlpIn * 4));
  MC_CUDA(dt.alloc((size_t)m * kMlpOut * 4));
  MC_CUDA(cudaMemcpyAsync(dx.p, x, dx.bytes, cudaMemcpyHostToDevice, s));
  MC_CUDA(cudaMemcpyAsync(dt.p, t, dt.bytes, cudaMemcpyHostToDevice, s));
  MC_CUDA(cudaMemsetAsync(c->m_loss.p, 0, 8, s));
  mc_status st = mlp_backward(c, m, dx.as<float>(), dt.as<float>());
  if (st) return st;
  double l = 0.;
  MC_CUDA(cudaMemcpyAsync(&l, c->m_loss.p, 8, cudaMemcpyDeviceToHost, s));
  if (grads) MC_CUDA(cudaMemcpyAsync(grads, c->m_g.p, kMlpParams * 4, cudaMemcpyDeviceToHost, s));
  if (y) MC_CUDA(cudaMemcpyAsync(y, c->m_y.p, (size_t)m * kMlpOut * 4, cudaMemcpyDeviceToHost, s));
  MC_CUDA(cudaStreamSynchronize(s));
  if (mcg::mlp_tc_take_error() > 0) return set_error(MC_ERR_TIMEOUT, "a tensor-core wait of the surrogate gave up");
  if (loss) *loss = l / ((double)m * mcg::kMlpTargets);
  return MC_OK;
}

extern "C" mc_status mc_ctx_surrogate_forward(mc_ctx_t *c, int32_t m, const float *x, float *y) {
  if (!c || !c->m_ready || m < 1 || !x || !y) return set_error(MC_ERR_ARG, "bad surrogate forward arguments");
  cudaStream_t s = c->stream;
  DBuf dx, h1, h2, h3, dy;
  MC_CUDA(dx.alloc((size_t)m * kMlpIn * 4));
  MC_CUDA(h1.alloc((size_t)m * kMlpHid * 4));
  MC_CUDA(h2.alloc((size_t)m * kMlpHid * 4));
  MC_CUDA(h3.alloc((size_t)m * kMlpHid * 4));
  MC_CUDA(dy.alloc((size_t)m * kMlpOut * 4));
  MC_CUDA(cudaMemcpyAsync(dx.p, x, dx.bytes, cudaMemcpyHostToDevice, s));
  mc_status st = mlp_forward(c, m, dx.as<float>(), h1.as<float>(), h2.as<float>(), h3.as<float>(), dy.as<float>(), true);
  if (st) return st;
  MC_CUDA(cudaMemcpyAsync(y, dy.p, dy.bytes, cudaMemcpyDeviceToHost, s));
  MC_CUDA(cudaStreamSynchronize(s));
  if (mcg::mlp_tc_take_error() > 0) return set_error(MC_ERR_TIMEOUT, "a tensor-core wait of the surrogate gave up");
  return MC_OK;
}

namespace {

// locate (interpolation_mod.f90:48-81): 1-based index of the last entry <= x
// (n above the grid, 0 below it, 1 for x equal to the last entry)
int locate_host(const float *xa, int n, float x) {
  if (x > xa[n - 1]) return n;
  if (x < xa[0]) return 0;
  for (int i = 0; i < n; ++i)
    if (xa[i] > x) return std::max(i, 1);
  return 1;
}

// HINuEdgeP & co. (initGammaCont, ph_mod.f90:135-197), 1-based
std::vector<int> edge_pointers(const float *nu, int nb, const float *nug, int nlim) {
  std::vector<int> p(nlim);
  for (int i = 0; i < nlim; ++i) {
    int k = locate_host(nu, nb, nug[i]);
    if (k < nb && k >= 1 && nug[i] > (nu[k - 1] + nu[k]) / 2.f) ++k;
    p[i] = k;
  }
  p[0] = 1;
  return p;
}

// two-photon spectral distribution of a hydrogenic ion (hydro2phot,
// emission_mod.f90:553-663) without its Te-dependent coefficient
float hydro2phot_shape(float nu, int z) {
  const float nu0 = z == 1 ? 0.7496f : 3.00f;
  if (nu >= nu0) return 0.f;
  const float y = nu / nu0, q = 4.f * y * (1.f - y);
  const float ay0 = 202.0f * (y * (1 - y) * (1 - powf(q, 0.8f)) + 0.88f * powf(y * (1 - y), 1.53f) * powf(q, 0.8f));
  const float z6 = (float)(z * z * z * z * z * z);
  const float ay = z == 1 ? ay0 : z6 * 0.9994667f * ay0;
  const float a2q = z == 1 ? 8.2249f : 8.226f * z6;
  return 6.6262e-27f * y * ay / a2q * 1e27f;
}

}  // namespace

// the line-total buffers of the emission build; e_ok starts at 0 (stale)
static mc_status ensure_line_totals(mc_ctx_t *c) {
  const size_t nc1 = (size_t)c->nc + 1;
  mc_status st;
  if ((st = put_buf(c->e_forb, nullptr, (size_t)std::max(c->u_ncel, 1) * nc1 * sizeof(float), c->stream)))
    return st;
  if (!c->e_ok.p) {
    MC_CUDA(c->e_ok.alloc(nc1 * sizeof(int)));
    MC_CUDA(cudaMemsetAsync(c->e_ok.p, 0, nc1 * sizeof(int), c->stream));
  }
  if (!c->e_list.p) MC_CUDA(c->e_list.alloc(nc1 * sizeof(int)));
  if (!c->e_cnt.p) MC_CUDA(c->e_cnt.alloc(sizeof(int)));
  return MC_OK;
}

extern "C" mc_status mc_ctx_set_emission_tables(mc_ctx_t *c, const mc_emission_tables_t *t) {
  if (!c || !t) return set_error(MC_ERR_ARG, "ctx and tables are required");
  const int nb = c->nb;
  if (t->nbins != nb) return set_error(MC_ERR_ARG, "emission tables: nbins %d, grid %d", t->nbins, nb);
  if (nb > mcg::kEmiMaxBins) return set_error(MC_ERR_ARG, "emission tables: at most %d bins", mcg::kEmiMaxBins);
  if (!t->nu || !t->wid_flx || !t->xs_h || !t->xs_hei || !t->xs_heii || !t->tk || !t->lg_hi || !t->lg_hei ||
      !t->lg_heii || !t->nu_gamma_hi || !t->nu_gamma_hei || !t->nu_gamma_heii || !t->y_ay || !t->hi_rec ||
      !t->heii_rec || !t->heii_lyman || !t->hei_rec || !t->gaunt_dd || (t->n_heavy > 0 && (!t->heavy || !t->xs_outer)))
    return set_error(MC_ERR_ARG, "emission tables: an array is missing");
  const int nlim[3] = {t->nlim_hi, t->nlim_hei, t->nlim_heii};
  for (int k = 0; k < 3; ++k)
    if (nlim[k] < 2 || nlim[k] > mcg::kEmiMaxLim || (nlim[k] & 1))
      return set_error(MC_ERR_ARG, "emission tables: gamma limits must be even, 2..%d", mcg::kEmiMaxLim);
  if (nlim[0] + nlim[1] + nlim[2] > 64) return set_error(MC_ERR_ARG, "emission tables: at most 64 gamma limits");
  if (t->ntk < 2 || t->n_heavy < 0 || t->n_heavy > mcg::kEmiMaxHeavy)
    return set_error(MC_ERR_ARG, "emission tables: ntk >= 2 and n_heavy <= %d required", mcg::kEmiMaxHeavy);
  const float *nu = t->nu;
  for (int i = 1; i < nb; ++i)
    if (!(nu[i] > nu[i - 1])) return set_error(MC_ERR_ARG, "emission tables: nu must increase");
  // everything derived goes into one float/int buffer
  std::vector<float> F;
  std::vector<int> I;
  auto putf = [&](const float *p, size_t n) { size_t o = F.size(); F.insert(F.end(), p, p + n); return o; };
  std::vector<float> lnu(nb), wid(nb), tph(nb), tphe(nb), tpheii(nb);
  for (int i = 0; i < nb; ++i) {
    lnu[i] = log10f(nu[i]);
    wid[i] = 3.2898423e15f * t->wid_flx[i] / 1.e15f;
    tph[i] = hydro2phot_shape(nu[i], 1);
    tpheii[i] = hydro2phot_shape(nu[i], 2);
  }
  // HeI 2^1S -> 1^1S (HeI2photSub, emission_mod.f90:665-705): the table
  // pointer moves on by at most one entry per bin
  {
    const float *ya = t->y_ay;
    int j = 1;
    for (int i = 0; i < nb; ++i) {
      const float y = nu[i] / 1.514f;
      if (y > ya[2 * (j - 1)]) ++j;
      if (j >= 41) break;
      const float fit1 = (ya[2 * j + 1] - ya[2 * (j - 1) + 1]) / (ya[2 * j] - ya[2 * (j - 1)]);
      const float fit2 = ya[2 * (j - 1) + 1] - ya[2 * (j - 1)] * fit1;
      float ay = fit1 * y + fit2;
      if (ay < 9.2163086E-03f) ay = 0.f;
      tphe[i] = ay * 0.66262f * y / 51.3f;
    }
  }
  const size_t o_nu = putf(nu, nb), o_lnu = putf(lnu.data(), nb), o_wid = putf(wid.data(), nb);
  const size_t o_xh = putf(t->xs_h, nb), o_xhei = putf(t->xs_hei, nb), o_xheii = putf(t->xs_heii, nb);
  const size_t o_tph = putf(tph.data(), nb), o_tphe = putf(tphe.data(), nb), o_tpheii = putf(tpheii.data(), nb);
  const size_t o_tk = putf(t->tk, t->ntk);
  const float *lgs[3] = {t->lg_hi, t->lg_hei, t->lg_heii};
  const float *nug[3] = {t->nu_gamma_hi, t->nu_gamma_hei, t->nu_gamma_heii};
  size_t o_lg[3], o_edge[3];
  std::vector<int> pair(3 * (size_t)nb, -1);
  int last_edge[3];
  for (int k = 0; k < 3; ++k) {
    o_lg[k] = putf(lgs[k], (size_t)t->ntk * nlim[k]);
    const std::vector<int> ep = edge_pointers(nu, nb, nug[k], nlim[k]);
    for (int p = 0; p < nlim[k] / 2; ++p) {
      const int ilow = ep[2 * p], iup = ep[2 * p + 1];
      if (iup == ilow || ilow < 1 || iup > nb)
        return set_error(MC_ERR_ARG, "emission tables: frequency grid too coarse for gamma edge %d", 2 * p + 1);
      for (int j = ilow; j <= iup - 1; ++j) pair[(size_t)k * nb + j - 1] = p;
    }
    o_edge[k] = I.size();
    for (int v : ep) I.push_back(v - 1);
    last_edge[k] = ep[nlim[k] - 1];
  }
  const size_t o_pair = I.size();
  I.insert(I.end(), pair.begin(), pair.end());
  std::vector<float> d(88);
  for (int j = 0; j < 8; ++j)
    for (int k = 0; k < 11; ++k) d[j * 11 + k] = (float)t->gaunt_dd[k * 8 + j];  // d(8, 11) column-major
  const size_t o_gd = putf(d.data(), 88);
  const int nh = t->n_heavy;
  std::vector<int> he(nh), hs(nh), hip(nh), hhi(nh);
  std::vector<float> hg(nh), hnu(nh);
  for (int h = 0; h < nh; ++h) {
    const int32_t *r = t->heavy + 8 * h;
    const int e = elem_index(r[0]);
    if (e < 2 || r[1] < 1 || r[1] > 6 || r[4] < 1 || r[5] < 1 || r[6] < 1 || r[6] > nb || r[7] < 1 || r[7] > nb)
      return set_error(MC_ERR_ARG, "emission tables: heavy ion row %d", h);
    he[h] = e;
    hs[h] = r[1] + 1;
    hg[h] = (float)r[4] / (float)r[5];
    hip[h] = r[6] - 1;
    hhi[h] = r[7] - 1;
    hnu[h] = nu[r[6] - 1];
  }
  const size_t o_he = I.size();
  I.insert(I.end(), he.begin(), he.end());
  const size_t o_hs = I.size();
  I.insert(I.end(), hs.begin(), hs.end());
  const size_t o_hip = I.size();
  I.insert(I.end(), hip.begin(), hip.end());
  const size_t o_hhi = I.size();
  I.insert(I.end(), hhi.begin(), hhi.end());
  const size_t o_hg = putf(hg.data(), nh), o_hnu = putf(hnu.data(), nh);
  const size_t o_xso = putf(t->xs_outer, (size_t)nh * nb);
  const int ns = t->n_sizes;
  if (ns < 0 || ns > mcg::kEmiMaxSizes || (ns > 0 && (!t->xs_abs || !t->grain_weight || !t->ndust)))
    return set_error(MC_ERR_ARG, "emission tables: 0..%d grain sizes with xs_abs, grain_weight, ndust",
                     mcg::kEmiMaxSizes);
  size_t o_xa = 0, o_gw = 0, o_nd = 0;
  const size_t o_wf = putf(t->wid_flx, nb);
  if (ns > 0) {
    o_xa = putf(t->xs_abs, (size_t)ns * nb);
    o_gw = putf(t->grain_weight, ns);
    o_nd = putf(t->ndust, (size_t)c->nc + 1);
  }
  const size_t o_hei = putf(t->hei_rec, 34 * 3 * 4);
  float hi_sum = 0.f, heii_sum = 0.f;
  for (int iup = 3; iup <= 15; ++iup)
    for (int ilow = 2; ilow <= std::min(8, iup - 1); ++ilow) hi_sum += t->hi_rec[iup * 9 + ilow];
  for (int iup = 3; iup <= 30; ++iup)
    for (int ilow = 2; ilow <= std::min(16, iup - 1); ++ilow) heii_sum += t->heii_rec[iup * 17 + ilow];
  // one buffer: floats first, then ints (both 4-byte)
  const size_t nf = F.size();
  if (c->e_tab.bytes != (nf + I.size()) * 4) {
    if (c->e_tab.p) { cudaFree(c->e_tab.p); c->e_tab.p = nullptr; c->e_tab.bytes = 0; }
    MC_CUDA(c->e_tab.alloc((nf + I.size()) * 4));
  }
  cudaStream_t s = c->stream;
  MC_CUDA(cudaMemcpyAsync(c->e_tab.p, F.data(), nf * 4, cudaMemcpyHostToDevice, s));
  MC_CUDA(cudaMemcpyAsync((char *)c->e_tab.p + nf * 4, I.data(), I.size() * 4, cudaMemcpyHostToDevice, s));
  MC_CUDA(cudaStreamSynchronize(s));  // the host vectors go out of scope
  const float *fb = c->e_tab.as<float>();
  const int *ib = (const int *)(fb + nf);
  mcg::EmiArgs &E = c->emi;
  E = mcg::EmiArgs{};
  E.nb = nb;
  E.nu = fb + o_nu; E.lnu = fb + o_lnu; E.wid = fb + o_wid;
  E.xs_h = fb + o_xh; E.xs_hei = fb + o_xhei; E.xs_heii = fb + o_xheii;
  E.tp_hi = fb + o_tph; E.tp_hei = fb + o_tphe; E.tp_heii = fb + o_tpheii;
  E.pair = ib + o_pair;
  for (int k = 0; k < 3; ++k) { E.nlim[k] = nlim[k]; E.lg[k] = fb + o_lg[k]; E.edge[k] = ib + o_edge[k]; }
  E.ntk = t->ntk;
  E.tk = fb + o_tk;
  const int pH = locate_host(nu, nb, 0.99946f), pHeI = locate_host(nu, nb, 1.80802f), pHeII = locate_host(nu, nb, 4.0f);
  if (pH < 1 || pHeI < 1 || pHeII < 1) return set_error(MC_ERR_ARG, "emission tables: thresholds below the grid");
  E.p_milne[0] = pH - 1; E.p_milne[1] = pHeI - 1; E.p_milne[2] = pHeII - 1;
  // the HeI and HeII Milne ranges nest inside the HI one (fb_ff :438-470)
  E.p_from[0] = pH - 1;
  E.p_from[1] = std::max(pH, last_edge[1]) - 1;
  E.p_from[2] = std::max(E.p_from[1] + 1, last_edge[2]) - 1;
  E.gaunt_d = fb + o_gd;
  E.nheavy = nh;
  E.h_e = ib + o_he; E.h_stage = ib + o_hs; E.h_ip = ib + o_hip; E.h_hi = ib + o_hhi;
  E.h_g = fb + o_hg; E.h_nuip = fb + o_hnu; E.xs_outer = fb + o_xso;
  E.j2 = locate_host(nu, nb, 1.45673f) - 1;
  for (int i = 0; i < 4; ++i) {
    E.ly_bin[i] = locate_host(nu, nb, t->heii_lyman[2 * i + 1]) - 1;
    E.ly_data[i] = t->heii_lyman[2 * i];
  }
  E.hi_rec_sum = hi_sum;
  E.heii_rec_sum = heii_sum;
  E.hei_rec = fb + o_hei;
  E.nsizes = ns;
  E.widflx = fb + o_wf;
  E.xs_abs = ns ? fb + o_xa : nullptr;
  E.gw = ns ? fb + o_gw : nullptr;
  E.ndust = ns ? fb + o_nd : nullptr;
  E.t_sub = t->t_sublime;
  // fourPi hcRyd constant 1e20 1e20 of fb_ff (:429-527), formed in FP64 (1e40 is not an FP32 number)
  E.milne_c = (float)((double)(4.f * 3.141592654f) * 2.1799153e-11 * (double)4.9874105e-6f * 1e40);
  c->e_ready = true;
  return MC_OK;
}

extern "C" mc_status mc_ctx_build_emission(mc_ctx_t *c, float *ms) {
  NvtxRange nvtx_range("mc emission CDFs");
  if (!c) return set_error(MC_ERR_ARG, "ctx is required");
  if (!c->e_ready) return set_error(MC_ERR_ARG, "mc_ctx_set_emission_tables has not been called");
  const int nc1 = c->nc + 1, nb = c->nb;
  const bool gas = (c->flags & MC_FLAG_GAS) != 0;
  if (gas && !c->u_ready) return set_error(MC_ERR_ARG, "mc_ctx_set_update_tables has not been called");
  if (gas && !c->s_ready) return set_error(MC_ERR_ARG, "mc_ctx_set_cell_state has not been called");
  if (!gas && c->emi.nsizes == 0) return set_error(MC_ERR_ARG, "a dust-only grid needs grains in the emission tables");
  if (c->emi.nsizes > 0 && c->d_tdust.p && c->d_nsizes != c->emi.nsizes)
    return set_error(MC_ERR_ARG, "grain temperatures of %d sizes, emission tables of %d", c->d_nsizes, c->emi.nsizes);
  cudaStream_t s = c->stream;
  mc_status st;
  if ((st = ensure_line_totals(c))) return st;
  if (!gas && !c->dust_cdf.p) {
    MC_CUDA(c->dust_cdf.alloc((size_t)nc1 * nb * sizeof(float)));
    std::vector<float> one(nb, 1.f);
    MC_CUDA(cudaMemcpyAsync(c->dust_cdf.p, one.data(), nb * sizeof(float), cudaMemcpyHostToDevice, s));
    MC_CUDA(cudaStreamSynchronize(s));
    c->g.dust_cdf = c->dust_cdf.as<float>();
  }
  if (gas && !c->rec_cdf.p) {
    MC_CUDA(c->rec_cdf.alloc((size_t)nc1 * nb * sizeof(float)));
    std::vector<float> one(nb, 1.f);  // row 0 (outside the nebula) is never sampled
    MC_CUDA(cudaMemcpyAsync(c->rec_cdf.p, one.data(), nb * sizeof(float), cudaMemcpyHostToDevice, s));
    MC_CUDA(cudaStreamSynchronize(s));
    c->g.rec_cdf = c->rec_cdf.as<float>();
  }
  if (gas && !c->tlines.p) {
    MC_CUDA(c->tlines.alloc((size_t)nc1 * sizeof(float)));
    MC_CUDA(cudaMemsetAsync(c->tlines.p, 0, (size_t)nc1 * sizeof(float), s));
    c->g.total_lines = c->tlines.as<float>();
  }
  mcg::UpdArgs a{};
  fill_update_tables(c, a);
  mcg::EmiArgs E = c->emi;
  E.nc = c->nc;
  E.te = c->s_te.as<double>(); E.ne = c->s_ne.as<double>(); E.X = c->s_X.as<double>();
  E.forb = c->e_forb.as<float>();
  E.ncel = c->u_ncel;
  E.ab = c->f_ab.as<float>();
  E.rec_cdf = c->rec_cdf.as<float>();
  E.total_lines = c->tlines.as<float>();
  E.gas = gas ? 1 : 0;
  E.tdust = E.nsizes > 0 ? c->d_tdust.as<float>() : nullptr;
  E.hden = c->u_hden.as<double>();
  E.dust_cdf = c->dust_cdf.as<float>();
  if (!gas) a.ncel = 0;  // no forbidden lines without gas
  MC_CUDA(cudaEventRecord(c->ev0, s));
  cudaError_t e = mcg::launch_emission(a, E, c->e_forb.as<float>(), c->e_ok.as<int>(), c->e_list.as<int>(),
                                       c->e_cnt.as<int>(), c->num_sms, s);
  if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "emission launch failed: %s", cudaGetErrorString(e));
  MC_CUDA(cudaEventRecord(c->ev1, s));
  MC_CUDA(cudaEventSynchronize(c->ev1));
  if (ms) MC_CUDA(cudaEventElapsedTime(ms, c->ev0, c->ev1));
  return MC_OK;
}

extern "C" mc_status mc_ctx_get_emission(mc_ctx_t *c, float *rec_rows, float *total_lines) {
  if (!c) return set_error(MC_ERR_ARG, "ctx is required");
  const size_t nc1 = (size_t)c->nc + 1;
  if (rec_rows) {
    if (!c->rec_cdf.p) return set_error(MC_ERR_ARG, "no emission CDF on the device");
    MC_CUDA(cudaMemcpyAsync(rec_rows, c->rec_cdf.p, nc1 * c->nb * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  }
  if (total_lines) {
    if (!c->tlines.p) return set_error(MC_ERR_ARG, "no totalLines on the device");
    MC_CUDA(cudaMemcpyAsync(total_lines, c->tlines.p, nc1 * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
  }
  MC_CUDA(cudaStreamSynchronize(c->stream));
  return MC_OK;
}

extern "C" mc_status mc_ctx_get_dust_emission(mc_ctx_t *c, float *dust_rows) {
  if (!c || !dust_rows) return set_error(MC_ERR_ARG, "ctx and dust_rows are required");
  if (!c->dust_cdf.p) return set_error(MC_ERR_ARG, "no dust-emission CDF on the device");
  MC_CUDA(cudaMemcpyAsync(dust_rows, c->dust_cdf.p, ((size_t)c->nc + 1) * c->nb * sizeof(float),
                          cudaMemcpyDeviceToHost, c->stream));
  MC_CUDA(cudaStreamSynchronize(c->stream));
  return MC_OK;
}

extern "C" mc_status mc_ctx_set_tuning(mc_ctx_t *c, int32_t refill_min, int32_t inner_steps) {
  if (!c) return set_error(MC_ERR_ARG, "ctx is NULL");
  if (refill_min < 1 || refill_min > 32 || inner_steps < 1 || inner_steps > 64)
    return set_error(MC_ERR_ARG, "refill_min must be 1..32 and inner_steps 1..64");
  c->refill_min = refill_min;
  c->inner_steps = inner_steps;
  return MC_OK;
}

extern "C" mc_status mc_ctx_get_tuning(mc_ctx_t *c, int32_t *refill_min, int32_t *inner_steps) {
  if (!c) return set_error(MC_ERR_ARG, "ctx is NULL");
  if (refill_min) *refill_min = c->refill_min;
  if (inner_steps) *inner_steps = c->inner_steps;
  return MC_OK;
}

extern "C" mc_status mc_ctx_get_opacity(mc_ctx_t *c, float *out) {
  if (!c || !out) return set_error(MC_ERR_ARG, "ctx and opacity are required");
  MC_CUDA(cudaMemcpyAsync(out, c->opacity.p, (size_t)(c->nc + 1) * c->nb * sizeof(float), cudaMemcpyDeviceToHost,
                          c->stream));
  MC_CUDA(cudaStreamSynchronize(c->stream));
  return MC_OK;
}

extern "C" mc_status mc_ctx_get_scattering(mc_ctx_t *c, float *out) {
  if (!c || !out) return set_error(MC_ERR_ARG, "ctx and scattering are required");
  if (!c->sca.p) return set_error(MC_ERR_ARG, "the grid has no scattering table");
  MC_CUDA(cudaMemcpyAsync(out, c->sca.p, (size_t)(c->nc + 1) * c->nb * sizeof(float), cudaMemcpyDeviceToHost,
                          c->stream));
  MC_CUDA(cudaStreamSynchronize(c->stream));
  return MC_OK;
}

extern "C" mc_status mc_ctx_set_fixed_opacity(mc_ctx_t *c, int32_t nrows, const float *den, const float *xs) {
  if (!c || nrows < 0 || nrows > 16 || (nrows > 0 && (!den || !xs)))
    return set_error(MC_ERR_ARG, "ctx, 0..16 rows, den and xs are required");
  const size_t nc1 = (size_t)c->nc + 1;
  mc_status st;
  if (nrows > 0 && ((st = put_buf(c->o_fix_den, den, nrows * nc1 * sizeof(float), c->stream)) ||
                    (st = put_buf(c->o_fix_xs, xs, (size_t)nrows * c->nb * sizeof(float), c->stream))))
    return st;
  MC_CUDA(cudaStreamSynchronize(c->stream));
  c->o_nfix = nrows;
  return MC_OK;
}

extern "C" mc_status mc_ctx_set_grain_opacity(mc_ctx_t *c, int32_t nsizes, const float *xs_ext, const float *xs_sca,
                                             const float *weight, const float *ndust, float t_sublime) {
  if (!c) return set_error(MC_ERR_ARG, "ctx is NULL");
  if (nsizes == 0) { c->go_n = 0; return MC_OK; }
  if (nsizes < 0 || nsizes > 32) return set_error(MC_ERR_ARG, "grain opacity: nsizes must be 0..32 (got %d)", nsizes);
  if (!xs_ext || !xs_sca || !weight || !ndust) return set_error(MC_ERR_ARG, "grain opacity: arrays are required");
  if (!c->sca.p) return set_error(MC_ERR_ARG, "grain opacity: the grid has no scattering table (not a dusty grid)");
  if (!(t_sublime > 0.f)) return set_error(MC_ERR_ARG, "grain opacity: t_sublime must be > 0");
  const int nc1 = c->nc + 1, nb = c->nb;
  mc_status st;
  if ((st = put_buf(c->go_ext, xs_ext, (size_t)nsizes * nb * sizeof(float), c->stream)) ||
      (st = put_buf(c->go_sca, xs_sca, (size_t)nsizes * nb * sizeof(float), c->stream)) ||
      (st = put_buf(c->go_w, weight, (size_t)nsizes * sizeof(float), c->stream)) ||
      (st = put_buf(c->go_nd, ndust, (size_t)nc1 * sizeof(float), c->stream)) ||
      (st = put_buf(c->go_den, nullptr, (size_t)nsizes * nc1 * sizeof(float), c->stream)))
    return st;
  MC_CUDA(cudaStreamSynchronize(c->stream));
  c->go_n = nsizes;
  c->go_tsub = t_sublime;
  return MC_OK;
}

extern "C" mc_status mc_ctx_set_res_lines(mc_ctx_t *c, const int32_t *counts) {
  if (!c) return set_error(MC_ERR_ARG, "ctx is NULL");
  c->res_per_star = 0;
  c->res_ncell = 0;
  if (!counts) return MC_OK;
  const int nc1 = c->nc + 1;
  long long tot = 0;
  for (int i = 1; i < nc1; ++i) {
    if (counts[i] < 0) return set_error(MC_ERR_ARG, "resonance-line packets: cell %d has %d", i, counts[i]);
    tot += counts[i];
  }
  if (tot == 0) return MC_OK;
  if (tot >= (1ll << 31)) return set_error(MC_ERR_ARG, "resonance-line packets: 2^31 or more per star");
  std::vector<int32_t> act((size_t)c->nx * c->ny * c->nz);
  MC_CUDA(cudaMemcpy(act.data(), c->active.p, act.size() * sizeof(int32_t), cudaMemcpyDeviceToHost));
  std::vector<uint32_t> cells;
  std::vector<long long> prefix(1, 0);
  for (int ix = 1; ix <= c->nx; ++ix)  // the reference's loop order: x outer, z inner
    for (int iy = 1; iy <= c->ny; ++iy)
      for (int iz = 1; iz <= c->nz; ++iz) {
        const int a = act[(size_t)(ix - 1) + (size_t)c->nx * ((iy - 1) + (size_t)c->ny * (iz - 1))];
        if (a <= 0 || a >= nc1 || counts[a] == 0) continue;
        cells.push_back(mcg::pack_cell_host(ix, iy, iz));
        prefix.push_back(prefix.back() + counts[a]);
      }
  mc_status st;
  if ((st = put_buf(c->res_cells, cells.data(), cells.size() * sizeof(uint32_t), c->stream)) ||
      (st = put_buf(c->res_prefix, prefix.data(), prefix.size() * sizeof(long long), c->stream)))
    return st;
  MC_CUDA(cudaStreamSynchronize(c->stream));
  c->res_ncell = (int)cells.size();
  c->res_per_star = prefix.back();
  return MC_OK;
}

extern "C" mc_status mc_ctx_opacity_from_state(mc_ctx_t *c, int32_t nspecies, const int32_t *species,
                                              const float *xs, int32_t method, double *kernel_ms) {
  NvtxRange nvtx_range("mc opacity");
  if (!c || !species || !xs) return set_error(MC_ERR_ARG, "ctx, species and xs are required");
  if (!c->u_ready || !c->s_ready) return set_error(MC_ERR_ARG, "cell state or tables missing");
  if (nspecies < 1 || nspecies + c->o_nfix + c->go_n > 64)
    return set_error(MC_ERR_ARG, "nspecies must be 1..%d (got %d)", 64 - c->o_nfix - c->go_n, nspecies);
  if (method != MC_OPAC_FP32 && method != MC_OPAC_BF16X3) return set_error(MC_ERR_ARG, "unknown opacity method");
  std::vector<int32_t> se(nspecies), ss(nspecies);
  for (int k = 0; k < nspecies; ++k) {
    se[k] = elem_index(species[2 * k]);
    ss[k] = species[2 * k + 1];
    if (se[k] < 0 || ss[k] < 1 || ss[k] > 7) return set_error(MC_ERR_ARG, "species %d: bad (Z, stage)", k);
  }
  const int nc1 = c->nc + 1, nb = c->nb;
  cudaStream_t s = c->stream;
  mc_status st;
  const int nrows = nspecies + c->o_nfix + c->go_n;
  const int g0 = nspecies + c->o_nfix;  // the grains' rows follow the fixed ones
  if ((st = put_buf(c->s_spe, se.data(), nspecies * sizeof(int32_t), s)) ||
      (st = put_buf(c->s_sps, ss.data(), nspecies * sizeof(int32_t), s)) ||
      (st = put_buf(c->s_xs, nullptr, (size_t)nrows * nb * sizeof(float), s)) ||
      (st = put_buf(c->s_den, nullptr, (size_t)nrows * nc1 * sizeof(float), s)) ||
      (st = put_buf(c->s_err, nullptr, sizeof(int), s)))
    return st;
  MC_CUDA(cudaMemcpyAsync(c->s_xs.p, xs, (size_t)nspecies * nb * sizeof(float), cudaMemcpyHostToDevice, s));
  if (c->o_nfix > 0) {
    // the fixed rows follow the species: their densities and cross-sections
    MC_CUDA(cudaMemcpyAsync(c->s_xs.as<float>() + (size_t)nspecies * nb, c->o_fix_xs.p,
                            (size_t)c->o_nfix * nb * sizeof(float), cudaMemcpyDeviceToDevice, s));
    MC_CUDA(cudaMemcpyAsync(c->s_den.as<float>() + (size_t)nspecies * nc1, c->o_fix_den.p,
                            (size_t)c->o_nfix * nc1 * sizeof(float), cudaMemcpyDeviceToDevice, s));
  }
  if (c->go_n > 0)
    MC_CUDA(cudaMemcpyAsync(c->s_xs.as<float>() + (size_t)g0 * nb, c->go_ext.p, (size_t)c->go_n * nb * sizeof(float),
                            cudaMemcpyDeviceToDevice, s));
  MC_CUDA(cudaStreamSynchronize(s));  // xs is the caller's (pageable) array
  MC_CUDA(cudaMemsetAsync(c->s_err.p, 0, sizeof(int), s));
  cudaEvent_t e0, e1;
  MC_CUDA(cudaEventCreate(&e0));
  MC_CUDA(cudaEventCreate(&e1));
  MC_CUDA(cudaEventRecord(e0, s));
  cudaError_t e = mcg::launch_species(c->nc, nspecies, c->s_spe.as<int>(), c->s_sps.as<int>(), c->s_X.as<double>(),
                                      c->u_ab.as<double>(), c->u_hden.as<double>(), c->s_den.as<float>(), c->num_sms, s);
  // the grains' densities from the grain temperatures (sublimated sizes drop out)
  const float *tdust = (c->go_n > 0 && c->d_tdust.p && c->d_nsizes == c->go_n) ? c->d_tdust.as<float>() : nullptr;
  if (e == cudaSuccess && c->go_n > 0)
    e = mcg::launch_grain_density(nc1, c->go_n, c->go_w.as<float>(), c->go_nd.as<float>(), tdust, c->go_tsub,
                                  c->s_den.as<float>() + (size_t)g0 * nc1, c->num_sms, s);
  if (e == cudaSuccess)
    e = mcg::launch_opacity(method, nc1, nrows, nb, c->s_den.as<float>(), c->s_xs.as<float>(), nullptr,
                            c->opacity.as<float>(), c->s_err.as<int>(), c->num_sms, s);
  // and the scattering table of the grains that are left
  if (e == cudaSuccess && c->go_n > 0)
    e = mcg::launch_opacity(method, nc1, c->go_n, nb, c->s_den.as<float>() + (size_t)g0 * nc1, c->go_sca.as<float>(),
                            nullptr, c->sca.as<float>(), c->s_err.as<int>(), c->num_sms, s);
  if (e == cudaSuccess && !c->identity)
    e = mcg::launch_wave_expand(c->opacity.as<float>(), c->opac_m.as<float>(), c->lin2cell.as<int32_t>(), c->ncell3,
                                nc1, nb, s);
  if (e == cudaSuccess && !c->identity && c->go_n > 0)
    e = mcg::launch_wave_expand(c->sca.as<float>(), c->sca_m.as<float>(), c->lin2cell.as<int32_t>(), c->ncell3, nc1,
                                nb, s);
  if (e != cudaSuccess) return set_error(MC_ERR_CUDA, "opacity rebuild failed: %s", cudaGetErrorString(e));
  MC_CUDA(cudaEventRecord(e1, s));
  int herr = 0;
  MC_CUDA(cudaMemcpyAsync(&herr, c->s_err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  MC_CUDA(cudaStreamSynchronize(s));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0); cudaEventDestroy(e1);
  if (kernel_ms) *kernel_ms = ms;
  if (herr) return set_error((mc_status)herr, "opacity kernel: tensor-core wait timed out");
  return MC_OK;
}

namespace {

__global__ void widen_kernel(const float *__restrict__ in, double *__restrict__ out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = (double)in[i];
}
__global__ void narrow_kernel(const double *__restrict__ in, float *__restrict__ out, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    out[i] = mcg::f64_to_f32_rn(in[i]);
}

// The first frequency bin a packet can march in: on a gas-only grid the
// packets below ionEdge(1) escape before any march (energyPacketRun,
// photon_mod.f90:370-465), so their opacity rows are never read.
int first_marched_bin(const mc_grid_t *g) {
  if (g->flags & MC_FLAG_DUST) return 0;
  int b = 0;
  while (b < g->nbins && g->nu_array[b] < g->ion_edge1) ++b;
  return b;
}

// flag[row] = 1 when row `row` of a [rows][len] array holds a nonzero value
// (grid: x tiles the row, y = row; flag zeroed before)
__global__ void row_nonzero_kernel(const double *__restrict__ a, long long len, unsigned char *flag,
                                   float *__restrict__ narrow) {
  const double *r = a + (long long)blockIdx.y * len;
  float *o = narrow ? narrow + (long long)blockIdx.y * len : nullptr;
  bool nz = false;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < len; i += (long long)gridDim.x * blockDim.x) {
    const double v = r[i];
    nz |= v != 0.0;
    if (o) o[i] = mcg::f64_to_f32_rn(v);
  }
  if (__syncthreads_or(nz) && threadIdx.x == 0) flag[blockIdx.y] = 1;
}

// the nonzero entries of a[0..n) as (index, value) pairs, in no set order,
// values as float (f32) or double: *count ends at their number; pairs beyond
// `cap` are not written
__global__ void compact_nonzero_kernel(const double *__restrict__ a, unsigned long long n, uint32_t *idx, void *val,
                                       int f32, unsigned long long cap, unsigned long long *count) {
  const unsigned int lane = threadIdx.x & 31;
  for (unsigned long long b = (blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x) & ~31ull; b < n;
       b += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned long long i = b + lane;
    const double v = i < n ? a[i] : 0.0;
    const unsigned int m = __ballot_sync(0xffffffffu, v != 0.0);
    if (!m) continue;
    unsigned long long base = 0;
    if (lane == 0) base = atomicAdd(count, (unsigned long long)__popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (v != 0.0) {
      const unsigned long long slot = base + __popc(m & ((1u << lane) - 1u));
      if (slot < cap) {
        idx[slot] = (uint32_t)i;
        if (f32) ((float *)val)[slot] = mcg::f64_to_f32_rn(v);
        else ((double *)val)[slot] = v;
      }
    }
  }
}

// out[idx[k]] = val[k] for k < n, floats (f32) or doubles (out: a
// device-visible view of the caller's pinned host array)
__global__ void scatter_pairs_kernel(const uint32_t *__restrict__ idx, const void *val, unsigned long long n, int f32,
                                     void *out) {
  for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n;
       k += (unsigned long long)gridDim.x * blockDim.x) {
    if (f32) ((float *)out)[idx[k]] = ((const float *)val)[k];
    else ((double *)out)[idx[k]] = ((const double *)val)[k];
  }
}

// a[idx[k]] = 0 for the n compacted entries
__global__ void zero_at_kernel(const uint32_t *__restrict__ idx, unsigned long long n, double *a) {
  for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n;
       k += (unsigned long long)gridDim.x * blockDim.x)
    a[idx[k]] = 0.0;
}


// MC_RUN_HOST_ZEROED download of one estimator [rows][len] (FP64 on the
// device; rounded to FP32 into `stage` in the same pass that finds the
// nonzero rows, when stage is given): the rows that hold a nonzero value, in
// one copy per run of such rows.
// With rezero, the rows are cleared on the device once copied.
mc_status download_rows(mc_ctx *c, const DBuf &d, const DBuf *stage, void *h, long long rows, long long len,
                        bool rezero) {
  cudaStream_t s = c->stream;
  mc_status st;
  if (c->z_mask.bytes != (size_t)rows && (st = put_buf(c->z_mask, nullptr, (size_t)rows, s))) return st;
  MC_CUDA(cudaMemsetAsync(c->z_mask.p, 0, (size_t)rows, s));
  const unsigned int tiles = (unsigned int)std::max(1ll, std::min(64ll, len / 4096));
  row_nonzero_kernel<<<dim3(tiles, (unsigned int)rows), 256, 0, s>>>(d.as<double>(), len, c->z_mask.as<unsigned char>(),
                                                                    stage ? stage->as<float>() : nullptr);
  MC_CUDA(cudaGetLastError());
  std::vector<unsigned char> mask((size_t)rows);
  MC_CUDA(cudaMemcpyAsync(mask.data(), c->z_mask.p, (size_t)rows, cudaMemcpyDeviceToHost, s));
  c->xfer_d2h += rows;
  MC_CUDA(cudaStreamSynchronize(s));
  const size_t elt = stage ? sizeof(float) : sizeof(double);
  const char *src = stage ? (const char *)stage->p : (const char *)d.p;
  for (long long r = 0; r < rows;) {
    if (!mask[r]) { ++r; continue; }
    long long e = r;
    while (e < rows && mask[e]) ++e;
    MC_CUDA(cudaMemcpyAsync((char *)h + r * len * elt, src + r * len * elt, (size_t)((e - r) * len) * elt,
                            cudaMemcpyDeviceToHost, s));
    c->xfer_d2h += (long long)((e - r) * len) * (long long)elt;
    if (rezero) MC_CUDA(cudaMemsetAsync((char *)d.p + r * len * sizeof(double), 0, (size_t)((e - r) * len) * sizeof(double), s));
    r = e;
  }
  return MC_OK;
}

// MC_RUN_HOST_ZEROED download of escapedPackets: its nonzero entries,
// compacted on the device and scattered into the caller's array (by the
// device into pinned memory, by the host otherwise); a dense copy when they
// are too many for the pair buffers.
// The compaction and the count's copy are queued on stream s by
// sparse_begin, which returns at once; sparse_end waits for the count and
// queues the rest on the same stream.
mc_status sparse_begin(mc_ctx *c, const DBuf &d, bool f32, cudaStream_t s) {
  mc_status st;
  const unsigned long long n = d.bytes / sizeof(double);
  const unsigned long long cap = std::min<unsigned long long>(n, 1ull << 24);
  if (c->z_idx.bytes < cap * sizeof(uint32_t) && (st = put_buf(c->z_idx, nullptr, cap * sizeof(uint32_t), s))) return st;
  if (c->z_val.bytes < cap * sizeof(double) && (st = put_buf(c->z_val, nullptr, cap * sizeof(double), s))) return st;
  if (!c->z_cnt.p && (st = put_buf(c->z_cnt, nullptr, sizeof(unsigned long long), s))) return st;
  MC_CUDA(cudaMemsetAsync(c->z_cnt.p, 0, sizeof(unsigned long long), s));
  compact_nonzero_kernel<<<c->num_sms * 8, 256, 0, s>>>(d.as<double>(), n, c->z_idx.as<uint32_t>(), c->z_val.p,
                                                         f32 ? 1 : 0, cap, c->z_cnt.as<unsigned long long>());
  MC_CUDA(cudaGetLastError());
  if (!c->h_cnt && cudaHostAlloc((void **)&c->h_cnt, sizeof(unsigned long long), cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    c->h_cnt = nullptr;
    return set_error(MC_ERR_CUDA, "pinned count allocation failed");
  }
  MC_CUDA(cudaMemcpyAsync(c->h_cnt, c->z_cnt.p, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  return MC_OK;
}

mc_status sparse_end(mc_ctx *c, const DBuf &d, void *h, bool f32, bool rezero, cudaStream_t s) {
  const unsigned long long n = d.bytes / sizeof(double);
  const unsigned long long cap = std::min<unsigned long long>(n, 1ull << 24);
  MC_CUDA(cudaStreamSynchronize(s));
  const unsigned long long cnt = *c->h_cnt;
  const size_t elt = f32 ? sizeof(float) : sizeof(double);
  c->xfer_d2h += (long long)sizeof(unsigned long long);
  if (cnt > cap) {
    if (!f32) {
      MC_CUDA(cudaMemcpyAsync(h, d.p, d.bytes, cudaMemcpyDeviceToHost, s));
    } else {
      narrow_kernel<<<c->num_sms * 8, 256, 0, s>>>(d.as<double>(), c->stage_e.as<float>(), (size_t)n);
      MC_CUDA(cudaGetLastError());
      MC_CUDA(cudaMemcpyAsync(h, c->stage_e.p, n * sizeof(float), cudaMemcpyDeviceToHost, s));
    }
    c->xfer_d2h += (long long)(n * elt);
    if (rezero) MC_CUDA(cudaMemsetAsync(d.p, 0, d.bytes, s));
    return MC_OK;
  }
  if (cnt == 0) return MC_OK;
  if (rezero) {  // the pairs hold the values: the entries can be cleared now
    zero_at_kernel<<<(unsigned int)std::min<unsigned long long>((unsigned long long)c->num_sms * 4, (cnt + 255) / 256),
                     256, 0, s>>>(c->z_idx.as<uint32_t>(), cnt, d.as<double>());
    MC_CUDA(cudaGetLastError());
  }
  // the pairs cross to the host either way: written there by the device, or
  // copied and scattered by the host
  c->xfer_d2h += (long long)(cnt * (sizeof(uint32_t) + elt));
  if (void *hv = pinned_view(h)) {
    const unsigned int blocks = (unsigned int)std::min<unsigned long long>((unsigned long long)c->num_sms * 4,
                                                                           (cnt + 255) / 256);
    scatter_pairs_kernel<<<blocks, 256, 0, s>>>(c->z_idx.as<uint32_t>(), c->z_val.p, cnt, f32 ? 1 : 0, hv);
    MC_CUDA(cudaGetLastError());
    return MC_OK;
  }
  std::vector<uint32_t> ix(cnt);
  std::vector<char> vl(cnt * elt);
  MC_CUDA(cudaMemcpyAsync(ix.data(), c->z_idx.p, cnt * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  MC_CUDA(cudaMemcpyAsync(vl.data(), c->z_val.p, cnt * elt, cudaMemcpyDeviceToHost, s));
  MC_CUDA(cudaStreamSynchronize(s));
  if (f32) {
    float *out = (float *)h;
    const float *v = (const float *)vl.data();
    for (unsigned long long k = 0; k < cnt; ++k) out[ix[k]] = v[k];
  } else {
    double *out = (double *)h;
    const double *v = (const double *)vl.data();
    for (unsigned long long k = 0; k < cnt; ++k) out[ix[k]] = v[k];
  }
  return MC_OK;
}

// the drop-in call with FP64 (f32 = false) or FP32 host estimators
mc_status transport_run_impl(const mc_grid_t *g, const mc_source_t *src, int32_t nsrc, const mc_run_opts_t *o,
                             void *jste, void *jdif, void *escaped, bool f32, mc_stats_t *stats) {
  NvtxRange nvtx_range("mc drop-in transport");
  if (!jste) return set_error(MC_ERR_ARG, "jste is NULL");
  if (!o) return set_error(MC_ERR_ARG, "opts is NULL");
  if (g && (g->flags & MC_FLAG_DEBUG) && !jdif) return set_error(MC_ERR_ARG, "debug grid needs jdif");
  mc_status st = check_grid(g);
  if (st) return st;
  std::lock_guard<std::mutex> lock(g_cache_mutex);
  mc_ctx *c = g_cached;
  int dev = 0;
  cudaGetDevice(&dev);
  bool reuse = c && c->device == dev && c->nx == g->nx && c->ny == g->ny && c->nz == g->nz && c->nc == g->ncells &&
               c->nb == g->nbins && c->flags == g->flags && c->n_angle == g->n_angle;
  if (reuse) {
    if (!c->side && (cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess ||
                     cudaEventCreateWithFlags(&c->ev_side0, cudaEventDisableTiming) != cudaSuccess ||
                     cudaEventCreateWithFlags(&c->ev_cdf, cudaEventDisableTiming) != cudaSuccess))
      return set_error(MC_ERR_CUDA, "side stream creation failed");
    // recPDF on the side stream, after whatever the context's stream still runs
    MC_CUDA(cudaEventRecord(c->ev_side0, c->stream));
    MC_CUDA(cudaStreamWaitEvent(c->side, c->ev_side0, 0));
    bool geo_ok = true;
    if (same_geometry(c, g)) {
      c->g.gc[0] = g->geo_corr[0]; c->g.gc[1] = g->geo_corr[1]; c->g.gc[2] = g->geo_corr[2];
      c->g.rout = g->r_out;
      c->g.ion_edge1 = g->ion_edge1;
    } else {
      geo_ok = refresh_geometry(c, g) == MC_OK;
    }
    if (!geo_ok || upload_arrays(c, g, false, c->side, first_marched_bin(g)) != MC_OK) {
      cudaStreamSynchronize(c->side);
      reuse = false;
    } else {
      MC_CUDA(cudaEventRecord(c->ev_cdf, c->side));
      c->cdf_pending = true;
    }
  }
  if (!reuse) {
    if (c) mc_ctx_destroy(c);
    g_cached = nullptr;
    if ((st = mc_ctx_create(g, &c))) return st;
    g_cached = c;
    same_geometry(c, g);  // records it
    // a new context uploads the whole grid
    const size_t plane = (size_t)(g->ncells + 1) * g->nbins * sizeof(float);
    const size_t n3 = (size_t)g->nx * g->ny * g->nz;
    c->xfer_h2d = (long long)(plane * (1 + (g->sca_opac ? 1 : 0) + (g->rec_pdf ? 1 : 0) + (g->dust_pdf ? 1 : 0)) +
                              (g->nx + g->ny + g->nz) * (sizeof(float) * 2 + sizeof(double)) +
                              2 * n3 * sizeof(int32_t) + g->nbins * sizeof(float) +
                              (g->total_lines ? (size_t)(g->ncells + 1) * sizeof(float) : 0));
  }
  long long h2d = c->xfer_h2d, d2h = 0;
  c->xfer_h2d = 0;
  for (int i = 0; i < nsrc; ++i) h2d += (long long)g->nbins * (long long)sizeof(float);  // the stars' CDFs
  // the estimators accumulate into the caller's arrays: their current
  // values go to the device first, the kernels add to them, and the sums
  // come back (no host-side pass over the arrays).  With MC_RUN_ZERO_FIRST
  // the caller states that its arrays hold zeros (the Fortran driver zeroes
  // them before each iteration, iteration_mod.f90:458-472): the device
  // copies are cleared instead of uploaded.  FP32 arrays go through a staging
  // buffer per array and a widening / narrowing pass on the device.
  const bool hostz = o->run_flags & MC_RUN_HOST_ZEROED;
  const bool zero = (o->run_flags & MC_RUN_ZERO_FIRST) || hostz;
  cudaStream_t s = c->stream;
  struct Item { void *h; DBuf *d; DBuf *stage; } items[3] = {
      {jste, &c->jste, &c->stage_j}, {jdif, &c->jdif, &c->stage_d}, {escaped, &c->esc, &c->stage_e}};
  const bool already_zero = hostz && c->est_zero;
  c->est_zero = false;
  for (auto &it : items) {
    if (!it.d->p) continue;
    const size_t n = it.d->bytes / sizeof(double);
    if (f32 && it.h && (st = put_buf(*it.stage, nullptr, n * sizeof(float), s))) return st;
    if (!it.h || zero) {
      if (!already_zero) MC_CUDA(cudaMemsetAsync(it.d->p, 0, it.d->bytes, s));
    } else if (!f32) {
      MC_CUDA(cudaMemcpyAsync(it.d->p, it.h, it.d->bytes, cudaMemcpyHostToDevice, s));
      h2d += (long long)it.d->bytes;
    } else {
      MC_CUDA(cudaMemcpyAsync(it.stage->p, it.h, n * sizeof(float), cudaMemcpyHostToDevice, s));
      h2d += (long long)(n * sizeof(float));
      widen_kernel<<<c->num_sms * 8, 256, 0, s>>>(it.stage->as<float>(), it.d->as<double>(), n);
      MC_CUDA(cudaGetLastError());
    }
  }
  mc_run_opts_t o2 = *o;
  o2.run_flags &= ~(MC_RUN_ZERO_FIRST | MC_RUN_HOST_ZEROED);
  st = mc_ctx_run(c, src, nsrc, &o2, stats);
  if (st != MC_OK) return st;
  c->xfer_d2h = 0;
  auto counted = [&](mc_status r) {
    if (stats) { stats->h2d_bytes = h2d; stats->d2h_bytes = c->xfer_d2h + d2h; }
    return r;
  };
  if (hostz) {
    // only what the transport made nonzero goes back, and is then cleared
    // on the device (on an identity grid the march adds into these arrays
    // directly), so that the next call starts from zero without a full clear
    const long long len = c->nc + 1;
    bool all = c->identity;
    // the escapes are compacted on the side stream while the Jste rows are
    // scanned and copied on the main one
    cudaStream_t es = s;
    if (c->esc.p && escaped && c->side) {
      if (!c->ev_done) MC_CUDA(cudaEventCreateWithFlags(&c->ev_done, cudaEventDisableTiming));
      MC_CUDA(cudaEventRecord(c->ev_done, s));
      MC_CUDA(cudaStreamWaitEvent(c->side, c->ev_done, 0));
      es = c->side;
    }
    if (c->esc.p && escaped && (st = sparse_begin(c, c->esc, f32, es))) return st;
    for (int k = 0; k < 2; ++k) {
      Item &it = items[k];
      if (!it.d->p) continue;
      if (!it.h) { all = false; continue; }
      const long long n = (long long)(it.d->bytes / sizeof(double));
      if ((st = download_rows(c, *it.d, f32 ? it.stage : nullptr, it.h, n / len, len, c->identity))) return st;
    }
    if (c->esc.p) {
      if (escaped) {
        if ((st = sparse_end(c, c->esc, escaped, f32, c->identity, es))) return st;
      } else {
        all = false;
      }
    }
    MC_CUDA(cudaStreamSynchronize(es));
    MC_CUDA(cudaStreamSynchronize(s));
    c->est_zero = all;
    return counted(MC_OK);
  }
  if (!f32) {
    for (auto &it : items)
      if (it.h && it.d->p) d2h += (long long)it.d->bytes;
    return counted(mc_ctx_download(c, (double *)jste, (double *)jdif, (double *)escaped, 0));
  }
  // narrow each array and start its copy back; the next array's narrowing
  // overlaps the previous copy
  for (auto &it : items) {
    if (!it.h || !it.d->p) continue;
    const size_t n = it.d->bytes / sizeof(double);
    narrow_kernel<<<c->num_sms * 8, 256, 0, s>>>(it.d->as<double>(), it.stage->as<float>(), n);
    MC_CUDA(cudaGetLastError());
    MC_CUDA(cudaMemcpyAsync(it.h, it.stage->p, n * sizeof(float), cudaMemcpyDeviceToHost, s));
    d2h += (long long)(n * sizeof(float));
  }
  MC_CUDA(cudaStreamSynchronize(s));
  return counted(MC_OK);
}

}  // namespace

mc_status mc_transport_run(const mc_grid_t *g, const mc_source_t *src, int32_t nsrc, const mc_run_opts_t *o,
                           double *jste, double *jdif, double *escaped, mc_stats_t *stats) {
  return transport_run_impl(g, src, nsrc, o, jste, jdif, escaped, false, stats);
}

mc_status mc_transport_run_f32(const mc_grid_t *g, const mc_source_t *src, int32_t nsrc, const mc_run_opts_t *o,
                               float *jste, float *jdif, float *escaped, mc_stats_t *stats) {
  return transport_run_impl(g, src, nsrc, o, jste, jdif, escaped, true, stats);
}

mc_status mc_transport_release(void) {
  std::lock_guard<std::mutex> lock(g_cache_mutex);
  if (g_cached) mc_ctx_destroy(g_cached);
  g_cached = nullptr;
  return MC_OK;
}

}  // extern "C"
