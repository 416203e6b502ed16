// transport_wave.cuh -- the chosen GPU form of mocassin's packet transport:
// frequency-sorted wavefront rounds with a persistent march.
//
// energyPacketDriver (source/photon_mod.f90:93-127) runs each packet history
// to its end before the next.  Here all histories advance together, round
// by round:
//
//  round 0 (stellar packets)
//   sample:  every packet draws its frequency (getNu2 on the star's CDF,
//            photon_mod.f90:720-764); non-ionising packets of a gas-only grid
//            escape on the spot (energyPacketRun :370-465) into per-block
//            histograms; the rest are counted per frequency bin.
//  round k >= 1 (packets absorbed in round k-1)
//   sample:  line/continuum choice, getNu2 on the cell's recPDF (or dustPDF),
//            the immediate escape (newPhotonPacket "diffuse" :907-992).
//  every round
//   sort:    counting sort of the round's packets by frequency bin.  Packets
//            in flight at the same time then read opacity(:,nu) and add into
//            Jste(:,nu) of the same few frequency slabs, which stay in L2.
//   emit:    in sorted order, one thread per packet: direction
//            (initPhotonPacket :650-675) and passProb (pathSegment :1181);
//            the march state is written in queue order, so a warp's refill
//            is a coalesced read.
//   march:   persistent kernel; each warp iteration is one pathSegment loop
//            body (:1194-2836) per lane.  Lanes whose packet escaped refill in
//            batches from the queue; an absorbed packet is appended to the
//            next round's list and its lane refills.  Dust scattering stays in
//            the march (it only turns the packet).
//
// Each packet consumes its own Philox stream in the reference draw order, so
// the FP64 instantiation (exact arithmetic, no contraction) reproduces the
// oracle to rounding; the FP32 one multiplies by reciprocals.
//
// Cells are addressed by grid position lin = (z-1) + nz*((y-1) + ny*(x-1)),
// which is active(x,y,z)-1 when every cell is active (the reference numbers
// active cells x outer, z inner, grid_mod.f90:1224-1290): the march then reads
// opacity and adds into Jste in place at row lin+1 without an active lookup.
// Otherwise it uses march-indexed copies and Jste is folded back into rows.
#pragma once

#include "mc_device.cuh"
#include "transport_plain.cuh"
#include "wave_types.cuh"

namespace mcg {

__device__ __forceinline__ int lin_of(const DevGrid &g, int x, int y, int z) {
  return (z - 1) + g.nz * ((y - 1) + g.ny * (x - 1));
}
__device__ __forceinline__ uint32_t pack_cell(int x, int y, int z) {
  return (uint32_t)x | ((uint32_t)y << 10) | ((uint32_t)z << 20);
}
__device__ __forceinline__ void unpack_cell(uint32_t c, int &x, int &y, int &z) {
  x = (int)(c & 1023u); y = (int)((c >> 10) & 1023u); z = (int)((c >> 20) & 1023u);
}
// meta word of a queue entry: nuP (16 bits) | runI (15 bits) | stellar (1 bit)
__device__ __forceinline__ uint32_t pack_meta(int nuP, int runI, bool stellar) {
  return (uint32_t)nuP | ((uint32_t)runI << 16) | (stellar ? 0x80000000u : 0u);
}

// Register-resident draw stream (no indexed local arrays); Replay = false
// compiles the replay reads out.
template <bool Replay> struct RStream {
  uint32_t plo, phi, block;
  uint4 buf;
  int have;
  const double *row;
  int used, stride;
  bool exhausted;

  __device__ __forceinline__ void init(unsigned long long packet, const DevReplay &rp, long long gp) {
    plo = (uint32_t)packet; phi = (uint32_t)(packet >> 32);
    block = 0; have = 0; used = 0; exhausted = false;
    if (Replay) { row = rp.draws + gp * rp.stride; stride = (int)rp.stride; }
    else { row = nullptr; stride = 0; }
  }
  // draws consumed so far (Philox words, or replay draws)
  __device__ __forceinline__ uint32_t consumed() const { return Replay ? (uint32_t)used : block * 4u - (uint32_t)have; }
  // resume after `w` consumed words / draws
  __device__ __forceinline__ void resume(uint32_t w, uint32_t k0, uint32_t k1) {
    if (Replay) { used = (int)w; return; }
    block = (w + 3u) >> 2;
    have = (int)(block * 4u - w);
    if (have > 0) buf = philox4x32_10(make_uint4(plo, phi, block - 1u, 0u), k0, k1);
  }
  __device__ __forceinline__ uint32_t word(uint32_t k0, uint32_t k1) {
    if (have == 0) {
      buf = philox4x32_10(make_uint4(plo, phi, block++, 0u), k0, k1);
      have = 4;
    }
    const uint32_t w = have == 4 ? buf.x : (have == 3 ? buf.y : (have == 2 ? buf.z : buf.w));
    --have;
    return w;
  }
  template <typename Real> __device__ __forceinline__ Real next(uint32_t k0, uint32_t k1) {
    if (Replay) {
      if (used >= stride) { exhausted = true; return (Real)0.5; }
      const double x = row[used++];
      if (sizeof(Real) == 8) return (Real)x;
      return (Real)(floor(x * 16777216.0) * (1.0 / 16777216.0));
    }
    if (sizeof(Real) == 8) {
      const unsigned long long hi = word(k0, k1);
      const unsigned long long lo = word(k0, k1);
      return (Real)((double)((hi << 21) | (lo >> 11)) * (1.0 / 9007199254740992.0));
    }
    return (Real)((float)(word(k0, k1) >> 8) * (1.0f / 16777216.0f));
  }
};

__device__ __forceinline__ int source_of(const DevSources &S, long long gp) {
  int s = 0;
  while (s + 1 < S.nsrc + S.nres && gp >= S.s[s + 1].base) ++s;
  return s;
}

// getNu2 on a monotone row (see transport_plain.cuh).
template <typename Real, bool Replay>
__device__ __forceinline__ int sample_bin(RStream<Replay> &st, uint32_t k0, uint32_t k1, const float *row, int nb,
                                          bool &ok) {
  Real random = st.template next<Real>(k0, k1);
  int i;
  for (i = 1; i <= 10000; ++i) {
    if (random == (Real)0 || random == (Real)1 || random == (Real)0.9999999f) random = st.template next<Real>(k0, k1);
    else break;
  }
  ok = i < 10000;
  int lo = 0, hi = nb;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (random >= (Real)__ldg(row + mid)) lo = mid + 1;
    else hi = mid;
  }
  int nuP = lo < 1 ? 1 : lo;
  if (nuP < nb - 1) nuP = nuP + 1;
  return nuP;
}

// isotropic direction with the reference's retry (randomUnitVector,
// vector_mod.f90:303-314; initPhotonPacket :650-663)
template <typename Real, bool Replay>
__device__ __forceinline__ bool sample_direction(RStream<Replay> &st, uint32_t k0, uint32_t k1, R3<Real> &d) {
  for (int irep = 1; irep <= 1000000; ++irep) {
    const Real r1 = st.template next<Real>(k0, k1);
    const Real ww = (Real)2 * r1 - (Real)1;
    const Real t = sqrt((Real)1 - ww * ww);
    const Real r2 = st.template next<Real>(k0, k1);
    const Real ang = (Real)3.141592654 * ((Real)2 * r2 - (Real)1);
    d = R3<Real>{t * cos(ang), t * sin(ang), ww};
    if (isnan(d.x)) return false;
    if (d.x != (Real)0 && d.y != (Real)0 && d.z != (Real)0) break;
  }
  return true;
}

// origin(2) of a stellar packet: the active cell of the star
__device__ __forceinline__ int origin_of(const DevGrid &g, const DevSource &src) {
  return __ldg(g.active + (src.cell[0] - 1) + (long long)g.nx * ((src.cell[1] - 1) + (long long)g.ny * (src.cell[2] - 1)));
}

// ------------------------------------------------------------ round 0 sample
template <typename Real, bool Replay>
__global__ void __launch_bounds__(256) wave_sample_stellar_kernel(const __grid_constant__ DevGrid g,
                                                                 const __grid_constant__ DevSources S,
                                                                 const __grid_constant__ DevReplay rp,
                                                                 const __grid_constant__ WaveGrid w,
                                                                 DevCounters *cnt) {
  extern __shared__ unsigned int sh[];  // [nb] marching counts, [nsrc*nb] escape counts
  unsigned int *hcount = sh;
  unsigned int *hesc = sh + g.nb;
  const int nh = g.nb * (1 + S.nsrc);
  for (int i = threadIdx.x; i < nh; i += blockDim.x) sh[i] = 0u;
  __syncthreads();
  const bool gas_only = !(g.flags & MC_FLAG_DUST);
  const bool fold = (g.flags & MC_FLAG_SYMMETRIC_XYZ) && !(g.flags & MC_FLAG_MULTISTARS);
  unsigned long long nesc_direct = 0;
  double q = 0.0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long gp = (long long)blockIdx.x * blockDim.x + threadIdx.x; gp < S.total; gp += stride) {
    const int s = source_of(S, gp);
    const DevSource &src = S.s[s];
    RStream<Replay> st;
    st.init((unsigned long long)(gp - src.base), rp, gp);
    bool ok;
    const int nuP = sample_bin<Real, Replay>(st, src.k0, src.k1, src.cdf, g.nb, ok);
    if (!ok || nuP >= g.nb || nuP < 1 || st.exhausted) {
      raise_error(cnt, st.exhausted ? MC_ERR_REPLAY : MC_ERR_BOUNDS, gp);
      w.s_nu[gp] = 0xFFFFu;
      continue;
    }
    const Real nu = (Real)__ldg(g.nu + nuP - 1);
    if (nu > (Real)1) q += (double)((Real)src.delta_e / ((Real)2.1799153e-11f * nu));
    if (gas_only && nu < (Real)g.ion_edge1) {
      w.s_nu[gp] = 0xFFFFu;
      if (g.n_angle > 0) {
        // the direction initPhotonPacket drew picks the viewing-angle plane
        R3<Real> d;
        bool ok = sample_direction<Real, Replay>(st, src.k0, src.k1, d);
        if (fold) { d.x = fabs(d.x); d.y = fabs(d.y); d.z = fabs(d.z); }
        const int view = ok ? escape_view<Real>(g, d.x, d.y, d.z, ok) : 0;
        if (!ok || st.exhausted) { raise_error(cnt, st.exhausted ? MC_ERR_REPLAY : MC_ERR_NAN, gp); continue; }
        add_escape(g, origin_of(g, src), nuP, view, (double)(Real)src.delta_e);
        ++nesc_direct;
      } else {
        atomicAdd(&hesc[s * g.nb + nuP], 1u);
      }
    } else {
      atomicAdd(&hcount[nuP], 1u);
      w.s_nu[gp] = (uint16_t)nuP;
      w.s_words[gp] = st.consumed();
    }
  }
  q = warp_sum(q);
  if ((threadIdx.x & 31) == 0 && q != 0.0) atomicAdd(&cnt->qphot, q);
  __syncthreads();
  for (int i = threadIdx.x; i < g.nb; i += blockDim.x)
    if (hcount[i]) atomicAdd(&w.bin_count[i], hcount[i]);
  unsigned long long nesc = 0;
  for (int i = threadIdx.x; i < g.nb * S.nsrc; i += blockDim.x) {
    const unsigned int c = hesc[i];
    if (!c) continue;
    const int s = i / g.nb, nuP = i % g.nb;
    const DevSource &src = S.s[s];
    if (g.esc) atomicAdd(g.esc + origin_of(g, src) + (long long)(g.nc + 1) * nuP, (double)c * (double)(Real)src.delta_e);
    nesc += c;
  }
  nesc = warp_sum(nesc + nesc_direct);
  if ((threadIdx.x & 31) == 0 && nesc) atomicAdd(&cnt->escaped, nesc);
}

// ----------------------------------------------------- round k >= 1 sample
// Re-emission of absorbed packets (energyPacketRun with "diffuse" or
// "dustEmi", newPhotonPacket :907-1047), up to the frequency draw.
template <typename Real, bool Replay>
__global__ void __launch_bounds__(256) wave_sample_reemit_kernel(const __grid_constant__ DevGrid g,
                                                                const __grid_constant__ DevSources S,
                                                                const __grid_constant__ DevReplay rp,
                                                                const __grid_constant__ WaveGrid w,
                                                                unsigned int n_param, DevCounters *cnt) {
  const unsigned int n_abs = n_param == kDeviceCount ? *w.a_count : n_param;
  if (n_param == kDeviceCount && blockIdx.x == 0 && threadIdx.x == 0) *w.n_round = n_abs;
  extern __shared__ unsigned int sh[];  // [nb] counts
  for (int i = threadIdx.x; i < g.nb; i += blockDim.x) sh[i] = 0u;
  __syncthreads();
  const bool gas = g.flags & MC_FLAG_GAS;
  const bool dust = g.flags & MC_FLAG_DUST;
  unsigned long long nline = 0, nesc = 0, ntrap = 0;
  const unsigned int stride = gridDim.x * blockDim.x;
  for (unsigned int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_abs; i += stride) {
    const uint32_t id = w.a_id[i];
    const int s = source_of(S, id);
    const DevSource &src = S.s[s];
    RStream<Replay> st;
    st.init((unsigned long long)(id - src.base), rp, id);
    st.resume(w.a_words[i], src.k0, src.k1);
    int x, y, z;
    unpack_cell(w.a_cell[i], x, y, z);
    const int a = __ldg(g.active + (x - 1) + (long long)g.nx * ((y - 1) + (long long)g.ny * (z - 1)));
    const bool trapped_at_end = (int)w.a_run[i] + 1 >= g.recursion_limit;
    w.s_nu[i] = 0xFFFFu;
    if (a <= 0) { raise_error(cnt, MC_ERR_BOUNDS, id); continue; }
    int nuP;
    bool ok = true;
    if (gas) {
      const Real random = (Real)1 - st.template next<Real>(src.k0, src.k1);
      if (random <= (Real)__ldg(g.total_lines + a)) {  // a line packet: it escapes as a line
        ++nline;
        if (trapped_at_end) ++ntrap;
        continue;
      }
      nuP = sample_bin<Real, Replay>(st, src.k0, src.k1, g.rec_cdf + (long long)a * g.nb, g.nb, ok);
    } else {
      nuP = sample_bin<Real, Replay>(st, src.k0, src.k1, g.dust_cdf + (long long)a * g.nb, g.nb, ok);
    }
    if (!ok || nuP >= g.nb || nuP < 1 || st.exhausted) {
      raise_error(cnt, st.exhausted ? MC_ERR_REPLAY : MC_ERR_BOUNDS, id);
      continue;
    }
    if (!dust && (Real)__ldg(g.nu + nuP - 1) < (Real)g.ion_edge1) {
      // escapes before any march; the direction initPhotonPacket draws is
      // needed only for the viewing-angle plane
      int view = 0;
      if (g.n_angle > 0) {
        R3<Real> d;
        ok = sample_direction<Real, Replay>(st, src.k0, src.k1, d);
        if (ok) view = escape_view<Real>(g, d.x, d.y, d.z, ok);
        if (!ok || st.exhausted) { raise_error(cnt, st.exhausted ? MC_ERR_REPLAY : MC_ERR_NAN, id); continue; }
      }
      add_escape(g, a, nuP, view, (double)(Real)src.delta_e);
      ++nesc;
      if (trapped_at_end) ++ntrap;
      continue;
    }
    w.s_nu[i] = (uint16_t)nuP;
    w.s_words[i] = st.consumed();
    atomicAdd(&sh[nuP], 1u);
  }
  nline = warp_sum(nline);
  nesc = warp_sum(nesc);
  ntrap = warp_sum(ntrap);
  if ((threadIdx.x & 31) == 0) {
    if (nline) atomicAdd(&cnt->lines, nline);
    if (nesc) atomicAdd(&cnt->escaped, nesc);
    if (ntrap) atomicAdd(&cnt->trapped, ntrap);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < g.nb; i += blockDim.x)
    if (sh[i]) atomicAdd(&w.bin_count[i], sh[i]);
}

// Resonance-line packets (energyPacketDriver :180-266): after round 0 each
// star's block of diffuse packets joins the absorbed list that round 1
// re-emits, packet p of a block at the node (xAxis(ix), yAxis(iy),
// zAxis(iz)) of its cell, with a fresh draw stream and no re-emission yet.
// cells [ncell] packed, prefix [ncell + 1] the packets before each cell.
template <typename Real>
__global__ void __launch_bounds__(256) wave_res_inject_kernel(const __grid_constant__ DevGrid g,
                                                             const __grid_constant__ DevSources S,
                                                             const __grid_constant__ WaveGrid w,
                                                             const uint32_t *cells, const long long *prefix,
                                                             int ncell) {
  const long long per = prefix[ncell], total = per * S.nres;
  const unsigned int lane = threadIdx.x & 31;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long k0 = (long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); k0 < total; k0 += stride) {
    const long long k = k0 + lane;
    const bool mine = k < total;
    const unsigned int m = __ballot_sync(0xffffffffu, mine);
    unsigned int base = 0;
    if (lane == 0) base = atomicAdd(w.a_count, (unsigned int)__popc(m));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (!mine) continue;
    const int b = (int)(k / per);
    const long long p = k - (long long)b * per;
    int lo = 0, hi = ncell - 1;  // the cell j with prefix[j] <= p < prefix[j + 1]
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (prefix[mid] <= p) lo = mid;
      else hi = mid - 1;
    }
    const unsigned int slot = base + lane;
    int x, y, z;
    unpack_cell(cells[lo], x, y, z);
    w.a_id[slot] = (uint32_t)(S.s[S.nsrc + b].base + p);
    w.a_cell[slot] = cells[lo];
    w.a_words[slot] = 0u;
    w.a_run[slot] = 0;
    Real *ar = (Real *)w.a_r + 3 * (size_t)slot;
    ar[0] = (Real)g.xa[x - 1];
    ar[1] = (Real)g.ya[y - 1];
    ar[2] = (Real)g.za[z - 1];
  }
}

// ------------------------------------------------------------------ emit
// One thread per queue slot: direction and passProb, written in queue order.
template <typename Real, bool Replay>
__global__ void __launch_bounds__(256) wave_emit_kernel(const __grid_constant__ DevGrid g,
                                                       const __grid_constant__ DevSources S,
                                                       const __grid_constant__ DevReplay rp,
                                                       const __grid_constant__ WaveGrid w, int round,
                                                       DevCounters *cnt) {
  const unsigned int qlen = w.bin_count[0];
  const unsigned int stride = gridDim.x * blockDim.x;
  const bool fold = round == 0 && (g.flags & MC_FLAG_SYMMETRIC_XYZ) && !(g.flags & MC_FLAG_MULTISTARS);
  for (unsigned int q = blockIdx.x * blockDim.x + threadIdx.x; q < qlen; q += stride) {
    const uint32_t k = w.queue[q];  // packet id (round 0) or absorbed-list index
    uint32_t id, cell, run;
    R3<Real> r;
    if (round == 0) {
      id = k;
      const DevSource &src = S.s[source_of(S, id)];
      cell = pack_cell(src.cell[0], src.cell[1], src.cell[2]);
      r = R3<Real>{(Real)src.pos[0], (Real)src.pos[1], (Real)src.pos[2]};
      run = 1;
    } else {
      id = w.a_id[k];
      cell = w.a_cell[k];
      const Real *ar = (const Real *)w.a_r + 3 * (size_t)k;
      r = R3<Real>{ar[0], ar[1], ar[2]};
      run = w.a_run[k] + 1;
    }
    const int s = source_of(S, id);
    const DevSource &src = S.s[s];
    RStream<Replay> st;
    st.init((unsigned long long)(id - src.base), rp, id);
    st.resume(w.s_words[k], src.k0, src.k1);
    R3<Real> d;
    bool ok = sample_direction<Real, Replay>(st, src.k0, src.k1, d);
    if (fold) {
      if (d.x < (Real)0) d.x = -d.x;
      if (d.y < (Real)0) d.y = -d.y;
      if (d.z < (Real)0) d.z = -d.z;
    }
    const Real pass = -log((Real)1 - st.template next<Real>(src.k0, src.k1));
    if (!ok || st.exhausted) {
      raise_error(cnt, st.exhausted ? MC_ERR_REPLAY : MC_ERR_NAN, id);
      w.q_meta[q] = 0u;  // nuP = 0: the march skips it
      continue;
    }
    int x, y, z;
    unpack_cell(cell, x, y, z);
    w.q_id[q] = id;
    w.q_cell[q] = cell;
    w.q_words[q] = st.consumed();
    w.q_meta[q] = pack_meta(w.s_nu[k], (int)run, round == 0);
    w.q_origin[q] = __ldg(g.active + (x - 1) + (long long)g.nx * ((y - 1) + (long long)g.ny * (z - 1)));
    Real *qr = (Real *)w.q_r + 3 * (size_t)q;
    qr[0] = r.x; qr[1] = r.y; qr[2] = r.z;
    Real *qv = (Real *)w.q_v + 3 * (size_t)q;
    qv[0] = d.x; qv[1] = d.y; qv[2] = d.z;
    ((Real *)w.q_pass)[q] = pass;
  }
}

// ---------------------------------------------------------------- march
// Per-axis tables in shared memory, entry (axis a, cell i) = 5 Reals:
// node x_i, wall above (mid(i,i+1), or the last node), wall below
// (mid(i-1,i), or the first node), dV width / 1e15, its inverse.
template <typename Real> struct Tables {
  const Real *base;
  int o1, o2;  // entry offsets of the y and z axes
  __device__ __forceinline__ const Real *e(int a, int i) const {
    return base + 5 * ((a == 0 ? 0 : (a == 1 ? o1 : o2)) + i);
  }
  __device__ __forceinline__ Real node(int a, int i) const { return e(a, i)[0]; }
  __device__ __forceinline__ Real wid(int a, int i) const { return e(a, i)[3]; }
  __device__ __forceinline__ Real iwid(int a, int i) const { return e(a, i)[4]; }
};

constexpr int kHotHalf = 3;                    // cube half width (cells)
constexpr int kHot = 2 * kHotHalf + 1;         // cube edge
constexpr int kHot3 = kHot * kHot * kHot;      // cells per cube
constexpr int kHotSrc = 2;                     // stars with a cube

// event counts of the fast march: warp-private slots in shared memory (the
// nine 64-bit per-lane counters of LocalCounts would take 18 registers of the
// 64 the fast march runs with)
enum { kCntAbs = 0, kCntSca, kCntEsc, kCntTrap, kCntSilent, kCntSafe, kCntSlots };

template <typename Real, bool Fast, bool Dust, bool Replay> struct Marcher {
  const DevGrid &g;
  const DevSources &S;
  const DevReplay &rp;
  const WaveGrid &w;
  const Tables<Real> &T;
  DevCounters *cnt;
  LocalCounts &lc;
  unsigned int *wc;         // Fast: this warp's kCntSlots event counters in shared memory
  unsigned long long *wcx;  // Fast: this warp's crossing counter in shared memory

  // lane state
  R3<Real> r, v, iv;  // position, direction, 1/direction (fast path)
  R3<Real> dir0;      // enPacket%direction (turned by HG scattering)
  int xP, yP, zP, nuP, origin, runI, segI;
  uint32_t id;
  Real absTau, passProb;
  bool stellar, valid;
  bool pend;  // absorbed: the entry for the next round is written after the step
  int pev;    // Fast: the parked event (EV_* | axis << 2) that stopped the lane's crossings, 0 = none
  RStream<Replay> st;

  __device__ Marcher(const DevGrid &g_, const DevSources &S_, const DevReplay &rp_, const WaveGrid &w_,
                     const Tables<Real> &T_, DevCounters *c_, LocalCounts &lc_)
      : g(g_), S(S_), rp(rp_), w(w_), T(T_), cnt(c_), lc(lc_), wc(nullptr), wcx(nullptr), valid(false), pend(false),
        pev(0), segI(0) {}

  // one event of kind K (the fast march counts crossings per packet, from segI)
  template <int K> __device__ __forceinline__ void bump() {
    if (Fast) {
      atomicAdd(wc + K, 1u);
    } else {
      if (K == kCntAbs) ++lc.absorptions;
      else if (K == kCntSca) ++lc.scatterings;
      else if (K == kCntEsc) ++lc.escaped;
      else if (K == kCntTrap) ++lc.trapped;
      else if (K == kCntSilent) ++lc.silent;
      else if (K == kCntSafe) ++lc.safe_hits;
    }
  }
  // the crossings of the lane's last packet (Fast: every crossing is one segI)
  __device__ __forceinline__ void count_crossings() {
    if (Fast && segI > 0) { atomicAdd(wcx, (unsigned long long)segI); segI = 0; }
  }

  __device__ __forceinline__ const DevSource &source() const { return S.s[source_of(S, id)]; }
  __device__ __forceinline__ Real rnd() {
    const DevSource &s = source();
    return st.template next<Real>(s.k0, s.k1);
  }
  __device__ __forceinline__ void fail(int code) {
    raise_error(cnt, code, id);
    valid = false;
  }
  __device__ __forceinline__ void end_history() {
    if (runI >= g.recursion_limit) bump<kCntTrap>();
    valid = false;
  }
  __device__ __forceinline__ void escape() {
    int view = 0;
    if (g.n_angle > 0) {
      bool ok;
      view = escape_view<Real>(g, v.x, v.y, v.z, ok);
      if (!ok) { fail(MC_ERR_NAN); return; }
    }
    const int s0 = source_of(S, id);
    if (Fast && stellar && nuP == hot_nu && s0 < kHotSrc && origin == esc_org[s0]) {
      // escapedPackets(star cell, hot_nu, 0): counted in the warp, added as
      // count x deltaE when the warp's bin changes (every stellar packet of a
      // bin escapes into the same entry, so the atomics would serialise)
      atomicAdd(esc_n + s0, 1u);
      if (view > 0 && g.esc)
        atomicAdd(g.esc + origin + (long long)(g.nc + 1) * nuP + (long long)(g.nc + 1) * (g.nb + 1) * view,
                  (double)(Real)S.s[s0].delta_e);
    } else {
      add_escape(g, origin, nuP, view, (double)(Real)source().delta_e);
    }
    bump<kCntEsc>();
    end_history();
  }
  __device__ __forceinline__ void set_v(R3<Real> d) {
    v = d;
    if (Fast) iv = R3<Real>{(Real)__frcp_rn((float)d.x), (Real)__frcp_rn((float)d.y), (Real)__frcp_rn((float)d.z)};
  }
  __device__ __forceinline__ void flip(int a) {
    if (a == 0) { v.x = -v.x; if (Fast) iv.x = -iv.x; }
    else if (a == 1) { v.y = -v.y; if (Fast) iv.y = -iv.y; }
    else { v.z = -v.z; if (Fast) iv.z = -iv.z; }
  }
  // lower-plane reflection of a symmetric octant (photon_mod.f90:1248-1261)
  __device__ __forceinline__ void reflect_low(Real X1, Real Y1, Real Z1) {
    if (r.x <= X1) { if (v.x < (Real)0) flip(0); r.x = X1; }
    if (r.y <= Y1) { if (v.y < (Real)0) flip(1); r.y = Y1; }
    if (r.z <= Z1) { if (v.z < (Real)0) flip(2); r.z = Z1; }
  }
  // wall distance along one axis (photon_mod.f90:1263-1379); false on the
  // silent wall-sitting exit at the last node
  __device__ __forceinline__ bool axis_dist(int a, Real &ra, int &pa, Real va, Real iva, int na, Real &ds) {
    const Real tiny = (Real)1.e-10f;
    const bool up = va > tiny, down = va < -tiny;
    const Real *e = T.e(a, pa - 1);
    const Real wall = up ? e[1] : e[2];
    ds = Fast ? (wall - ra) * iva : (wall - ra) / va;
    if (!(up || down)) ds = (Real)1.e35f;
    if (fabs(ds) < tiny) {
      if (up) {
        if (pa < na) { ra = wall; pa = pa + 1; }
        else return false;
      } else if (down) {
        ra = wall;
        if (pa > 1) pa = pa - 1;
      }
    }
    return true;
  }

  // a queue entry written by the emission pass
  __device__ __forceinline__ void start(unsigned int q) {
    count_crossings();
    const uint32_t meta = __ldg(w.q_meta + q);
    nuP = (int)(meta & 0xFFFFu);
    if (nuP == 0) return;  // emission failed (error already raised)
    runI = (int)((meta >> 16) & 0x7FFFu);
    stellar = meta >> 31;
    id = __ldg(w.q_id + q);
    unpack_cell(__ldg(w.q_cell + q), xP, yP, zP);
    origin = __ldg(w.q_origin + q);
    const Real *qr = (const Real *)w.q_r + 3 * (size_t)q;
    r = R3<Real>{__ldg(qr), __ldg(qr + 1), __ldg(qr + 2)};
    const Real *qv = (const Real *)w.q_v + 3 * (size_t)q;
    const R3<Real> d{__ldg(qv), __ldg(qv + 1), __ldg(qv + 2)};
    dir0 = d;
    set_v(d);
    passProb = __ldg((const Real *)w.q_pass + q);
    absTau = (Real)0;
    segI = 0;
    const DevSource &s = source();
    st.init((unsigned long long)(id - s.base), rp, id);
    st.resume(__ldg(w.q_words + q), s.k0, s.k1);
    valid = true;
    if (Fast) { set_rows(); dda_init(); }
  }

  // absorbed: hand the packet to the next round (rerun = 1, :2861-2870)
  __device__ __forceinline__ void absorbed() {
    bump<kCntAbs>();
    if (segI >= g.safe_limit) { bump<kCntSafe>(); end_history(); return; }
    if (runI >= g.recursion_limit) { bump<kCntTrap>(); valid = false; return; }
    pend = true;
    valid = false;
  }
  // writes the next round's entry of an absorbed packet into `slot`
  __device__ __forceinline__ void write_absorbed(unsigned int slot) {
    w.a_id[slot] = id;
    w.a_cell[slot] = pack_cell(xP, yP, zP);
    w.a_words[slot] = st.consumed();
    w.a_run[slot] = (uint16_t)runI;
    Real *ar = (Real *)w.a_r + 3 * (size_t)slot;
    ar[0] = r.x; ar[1] = r.y; ar[2] = r.z;
    pend = false;
  }

  __device__ __forceinline__ void deposit(int ci, Real val) {
    double *J = (stellar || !(g.flags & MC_FLAG_DEBUG)) ? w.jste : w.jdif;
    atomicAdd(J + (long long)(nuP - 1) * w.S + ci, (double)val);
  }

  // hg (photon_mod.f90:2875-3101) on the emission direction
  __device__ int hg(R3<Real> &dir) {
    const Real twoPi = (Real)2 * (Real)3.141592654;
    const Real vin0 = dir.x, vin1 = dir.y, vin2 = dir.z;
    Real v0, v1, v2;
    const Real hgg = (Real)__ldg(g.gsca + nuP - 1);
    const Real s = (Real)2 * rnd() - (Real)1;
    Real cost, sint;
    if (hgg >= (Real)0.0001f) {
      const Real q = ((Real)1 - hgg * hgg) / ((Real)1 + hgg * s);
      cost = (Real)0.5 / hgg * ((Real)1 + hgg * hgg - q * q);
    } else {
      cost = s;
    }
    if (cost >= (Real)1) { cost = (Real)1; sint = (Real)0; }
    else if (cost < (Real)-1) { cost = (Real)-1; sint = (Real)0; }
    else sint = sqrt((Real)1 - cost * cost);
    const Real phi = twoPi * rnd();
    const Real cosp = cos(phi), sinp = sin(phi);
    const Real denom = sqrt((Real)1 - vin2 * vin2);
    if (denom > (Real)0.001f) {
      v0 = sint / denom * (vin0 * vin2 * cosp - vin1 * sinp) + vin0 * cost;
      v1 = sint / denom * (vin1 * vin2 * cosp + vin0 * sinp) + vin1 * cost;
      v2 = -sint * cosp * denom + vin2 * cost;
    } else {
      v0 = sint * cosp;
      v1 = sint * sinp;
      v2 = (vin2 >= (Real)0) ? cost : -cost;
    }
    const bool n0 = !isnan(v0), n1 = !isnan(v1), n2 = !isnan(v2);
    if (fabs(v0) <= (Real)1 && fabs(v1) <= (Real)1 && fabs(v2) <= (Real)1 && n0 && n1 && n2) {
      dir = R3<Real>{v0, v1, v2};
      return 0;
    }
    if (fabs(v0) >= (Real)1 || fabs(v1) >= (Real)1 || (fabs(v2) >= (Real)1 && n0 && n1 && n2)) return 0;
    return 1;
  }

  // dust scattering (photon_mod.f90:1718-1798): the packet turns and keeps
  // marching with a fresh passProb
  __device__ void scatter() {
    bump<kCntSca>();
    origin = w.identity ? lin_of(g, xP, yP, zP) + 1 : __ldg(w.lin2cell + lin_of(g, xP, yP, zP));
    stellar = false;
    if (g.flags & MC_FLAG_ISOTROPIC) {
      R3<Real> d;
      const DevSource &s = source();
      if (!sample_direction<Real, Replay>(st, s.k0, s.k1, d)) { fail(MC_ERR_NAN); return; }
      dir0 = d;
    } else {
      for (int ihg = 1; ihg <= 10; ++ihg)
        if (hg(dir0) == 0) break;
    }
    set_v(dir0);
    if (isnan(v.x)) { fail(MC_ERR_NAN); return; }
    absTau = (Real)0;
    passProb = -log((Real)1 - rnd());
    if (segI >= g.safe_limit) { bump<kCntSafe>(); end_history(); }
  }

  // ---- fast path: 3D-DDA march (Amanatides & Woo 1987) ---------------
  // The ray is r0 + t v.  tN0..2 are the ray parameters of the next wall on
  // each axis; a crossing advances the nearest axis, so a cell's chord dS is
  // the difference of two wall parameters (the dS of photon_mod.f90:1395-1425)
  // and the position is rebuilt only at interactions and reflections.  The
  // axis step is branch-free (selects), so lanes stepping different axes stay
  // converged; the opacity of the next cell is loaded as soon as its index is
  // known.
  R3<Real> r0;
  Real tc, tN0, tN1, tN2;
  Real kap;            // opacity of the current cell
  Real idv0, idv1, idv2;  // 1 / (cell widths / 1e15) of the current cell
  Real de;             // deltaE of the packet's star
  int lin;
  const float *orow;   // opacity(:, nuP) in march order (+ off)
  double *jrow;        // Jste or Jdif(:, nuP) in march order (+ off)
  // warp-private FP32 accumulator of Jste(:, hot_nu) over the cube of
  // kHot^3 cells around each of the first kHotSrc stars, flushed to the FP64
  // sums (every packet of a frequency bin crosses the cells next to its star,
  // so their atomics would serialise in L2)
  float *hot;          // this warp's slice of shared memory
  unsigned int *esc_n; // this warp's escape counts of (star kHotSrc, hot_nu)
  const int *esc_org;  // origin of each of the first kHotSrc stars
  int hot_nu;          // bin held by the accumulator (warp-uniform), 0 = none
  bool hot_ok;         // this packet's deposits may go to the accumulator

  __device__ __forceinline__ Real wall_param(int a, int p, Real r0a, Real va, Real iva) const {
    const Real tiny = (Real)1.e-10f;
    if (va > tiny) return (T.e(a, p - 1)[1] - r0a) * iva;
    if (va < -tiny) return (T.e(a, p - 1)[2] - r0a) * iva;
    return (Real)1.e35f;
  }
  __device__ __forceinline__ void load_cell() {
    lin = lin_of(g, xP, yP, zP);
    kap = (Real)__ldg(orow + lin);
    idv0 = T.iwid(0, xP - 1);
    idv1 = T.iwid(1, yP - 1);
    idv2 = T.iwid(2, zP - 1);
  }
  __device__ __forceinline__ void set_rows() {
    orow = w.opac + (long long)(nuP - 1) * w.S + w.off;
    double *J = (stellar || !(g.flags & MC_FLAG_DEBUG)) ? w.jste : w.jdif;
    jrow = J + (long long)(nuP - 1) * w.S + w.off;
    de = (Real)source().delta_e;
    refresh_hot();
  }
  __device__ __forceinline__ void refresh_hot() {
    hot_ok = Fast && valid && nuP == hot_nu && (stellar || !(g.flags & MC_FLAG_DEBUG)) &&
             source_of(S, id) < (S.nsrc < kHotSrc ? S.nsrc : kHotSrc);  // a star with a cube (not a resonance block)
  }
  // (re)start the ray at r0 = r with direction v
  __device__ void dda_init() {
    const Real tiny = (Real)1.e-10f;
    r0 = r;
    tc = (Real)0;
    tN0 = wall_param(0, xP, r0.x, v.x, iv.x);
    tN1 = wall_param(1, yP, r0.y, v.y, iv.y);
    tN2 = wall_param(2, zP, r0.z, v.z, iv.z);
    // a packet sitting on the wall it heads for steps through it first
    // (photon_mod.f90:1268-1290); on the outer wall it leaves silently
    if (fabs(tN0) < tiny || fabs(tN1) < tiny || fabs(tN2) < tiny) {
      if (fabs(tN0) < tiny) { if (v.x > (Real)0) { if (xP < g.nx) ++xP; else { bump<kCntSilent>(); end_history(); return; } } else if (xP > 1) --xP; tN0 = wall_param(0, xP, r0.x, v.x, iv.x); }
      if (fabs(tN1) < tiny) { if (v.y > (Real)0) { if (yP < g.ny) ++yP; else { bump<kCntSilent>(); end_history(); return; } } else if (yP > 1) --yP; tN1 = wall_param(1, yP, r0.y, v.y, iv.y); }
      if (fabs(tN2) < tiny) { if (v.z > (Real)0) { if (zP < g.nz) ++zP; else { bump<kCntSilent>(); end_history(); return; } } else if (zP > 1) --zP; tN2 = wall_param(2, zP, r0.z, v.z, iv.z); }
    }
    load_cell();
  }
  // reflection at a lower plane of a symmetric octant (photon_mod.f90:2680-2697)
  __device__ void dda_reflect(int a) {
    r = R3<Real>{r0.x + tc * v.x, r0.y + tc * v.y, r0.z + tc * v.z};
    if (a == 0) { r.x = T.node(0, 0); xP = 1; }
    else if (a == 1) { r.y = T.node(1, 0); yP = 1; }
    else { r.z = T.node(2, 0); zP = 1; }
    flip(a);
    dda_init();
  }

  __device__ __forceinline__ void add_j(Real val) {
    if (hot_ok) {
      const int s0 = source_of(S, id);
      const DevSource &sp = S.s[s0];
      const unsigned dx = (unsigned)(xP - sp.cell[0] + kHotHalf), dy = (unsigned)(yP - sp.cell[1] + kHotHalf),
                     dz = (unsigned)(zP - sp.cell[2] + kHotHalf);
      if (dx < (unsigned)kHot && dy < (unsigned)kHot && dz < (unsigned)kHot) {
        atomicAdd(hot + s0 * kHot3 + (dx * kHot + dy) * kHot + dz, (float)val);
        return;
      }
      hot_ok = false;  // a packet rarely comes back to its star's cube
    }
    atomicAdd(jrow + lin, (double)val);
  }

  enum { EV_NONE = 0, EV_INTERACT = 1, EV_EDGE = 2, EV_SAFE = 3 };

  // One crossing without events: returns EV_NONE, or the event that stops
  // the packet's run of crossings (the state is left at the event).
  __device__ __forceinline__ int cross(int &ea) {
    // nearest wall; ties go x, y, z as in photon_mod.f90:1961-1972
    const bool c1 = tN1 < tN0;
    Real tE = c1 ? tN1 : tN0;
    int a = c1 ? 1 : 0;
    const bool c2 = tN2 < tE;
    tE = c2 ? tN2 : tE;
    a = c2 ? 2 : a;
    const Real dS = tE - tc;
    const Real tau = dS * kap;
    ++segI;
    const bool active = w.identity ? true : (__ldg(w.lin2cell + lin) > 0);
    if ((absTau + tau > passProb) && active) { ea = a; return EV_INTERACT; }
    add_j(dS * de * (idv0 * idv1 * idv2));
    absTau = absTau + tau;
    tc = tE;
    const Real va = a == 0 ? v.x : (a == 1 ? v.y : v.z);
    const Real iva = a == 0 ? iv.x : (a == 1 ? iv.y : iv.z);
    const Real r0a = a == 0 ? r0.x : (a == 1 ? r0.y : r0.z);
    const int na = a == 0 ? g.nx : (a == 1 ? g.ny : g.nz);
    const int up = va > (Real)0;
    const int p = (a == 0 ? xP : (a == 1 ? yP : zP)) + (up ? 1 : -1);
    if (p > na || p < 1) { ea = a; return EV_EDGE; }
    xP = a == 0 ? p : xP;
    yP = a == 1 ? p : yP;
    zP = a == 2 ? p : zP;
    const Real *e = T.e(a, p - 1);
    const Real tNa = (e[up ? 1 : 2] - r0a) * iva;
    const Real idva = e[4];
    tN0 = a == 0 ? tNa : tN0;
    tN1 = a == 1 ? tNa : tN1;
    tN2 = a == 2 ? tNa : tN2;
    idv0 = a == 0 ? idva : idv0;
    idv1 = a == 1 ? idva : idv1;
    idv2 = a == 2 ? idva : idv2;
    const int stride = a == 0 ? g.ny * g.nz : (a == 1 ? g.nz : 1);
    lin += up ? stride : -stride;
    kap = (Real)__ldg(orow + lin);
    return EV_NONE;
  }

  // the interaction inside the current cell (photon_mod.f90:1517-1815)
  __device__ void interact() {
    const Real dl = (passProb - absTau) / kap;
    const Real ti = tc + dl;
    r = R3<Real>{r0.x + ti * v.x, r0.y + ti * v.y, r0.z + ti * v.z};
    add_j(dl * de * (idv0 * idv1 * idv2));
    const Real rout = (Real)g.rout;
    if (rout > (Real)0) {
      const Real e10 = (Real)1.e10f;
      const Real rx = r.x / e10, ry = r.y / e10, rz = r.z / e10;
      if (sqrt(rx * rx + ry * ry + rz * rz) * e10 >= rout) { escape(); return; }
    }
    if (Dust) {
      const Real probSca = (Real)__ldg(w.sca + (long long)(nuP - 1) * w.S + w.off + lin) / kap;
      const Real rr = (Real)1 - rnd();
      if (rr > probSca) { absorbed(); return; }
      scatter();
      if (valid) { set_rows(); dda_init(); }
      return;
    }
    absorbed();
  }

  // the packet left the index range on axis a: escape, or reflect at a
  // lower plane of a symmetric octant
  __device__ void edge(int a) {
    const Real va = a == 0 ? v.x : (a == 1 ? v.y : v.z);
    if (va > (Real)0 || !(g.flags & MC_FLAG_SYMMETRIC_XYZ)) { escape(); return; }
    dda_reflect(a);
    if (valid && segI >= g.safe_limit) { bump<kCntSafe>(); end_history(); }
  }

  // adds the accumulator into Jste(:, hot_nu) and clears it (whole warp)
  __device__ void hot_flush(unsigned int lane) {
    __syncwarp();
    if (hot_nu > 0) {
      const int ncube = S.nsrc < kHotSrc ? S.nsrc : kHotSrc;
      if ((int)lane < ncube) {
        const unsigned int c = esc_n[lane];
        if (c) {
          esc_n[lane] = 0u;
          if (g.esc)
            atomicAdd(g.esc + esc_org[lane] + (long long)(g.nc + 1) * hot_nu, (double)c * (double)(Real)S.s[lane].delta_e);
        }
      }
      double *row = w.jste + (long long)(hot_nu - 1) * w.S + w.off;
      for (int i = (int)lane; i < ncube * kHot3; i += 32) {
        const float val = hot[i];
        if (val == 0.f) continue;
        hot[i] = 0.f;
        const int s0 = i / kHot3, c = i % kHot3;
        const int x = S.s[s0].cell[0] - kHotHalf + c / (kHot * kHot);
        const int y = S.s[s0].cell[1] - kHotHalf + (c / kHot) % kHot;
        const int z = S.s[s0].cell[2] - kHotHalf + c % kHot;
        atomicAdd(row + lin_of(g, x, y, z), (double)val);
      }
    }
    __syncwarp();
  }

  // up to k crossings; the event that stopped them is parked and handled
  // together with the warp's other parked events (the event code then runs
  // with many lanes instead of one or two)
  __device__ void advance(int k) {
    int ev = EV_NONE, ea = 0;
    // at most the crossings left before safeLimit: the run then ends in
    // EV_SAFE after the crossing that reaches it, as a per-crossing test would
    const int left = g.safe_limit - segI;
    const int kk = left < k ? left : k;
    for (int i = 0; i < kk; ++i) {
      ev = cross(ea);
      if (ev != EV_NONE) break;
    }
    if (ev == EV_NONE && segI >= g.safe_limit) ev = EV_SAFE;
    pev = ev | (ea << 2);
  }
  __device__ void handle_parked() {
    const int ev = pev & 3, ea = pev >> 2;
    pev = 0;
    if (ev == EV_INTERACT) interact();
    else if (ev == EV_EDGE) edge(ea);
    else if (ev == EV_SAFE) { bump<kCntSafe>(); end_history(); }
  }

  // One pathSegment loop body.  Leaves `valid` false when the packet ended
  // or was handed to the next round.
  __device__ void step() {
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const bool sym = g.flags & MC_FLAG_SYMMETRIC_XYZ;
    const Real tiny = (Real)1.e-10f;
    ++segI;
    if (xP > nx || xP < 1 || yP > ny || yP < 1 || zP > nz || zP < 1) { fail(MC_ERR_BOUNDS); return; }
    const Real X1 = T.node(0, 0), Y1 = T.node(1, 0), Z1 = T.node(2, 0);
    const Real Xn = T.node(0, nx - 1), Yn = T.node(1, ny - 1), Zn = T.node(2, nz - 1);
    if (sym) reflect_low(X1, Y1, Z1);
    Real dSx, dSy, dSz;
    if (!axis_dist(0, r.x, xP, v.x, iv.x, nx, dSx) || !axis_dist(1, r.y, yP, v.y, iv.y, ny, dSy) ||
        !axis_dist(2, r.z, zP, v.z, iv.z, nz, dSz)) {
      bump<kCntSilent>();
      end_history();
      return;
    }
    if (isnan(dSx) || isnan(dSy) || isnan(dSz)) { fail(MC_ERR_NAN); return; }
    if (xP > nx || xP < 1 || yP > ny || yP < 1 || zP > nz || zP < 1) { fail(MC_ERR_BOUNDS); return; }
    if (fabs(dSx) < tiny) dSx = Xn;
    if (fabs(dSy) < tiny) dSy = Yn;
    if (fabs(dSz) < tiny) dSz = Zn;
    dSx = fabs(dSx);
    dSy = fabs(dSy);
    dSz = fabs(dSz);
    Real dS;
    if (dSx <= (Real)0) dS = fmin(dSy, dSz);
    else if (dSy <= (Real)0) dS = fmin(dSx, dSz);
    else if (dSz <= (Real)0) dS = fmin(dSx, dSy);
    else { dS = fmin(dSx, dSy); dS = fmin(dS, dSz); }
    if (dS <= (Real)0) { fail(MC_ERR_BOUNDS); return; }

    const int lin = lin_of(g, xP, yP, zP);
    const int ci = lin + w.off;
    const Real kap = (Real)__ldg(w.opac + (long long)(nuP - 1) * w.S + ci);
    const bool active = w.identity ? true : (__ldg(w.lin2cell + lin) > 0);
    const Real tauCell = dS * kap;
    Real dV, idV;
    if (Fast) { dV = (Real)0; idV = T.iwid(0, xP - 1) * T.iwid(1, yP - 1) * T.iwid(2, zP - 1); }
    else { dV = T.wid(0, xP - 1) * T.wid(1, yP - 1) * T.wid(2, zP - 1); idV = (Real)0; }
    const Real deltaE = (Real)source().delta_e;
    ++lc.crossings;

    if ((absTau + tauCell > passProb) && active) {
      const Real dlLoc = (passProb - absTau) / kap;
      r.x = r.x + dlLoc * v.x;
      r.y = r.y + dlLoc * v.y;
      r.z = r.z + dlLoc * v.z;
      if (isnan(r.x) || isnan(r.y) || isnan(r.z)) { fail(MC_ERR_NAN); return; }
      if (sym) reflect_low(X1, Y1, Z1);
      deposit(ci, Fast ? dlLoc * deltaE * idV : dlLoc * deltaE / dV);
      const Real e10 = (Real)1.e10f;
      const Real rx = r.x / e10, ry = r.y / e10, rz = r.z / e10;
      const Real rout = (Real)g.rout;
      if (sqrt(rx * rx + ry * ry + rz * rz) * e10 >= rout && rout > (Real)0) { escape(); return; }
      if (Dust) {
        const Real probSca = (Real)__ldg(w.sca + (long long)(nuP - 1) * w.S + ci) / kap;
        const Real rr = (Real)1 - rnd();
        if (rr > probSca) { absorbed(); return; }
        if (!(rr <= probSca)) { fail(MC_ERR_NAN); return; }
        scatter();
        return;
      }
      absorbed();
      return;
    }

    // full crossing
    deposit(ci, Fast ? dS * deltaE * idV : dS * deltaE / dV);
    absTau = absTau + tauCell;
    r.x = r.x + dS * v.x;
    r.y = r.y + dS * v.y;
    r.z = r.z + dS * v.z;
    if (dS == dSx && v.x > (Real)0) xP = xP + 1;
    else if (dS == dSx && v.x < (Real)0) xP = xP - 1;
    else if (dS == dSy && v.y > (Real)0) yP = yP + 1;
    else if (dS == dSy && v.y < (Real)0) yP = yP - 1;
    else if (dS == dSz && v.z > (Real)0) zP = zP + 1;
    else if (dS == dSz && v.z < (Real)0) zP = zP - 1;
    const Real gcx = (Real)g.gc[0], gcy = (Real)g.gc[1], gcz = (Real)g.gc[2];
    if (!sym) {
      if (r.y <= Y1 - gcy || yP < 1 || r.y > Yn + gcy || yP > ny || r.x <= X1 - gcx || xP < 1 ||
          r.x >= Xn + gcx || xP > nx || r.z <= Z1 - gcz || zP < 1 || r.z >= Zn + gcz || zP > nz) {
        escape();
        return;
      }
    }
    if ((!sym && (r.x <= X1 - gcx || r.y <= Y1 - gcy || r.z <= Z1 - gcz)) || r.x >= Xn + gcx ||
        r.y >= Yn + gcy || r.z >= Zn + gcz || xP > nx || yP > ny || zP > nz) {
      escape();
      return;
    }
    if (sym) {
      if (r.x <= X1 || xP < 1) { if (v.x < (Real)0) flip(0); xP = 1; r.x = X1; }
      if (r.y <= Y1 || yP < 1) { if (v.y < (Real)0) flip(1); yP = 1; r.y = Y1; }
      if (r.z <= Z1 || zP < 1) { if (v.z < (Real)0) flip(2); zP = 1; r.z = Z1; }
    }
    if (segI >= g.safe_limit) { bump<kCntSafe>(); end_history(); }
  }
};

template <typename Real>
__device__ void build_tables(const DevGrid &g, char *smem, Tables<Real> &T) {
  const int n[3] = {g.nx, g.ny, g.nz};
  const float *ax[3] = {g.xa, g.ya, g.za};
  const bool sym = g.flags & MC_FLAG_SYMMETRIC_XYZ;
  Real *base = (Real *)smem;
  T.base = base;
  T.o1 = g.nx;
  T.o2 = g.nx + g.ny;
  const int off[3] = {0, g.nx, g.nx + g.ny};
  for (int a = 0; a < 3; ++a) {
    const int na = n[a];
    for (int i = threadIdx.x; i < na; i += blockDim.x) {
      const int pp = i + 1;
      auto A = [&](int k) { return (Real)ax[a][k - 1]; };
      Real *e = base + 5 * (off[a] + i);
      e[0] = A(pp);
      e[1] = pp < na ? (A(pp + 1) + A(pp)) / (Real)2 : A(na);
      e[2] = pp > 1 ? (A(pp) + A(pp - 1)) / (Real)2 : A(1);
      Real dd;
      if (pp > 1 && pp < na) dd = fabs(A(pp + 1) - A(pp - 1)) / (Real)2;
      else if (pp == 1) dd = sym ? fabs(A(pp + 1) - A(pp)) / (Real)2 : fabs(A(pp + 1) - A(pp));
      else dd = fabs(A(pp) - A(pp - 1));
      dd = dd / (Real)1.e15f;
      e[3] = dd;
      e[4] = (Real)1 / dd;
    }
  }
  __syncthreads();
}

template <typename Real> __host__ __device__ inline size_t table_bytes(int nx, int ny, int nz) {
  return (size_t)(nx + ny + nz) * 5 * sizeof(Real);
}

// The persistent march of one round.  Lanes refill from the sorted queue in
// batches of at least `refill_min` free lanes (or when the warp is empty).
// Gas-only fast path: 64 registers (4 blocks of 256 per SM: the latency of
// the opacity gather and the L2 atomics is hidden by warps); dust fast path:
// 80 registers (3 blocks; 4 spill the scattering state); the exact path keeps
// its registers.
template <bool Fast, bool Dust> struct MarchOccupancy { static constexpr int kMinBlocks = Fast ? (Dust ? 3 : 4) : 1; };

// The march of one model's round by one block: tables, accumulators and
// counters in `smem`, then the warps drain the model's sorted queue.
template <typename Real, bool Fast, bool Dust, bool Replay>
__device__ __forceinline__ void march_body(const DevGrid &g, const DevSources &S, const DevReplay &rp,
                                           const WaveGrid &w, DevCounters *cnt, char *smem) {
  Tables<Real> T;
  build_tables<Real>(g, smem, T);
  LocalCounts lc;
  Marcher<Real, Fast, Dust, Replay> m(g, S, rp, w, T, cnt, lc);
  // per-warp accumulators follow the tables (16-byte aligned)
  float *hot_all = (float *)(smem + ((table_bytes<Real>(g.nx, g.ny, g.nz) + 15) & ~(size_t)15));
  m.hot = hot_all + (threadIdx.x >> 5) * (kHotSrc * kHot3);
  for (int i = threadIdx.x & 31; i < kHotSrc * kHot3; i += 32) m.hot[i] = 0.f;
  m.hot_nu = 0;
  // the warps' counters follow the accumulators (8-byte aligned): crossings
  // (64-bit), then the event counts (32-bit: at most one per queue entry)
  const int nwarps = blockDim.x >> 5;
  unsigned long long *wcx_all = (unsigned long long *)(hot_all + nwarps * (kHotSrc * kHot3));
  m.wcx = wcx_all + (threadIdx.x >> 5);
  m.wc = (unsigned int *)(wcx_all + nwarps) + (threadIdx.x >> 5) * kCntSlots;
  if ((threadIdx.x & 31) == 0) *m.wcx = 0ull;
  if ((threadIdx.x & 31) < kCntSlots) m.wc[threadIdx.x & 31] = 0u;
  // then the warps' escape counts and the stars' origins
  m.esc_n = (unsigned int *)(wcx_all + nwarps) + nwarps * kCntSlots + (threadIdx.x >> 5) * kHotSrc;
  int *org = (int *)((unsigned int *)(wcx_all + nwarps) + nwarps * (kCntSlots + kHotSrc)) + (threadIdx.x >> 5) * kHotSrc;
  if ((threadIdx.x & 31) < kHotSrc) {
    m.esc_n[threadIdx.x & 31] = 0u;
    org[threadIdx.x & 31] = (int)(threadIdx.x & 31) < S.nsrc ? origin_of(g, S.s[threadIdx.x & 31]) : -1;
  }
  m.esc_org = org;
  __syncwarp();
  const unsigned long long t0 = global_ns();
  const unsigned int lane = threadIdx.x & 31;
  const unsigned int lt_mask = (1u << lane) - 1u;
  const unsigned int qlen = w.bin_count[0];
  const int refill_min = w.refill_min;
  // the warp's current chunk [cbeg, cend) of the sorted queue
  // (64..512 packets: at least four chunks per warp; a warp's consecutive
  // chunks lie far apart in the sorted queue, so each starts a new bin and a
  // flush of the warp's accumulators)
  const unsigned int kChunk = max(64u, min(512u, qlen / (gridDim.x * (blockDim.x >> 5) * 4u)));
  unsigned long long cbeg = 0, cend = 0;
  bool qdone = qlen == 0;
  unsigned int iter = 0;
  // warp-aggregated append of the absorbed packets to the next round's list
  auto append_absorbed = [&]() {
    const unsigned int pm = __ballot_sync(0xffffffffu, m.pend);
    if (pm) {
      const int leader = __ffs(pm) - 1;
      unsigned int base = 0;
      if ((int)lane == leader) base = atomicAdd(w.a_count, (unsigned int)__popc(pm));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (m.pend) m.write_absorbed(base + __popc(pm & lt_mask));
    }
  };
  while (true) {
    if (Fast) {
      // parked events are handled together, once they and the free lanes
      // number refill_min or no lane is left crossing; the lanes they free
      // are refilled right after
      const unsigned int parked = __ballot_sync(0xffffffffu, m.valid && m.pev != 0);
      const unsigned int idle = parked | __ballot_sync(0xffffffffu, !m.valid);
      if (parked && (__popc(idle) >= refill_min || idle == 0xffffffffu)) {
        if (m.valid && m.pev != 0) m.handle_parked();
        append_absorbed();
      }
    }
    const unsigned int need = __ballot_sync(0xffffffffu, !m.valid);
    if (!qdone && (__popc(need) >= refill_min || need == 0xffffffffu)) {
      const unsigned int nneed = __popc(need);
      const unsigned long long have = cend - cbeg;
      unsigned long long nbeg = 0;
      if (have < nneed) {  // a new chunk (one atomic per kChunk packets)
        if (lane == 0) nbeg = atomicAdd(w.qhead, (unsigned long long)kChunk);
        nbeg = __shfl_sync(0xffffffffu, nbeg, 0);
      }
      const unsigned int rank = __popc(need & lt_mask);
      unsigned long long q = rank < have ? cbeg + rank : nbeg + (rank - have);
      if (have < nneed) {
        cbeg = nbeg + (nneed - have);
        cend = nbeg + kChunk;
      } else {
        cbeg += nneed;
      }
      if (cend > qlen) cend = qlen;
      if (cbeg >= cend && (have < nneed ? nbeg + kChunk >= qlen : cend >= qlen)) qdone = true;
      if (Fast) {
        // the accumulator follows the bin of the first new packet
        const unsigned long long q0 = __shfl_sync(0xffffffffu, q, __ffs(need) - 1);
        const int nu0 = q0 < qlen ? (int)(__ldg(w.q_meta + q0) & 0xFFFFu) : m.hot_nu;
        if (nu0 != m.hot_nu && nu0 != 0) {
          m.hot_flush(lane);
          m.hot_nu = nu0;
          m.refresh_hot();
        }
      }
      if (!m.valid && q < qlen) m.start((unsigned int)q);
    }
    if (!__any_sync(0xffffffffu, m.valid)) {
      if (qdone) break;
      continue;
    }
    if (Fast) {
      if (m.valid && m.pev == 0) m.advance(w.inner_steps);
    } else {
      if (m.valid) m.step();
      append_absorbed();
    }
    if (((++iter) & 1023u) == 1u) {
      const unsigned long long el = global_ns() - t0;
      const bool stop = (el > cnt->budget_ns) || (*(volatile int *)&cnt->error_code != 0);
      if (__any_sync(0xffffffffu, stop)) {
        if (m.valid && el > cnt->budget_ns) m.fail(MC_ERR_TIMEOUT);
        break;
      }
    }
  }
  if (Fast) {
    m.hot_flush(lane);
    m.count_crossings();
    __syncwarp();
    if (lane == 0) {
      lc.crossings = *m.wcx; lc.absorptions = m.wc[kCntAbs]; lc.scatterings = m.wc[kCntSca];
      lc.escaped = m.wc[kCntEsc]; lc.trapped = m.wc[kCntTrap]; lc.silent = m.wc[kCntSilent];
      lc.safe_hits = m.wc[kCntSafe];
    }
  }
  flush_counts(cnt, lc);
}

template <typename Real, bool Fast, bool Dust, bool Replay>
__global__ void __launch_bounds__(256, (MarchOccupancy<Fast, Dust>::kMinBlocks)) wave_march_kernel(const __grid_constant__ DevGrid g,
                                                        const __grid_constant__ DevSources S,
                                                        const __grid_constant__ DevReplay rp,
                                                        const __grid_constant__ WaveGrid w, DevCounters *cnt) {
  extern __shared__ __align__(16) char smem[];
  march_body<Real, Fast, Dust, Replay>(g, S, rp, w, cnt, smem);
}

// One persistent march over the same round of many models.  Each model's
// round is split into `share` tasks, listed twice (every model's first
// shares, then every model's second ones) so that all models start at once
// and blocks freed by a small model join the larger ones; a block takes
// tasks from one global counter, copies the model's descriptors into shared
// memory, builds its axis tables and joins that model's queue until it is
// empty.  Philox draws only (no replay).
template <typename Real, bool Fast, bool Dust>
__global__ void __launch_bounds__(256, (MarchOccupancy<Fast, Dust>::kMinBlocks))
    wave_march_batch_kernel(const BatchModel *models, int nmodels, unsigned int tasks_per_pass,
                            unsigned int *task_ctr) {
  extern __shared__ __align__(16) char smem[];
  __shared__ __align__(16) BatchModel bm;
  __shared__ int s_model;
  const DevReplay rp{nullptr, 0};
  while (true) {
    if (threadIdx.x == 0) {
      const unsigned int t = atomicAdd(task_ctr, 1u);
      int m = -1;
      if (t < 2u * tasks_per_pass) {
        const unsigned int tp = t % tasks_per_pass;
        int lo = 0, hi = nmodels - 1;  // first model whose task_end > tp
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (models[mid].task_end > tp) hi = mid;
          else lo = mid + 1;
        }
        m = lo;
      }
      s_model = m;
    }
    __syncthreads();
    const int m = s_model;
    if (m < 0) break;
    const int *src = (const int *)(models + m);
    for (int i = threadIdx.x; i < (int)(sizeof(BatchModel) / sizeof(int)); i += blockDim.x) ((int *)&bm)[i] = src[i];
    __syncthreads();
    march_body<Real, Fast, Dust, false>(bm.g, bm.S, rp, bm.w, bm.cnt, smem);
    __syncthreads();
  }
}

template <typename Real> __host__ __device__ inline size_t march_smem_bytes(int nx, int ny, int nz, int warps) {
  return ((table_bytes<Real>(nx, ny, nz) + 15) & ~(size_t)15) + (size_t)warps * kHotSrc * kHot3 * sizeof(float) +
         (size_t)warps * (sizeof(unsigned long long) + (kCntSlots + 2 * kHotSrc) * sizeof(unsigned int));
}

}  // namespace mcg
