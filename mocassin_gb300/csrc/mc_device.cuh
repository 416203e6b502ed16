// mc_device.cuh -- device-side types shared by the transport kernels:
// the resident grid view, per-source parameters, Philox4x32-10 draw streams
// and the error / counter plumbing.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/mocassin_gpu.h"

namespace mcg {

constexpr int kMaxSources = 16;

// Resident grid in HBM.  Layouts:
//  active   [nz][ny][nx] int32 (x fastest, the Fortran order)
//  opacity  [nb][nc+1] float (cell fastest, the Fortran order: a packet at
//           fixed nu reads one contiguous slab)
//  sca      [nb][nc+1] float or null
//  rec_cdf  [nc+1][nb] float: CDF rows transposed to one contiguous row per
//           cell and made monotone by a running maximum, so a binary search
//           returns exactly what getNu2's linear scan returns
//  dust_cdf [nc+1][nb] float or null
//  dx/dy/dz per-index cell widths / 1e15 (the dV factors of
//           photon_mod.f90:1469-1512) at FP32 and FP64
//  jste/jdif [nb][nc+1] double accumulators; esc [n_angle+1][nb+1][nc+1] double
struct DevGrid {
  int nx, ny, nz, nc, nb;
  const float *xa, *ya, *za;
  const int32_t *active;
  const float *opacity;
  const float *sca;
  const float *rec_cdf;
  const float *dust_cdf;
  const float *total_lines;
  const float *nu;
  const float *gsca;
  const float *dx32, *dy32, *dz32;
  const double *dx64, *dy64, *dz64;
  float gc[3];
  float rout;
  float ion_edge1;
  uint32_t flags;
  int recursion_limit;
  int safe_limit;
  double *jste, *jdif, *esc;
  // viewing angles of the escape SED (n_angle = 0: plane 0 only)
  int n_angle, n_theta, n_phi;
  float dtheta, dphi;     // Pi / totAngleBinsTheta, twoPi / totAngleBinsPhi (FP32)
  const uint8_t *view;    // [n_theta+1][n_phi+1] viewpoint of each (theta, phi) bin, 0 = none
};

struct DevSource {
  const float *cdf;      // [nb] device copy of inSpectrumProbDen(iStar,:)
  int cell[3];
  float pos[3];
  double delta_e;
  uint32_t k0, k1;       // Philox key
  long long n;           // packets
  long long base;        // index of the first packet over all sources
};

struct DevSources {
  int nsrc;        // stars (entries 0..nsrc-1)
  int nres;        // resonance-line blocks that follow them (0 or nsrc), one per star
  long long total; // stellar packets (the resonance packets' ids follow)
  DevSource s[kMaxSources];
};

// Counters + first error, in device memory.
struct DevCounters {
  unsigned long long crossings, absorptions, scatterings, escaped, lines, trapped, silent,
      safe_hits;
  double qphot;
  int error_code;
  int error_packet;
  unsigned long long budget_ns;  // per-thread watchdog, from its kernel entry
};

// Replay draws (MC_RNG_REPLAY): row p of [total][stride] doubles.
struct DevReplay {
  const double *draws;
  long long stride;
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void raise_error(DevCounters *c, int code, long long packet) {
  if (atomicCAS(&c->error_code, 0, code) == 0) c->error_packet = (int)packet;
}

// Viewing-angle plane of an escaping packet (photon_mod.f90:372-412, and the
// same code at the six escape sites of pathSegment): theta bin from acos of
// the z cosine, phi bin from atan (not atan2) of y/x, both on |.| in a
// symmetric octant, clamped to the last bin; the table holds the viewpoint
// the reference's viewPointPtheta / viewPointPphi tests select (0 = none).
// ok = false where the reference stops (a cosine outside [-1, 1]).
template <typename Real>
__device__ __forceinline__ int escape_view(const DevGrid &g, Real dx, Real dy, Real dz, bool &ok) {
  const bool sym = g.flags & MC_FLAG_SYMMETRIC_XYZ;
  const Real cz = sym ? fabs(dz) : dz;
  ok = cz >= (Real)-1 && cz <= (Real)1;
  if (!ok) return 0;
  int it = (int)(acos(cz) / (Real)g.dtheta) + 1;
  if (it > g.n_theta) it = g.n_theta;
  int ip = 0;
  if (!(fabs(dx) < (Real)1.e-35f)) {
    const Real t = sym ? atan(fabs(dy) / fabs(dx)) : atan(dy / dx);
    ip = (int)(t / (Real)g.dphi);
  }
  if (ip < 0) ip = g.n_phi + ip;
  ip = ip + 1;
  if (ip > g.n_phi) ip = g.n_phi;
  ok = ip >= 1;
  return ok ? (int)__ldg(g.view + it * (g.n_phi + 1) + ip) : 0;
}

// escapedPackets(origin, nuP, 0) += dE, and plane `view` too when view > 0.
__device__ __forceinline__ void add_escape(const DevGrid &g, int origin, int nuP, int view, double de) {
  if (!g.esc) return;
  double *p = g.esc + origin + (long long)(g.nc + 1) * nuP;
  atomicAdd(p, de);
  if (view > 0) atomicAdd(p + (long long)(g.nc + 1) * (g.nb + 1) * view, de);
}

// Philox4x32-10, Salmon et al. (SC'11).
__device__ __forceinline__ uint4 philox4x32_10(uint4 ctr, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t lo0 = 0xD2511F53u * ctr.x;
    const uint32_t hi0 = __umulhi(0xD2511F53u, ctr.x);
    const uint32_t lo1 = 0xCD9E8D57u * ctr.z;
    const uint32_t hi1 = __umulhi(0xCD9E8D57u, ctr.z);
    ctr = make_uint4(hi1 ^ ctr.y ^ k0, lo1, hi0 ^ ctr.w ^ k1, lo0);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return ctr;
}

// Per-history draw stream.  The packet's stream is the sequence of Philox
// blocks (packet_lo, packet_hi, block, 0); an FP32 draw takes one word
// (top 24 bits), an FP64 draw two words (53 bits).  In replay mode draws are
// read from row `row` of the replay buffer instead.
struct Stream {
  uint32_t k0, k1;
  uint32_t plo, phi;
  uint32_t block;
  uint32_t buf[4];
  int have;
  const double *row;
  long long stride, used;
  bool exhausted;

  __device__ __forceinline__ void init(uint32_t key0, uint32_t key1, unsigned long long packet,
                                       const DevReplay &rp, long long gpacket) {
    k0 = key0; k1 = key1;
    plo = (uint32_t)packet; phi = (uint32_t)(packet >> 32);
    block = 0; have = 0;
    exhausted = false;
    used = 0;
    if (rp.draws) { row = rp.draws + gpacket * rp.stride; stride = rp.stride; }
    else { row = nullptr; stride = 0; }
  }
  __device__ __forceinline__ uint32_t word() {
    if (have == 0) {
      uint4 o = philox4x32_10(make_uint4(plo, phi, block++, 0u), k0, k1);
      buf[0] = o.x; buf[1] = o.y; buf[2] = o.z; buf[3] = o.w;
      have = 4;
    }
    return buf[4 - have--];
  }
  template <typename Real> __device__ __forceinline__ Real next();
};

template <> __device__ __forceinline__ double Stream::next<double>() {
  if (row) {
    if (used >= stride) { exhausted = true; return 0.5; }
    return row[used++];
  }
  const unsigned long long hi = word();
  const unsigned long long lo = word();
  const unsigned long long u53 = (hi << 21) | (lo >> 11);
  return (double)u53 * (1.0 / 9007199254740992.0);
}

template <> __device__ __forceinline__ float Stream::next<float>() {
  if (row) {
    if (used >= stride) { exhausted = true; return 0.5f; }
    const double x = row[used++];
    return (float)(floor(x * 16777216.0) * (1.0 / 16777216.0));
  }
  return (float)(word() >> 8) * (1.0f / 16777216.0f);
}

}  // namespace mcg
