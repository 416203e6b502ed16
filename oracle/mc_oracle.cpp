// mc_oracle.cpp -- CPU oracle of mocassin's energy-packet transport.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker the GPU library is
// compared against; nothing in the shipped library links or calls it.  It is
// loaded only by tests/, by __graft_entry__.smoke() and by bench.py's CPU
// baseline leg.
//
// It is a plain restatement, in the reference's own order of operations, of
//   energyPacketDriver   source/photon_mod.f90:26-285 (stellar branch :93-127)
//   energyPacketRun      source/photon_mod.f90:289-487
//   initPhotonPacket     source/photon_mod.f90:491-684
//   getNu2               source/photon_mod.f90:720-764
//   newPhotonPacket      source/photon_mod.f90:768-1059
//   pathSegment          source/photon_mod.f90:1061-2872
//   hg                   source/photon_mod.f90:2875-3101
//   randomUnitVector     source/vector_mod.f90:303-314
// for a single mother grid (nGrids = 1, no sub-grids), no plane-parallel
// ionisation and no 1D mode.  The
// Fortran intrinsic random_number is replaced by one of two draw sources:
// Philox4x32-10 (Salmon et al., SC'11) keyed by (seed, iteration, star) with
// the packet index in the counter, or a replay buffer of draws.
//
// Real = double is the FP64 "reference method" used for the 1e-12 replay
// gate; Real = float mirrors the reference's default 4-byte `real`
// (Makefile:36,53 add no -fdefault-real-8).  Built with -ffp-contract=off so
// that no multiply-add is fused (the GPU FP64 path is compiled the same way).
//
// Parallel over packet histories with OpenMP (the reference is MPI over
// packets, iteration_mod.f90:477-493); estimators are summed with atomics.
//
// Parity unpinned: the reference (Fortran 90 + MPI) cannot be built in this
// image and ships no tests or golden vectors, so this restatement is pinned
// only by the published Philox known-answer vectors and by analytic known
// answers of the transport (vacuum and grey-absorber path lengths, packet
// and energy conservation) in tests/test_oracle_pinning.py.

#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/mocassin_gpu.h"

namespace {

// ---------------------------------------------------------------- Philox
// Philox4x32-10 as published by Salmon, Moraes, Dror and Shaw (2011):
// multipliers 0xD2511F53 / 0xCD9E8D57, Weyl increments 0x9E3779B9 / 0xBB67AE85.
struct Philox4 {
  uint32_t v[4];
};

inline void mulhilo(uint32_t a, uint32_t b, uint32_t &hi, uint32_t &lo) {
  uint64_t p = (uint64_t)a * (uint64_t)b;
  hi = (uint32_t)(p >> 32);
  lo = (uint32_t)p;
}

inline Philox4 philox10(Philox4 ctr, uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0, lo0, hi1, lo1;
    mulhilo(0xD2511F53u, ctr.v[0], hi0, lo0);
    mulhilo(0xCD9E8D57u, ctr.v[2], hi1, lo1);
    Philox4 n;
    n.v[0] = hi1 ^ ctr.v[1] ^ k0;
    n.v[1] = lo1;
    n.v[2] = hi0 ^ ctr.v[3] ^ k1;
    n.v[3] = lo0;
    ctr = n;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return ctr;
}

// Key of one source's stream: seed word plus (iteration, star).
inline void stream_key(uint64_t seed, uint32_t iteration, int32_t istar,
                       uint32_t &k0, uint32_t &k1) {
  k0 = (uint32_t)seed;
  k1 = (uint32_t)(seed >> 32) ^ ((iteration & 0xFFFFFFu) << 8) ^
       ((uint32_t)istar & 0xFFu);
}

// Draw source of one packet history.
struct Draws {
  // philox
  uint32_t k0 = 0, k1 = 0;
  uint64_t packet = 0;
  uint32_t block = 0;
  uint32_t buf[4] = {0, 0, 0, 0};
  int have = 0;
  // replay
  const double *row = nullptr;
  int64_t stride = 0;
  int64_t used = 0;
  bool replay = false;
  bool exhausted = false;

  uint32_t word() {
    if (have == 0) {
      Philox4 c;
      c.v[0] = (uint32_t)packet;
      c.v[1] = (uint32_t)(packet >> 32);
      c.v[2] = block++;
      c.v[3] = 0;
      Philox4 o = philox10(c, k0, k1);
      for (int i = 0; i < 4; ++i) buf[i] = o.v[i];
      have = 4;
    }
    return buf[4 - have--];
  }

  // One uniform in [0,1) at the precision of Real.
  template <typename Real> Real next();
};

template <> double Draws::next<double>() {
  if (replay) {
    if (used >= stride) { exhausted = true; return 0.5; }
    return row[used++];
  }
  uint64_t hi = word();
  uint64_t lo = word();
  uint64_t u53 = (hi << 21) | (lo >> 11);
  return (double)u53 * (1.0 / 9007199254740992.0);
}

template <> float Draws::next<float>() {
  if (replay) {
    if (used >= stride) { exhausted = true; return 0.5f; }
    double x = row[used++];
    return (float)(std::floor(x * 16777216.0) * (1.0 / 16777216.0));
  }
  uint32_t w = word();
  return (float)(w >> 8) * (1.0f / 16777216.0f);
}

// ------------------------------------------------------------ the problem
template <typename Real, typename Acc> struct Problem {
  const mc_grid_t *g;
  int nx, ny, nz, nc, nb;
  std::vector<Real> xA, yA, zA;  // axes at working precision
  bool sym, gas, dust, iso, debug, multistars;
  Real gcx, gcy, gcz, rOut, ionEdge1;
  int recursionLimit, safeLimit;
  Acc *jste, *jdif, *esc;  // accumulators (cell fastest)
  std::atomic<int> err{0};
  std::atomic<int64_t> errPacket{-1};
  std::atomic<int64_t> crossings{0}, absorptions{0}, scatterings{0}, escaped{0},
      lines{0}, trapped{0}, silent{0}, safeHits{0};
  double qphot = 0.0;

  int act(int x, int y, int z) const {
    return g->active[(int64_t)(x - 1) + (int64_t)nx * ((y - 1) + (int64_t)ny * (z - 1))];
  }
  Real opac(int c, int nu) const { return (Real)g->opacity[c + (int64_t)(nc + 1) * (nu - 1)]; }
  Real scaOp(int c, int nu) const { return (Real)g->sca_opac[c + (int64_t)(nc + 1) * (nu - 1)]; }
  Real recPDF(int c, int nu) const { return (Real)g->rec_pdf[c + (int64_t)(nc + 1) * (nu - 1)]; }
  Real dustPDF(int c, int nu) const { return (Real)g->dust_pdf[c + (int64_t)(nc + 1) * (nu - 1)]; }

  void add(Acc *a, int c, int nu, Real v) {
    Acc *p = a + c + (int64_t)(nc + 1) * (nu - 1);
#pragma omp atomic
    *p += (Acc)v;
  }
  // escapedPackets(0:Nc, 0:Nnu, 0:nAngle), cell fastest
  void addEsc(int c, int nu, int plane, double de) {
    if (!esc) return;
    Acc *p = esc + c + (int64_t)(nc + 1) * nu + (int64_t)(nc + 1) * (nb + 1) * plane;
#pragma omp atomic
    *p += (Acc)(Real)de;
  }

  // viewing angles: initCartesianGrid, grid_mod.f90:416-468
  int nAngle = 0, nTheta = 10, nPhi = 20;
  float dTheta = 0.f, dPhi = 0.f;
  std::vector<int> ptheta, pphi;          // viewPointPtheta(0:nTheta), viewPointPphi(0:nPhi)
  std::vector<float> vTheta, vPhi;        // viewPointTheta / viewPointPhi(0:nAngle)
  int setupViews() {
    nAngle = g->n_angle;
    if (nAngle == 0) return 0;
    const float pi = 3.141592654f, twoPi = 2.f * pi;
    nTheta = g->n_theta_bins > 0 ? g->n_theta_bins : 10;
    nPhi = g->n_phi_bins > 0 ? g->n_phi_bins : 20;
    vTheta.assign(g->view_theta, g->view_theta + nAngle + 1);
    vPhi.assign(g->view_phi, g->view_phi + nAngle + 1);
    dTheta = pi / (float)nTheta;
    for (int i = 1; i <= nAngle; ++i) {
      if (vPhi[i] < 0.f) {
        nPhi = 1;
        for (auto &v : vPhi) v = -1.f;
        break;
      }
    }
    dPhi = twoPi / (float)nPhi;
    ptheta.assign(nTheta + 1, 0);
    pphi.assign(nPhi + 1, 0);
    for (int i = 1; i <= nAngle; ++i) {
      if (vTheta[i] > pi / 2.f && sym) return MC_ERR_ARG;
      const int a = (int)(vTheta[i] / dTheta) + 1, b = (int)(vPhi[i] / dPhi) + 1;
      if (a < 0 || a > nTheta || b < 0 || b > nPhi) return MC_ERR_ARG;
      ptheta[a] = i;
      pphi[b] = i;
    }
    return 0;
  }
  // the escape record of photon_mod.f90:372-462 (same at every escape site):
  // false where the reference stops
  bool escapeRecord(int origin, int nuP, Real dx, Real dy, Real dz, double de) {
    if (nAngle == 0) { addEsc(origin, nuP, 0, de); return true; }
    const Real cz = sym ? std::fabs(dz) : dz;
    if (!(cz >= (Real)-1 && cz <= (Real)1)) return false;  // acos -> NaN
    int idirT = (int)(std::acos(cz) / (Real)dTheta) + 1;
    if (idirT > nTheta) idirT = nTheta;
    if (idirT < 1 || idirT > nTheta) return false;
    int idirP;
    if (std::fabs(dx) < (Real)1.e-35f) idirP = 0;
    else if (sym) idirP = (int)(std::atan(std::fabs(dy) / std::fabs(dx)) / (Real)dPhi);
    else idirP = (int)(std::atan(dy / dx) / (Real)dPhi);
    if (idirP < 0) idirP = nPhi + idirP;
    idirP = idirP + 1;
    if (idirP > nPhi) idirP = nPhi;
    if (idirP < 1 || idirP > nPhi) return false;
    const int vt = ptheta[idirT], vp = pphi[idirP];
    if (vt > 0 && vPhi[vt] < 0.f) {
      addEsc(origin, nuP, vt, de);
      addEsc(origin, nuP, 0, de);
    } else if (vt == vp || vTheta[vp] == vTheta[vt] || vPhi[vt] == vPhi[vp]) {
      addEsc(origin, nuP, vt, de);
      if (vt != 0) addEsc(origin, nuP, 0, de);
    } else {
      addEsc(origin, nuP, 0, de);
    }
    return true;
  }
  void fail(int code, int64_t packet) {
    int z = 0;
    if (err.compare_exchange_strong(z, code)) errPacket.store(packet);
  }
};

template <typename Real> struct V3 {
  Real x, y, z;
};

// Packet state that survives between energyPacketRun calls (the chTypeIn,
// positionIn, inX/inY/inZ variables of energyPacketDriver).
enum PType { STELLAR = 0, DIFFUSE = 1, DUSTEMI = 2 };

template <typename Real> struct Packet {
  int nuP;
  int xP, yP, zP;
  int origin;  // origin(2): active cell of emission
  Real nu;
  bool lgStellar, lgLine;
  V3<Real> pos, dir;
};

template <typename Real, typename Acc> class Runner {
 public:
  Problem<Real, Acc> &P;
  const mc_source_t &src;
  Real deltaE;
  Draws d;
  int64_t gpacket;  // global packet index (error reports)
  double qphot = 0.0;

  Runner(Problem<Real, Acc> &p, const mc_source_t &s) : P(p), src(s), deltaE((Real)s.delta_e) {}

  Real rnd() { return d.template next<Real>(); }

  // getNu2, photon_mod.f90:720-764, on a CDF accessed through f(i) (1-based).
  template <typename F> int getNu2(F cdf, bool &ok) {
    Real random = rnd();
    int i;
    for (i = 1; i <= 10000; ++i) {
      if (random == (Real)0 || random == (Real)1 || random == (Real)0.9999999f)
        random = rnd();
      else
        break;
    }
    if (i >= 10000) { ok = false; return 0; }
    int nuP = 1;
    for (int is = 1; is <= P.nb; ++is) {
      if (random >= cdf(is)) nuP = is;
      else break;
    }
    if (nuP < P.nb - 1) nuP = nuP + 1;
    ok = true;
    return nuP;
  }

  // randomUnitVector, vector_mod.f90:303-314
  V3<Real> randomUnitVector() {
    Real r1 = rnd();
    Real w = (Real)2 * r1 - (Real)1;
    Real t = std::sqrt((Real)1 - w * w);
    Real r2 = rnd();
    Real ang = (Real)3.141592654 * ((Real)2 * r2 - (Real)1);
    Real u = t * std::cos(ang);
    Real v = t * std::sin(ang);
    return V3<Real>{u, v, w};
  }

  // initPhotonPacket, photon_mod.f90:491-684 (no plane ionisation).
  bool initPhotonPacket(Packet<Real> &pk, int nuP, V3<Real> position, V3<Real> direction,
                        bool lgLine, bool lgStellar, int xP, int yP, int zP, bool lgHG) {
    pk.dir = direction;
    if (std::isnan(direction.x)) { P.fail(MC_ERR_NAN, gpacket); return false; }
    pk.pos = position;
    pk.nuP = nuP;
    pk.lgStellar = lgStellar;
    if (lgLine) {
      pk.nu = (Real)0;
      pk.lgLine = true;
    } else {
      pk.nu = (Real)P.g->nu_array[nuP - 1];
      pk.lgLine = false;
    }
    pk.xP = xP; pk.yP = yP; pk.zP = zP;
    if (!lgHG || P.iso || pk.lgStellar) {
      for (int irepeat = 1; irepeat <= 1000000; ++irepeat) {
        pk.dir = randomUnitVector();
        if (std::isnan(pk.dir.x)) { P.fail(MC_ERR_NAN, gpacket); return false; }
        if (pk.dir.x != (Real)0 && pk.dir.y != (Real)0 && pk.dir.z != (Real)0) break;
      }
      if (P.sym && pk.lgStellar && !P.multistars) {
        if (pk.dir.x < (Real)0) pk.dir.x = -pk.dir.x;
        if (pk.dir.y < (Real)0) pk.dir.y = -pk.dir.y;
        if (pk.dir.z < (Real)0) pk.dir.z = -pk.dir.z;
      }
    }
    pk.origin = P.act(pk.xP, pk.yP, pk.zP);
    return true;
  }

  // hg, photon_mod.f90:2875-3101.  Returns ierr.
  int hg(Packet<Real> &pk) {
    const Real twoPi = (Real)2 * (Real)3.141592654;
    Real vin[3] = {pk.dir.x, pk.dir.y, pk.dir.z};
    Real vout[3];
    Real hgg = (Real)P.g->g_sca[pk.nuP - 1];
    Real random0 = rnd();
    Real s = (Real)2 * random0 - (Real)1;
    Real cost, sint;
    if (hgg >= (Real)0.0001f) {
      Real q = ((Real)1 - hgg * hgg) / ((Real)1 + hgg * s);
      cost = (Real)0.5 / hgg * ((Real)1 + hgg * hgg - q * q);
    } else {
      cost = s;
    }
    if (cost >= (Real)1) {
      cost = (Real)1; sint = (Real)0;
    } else if (cost < (Real)-1) {
      cost = (Real)-1; sint = (Real)0;
    } else {
      sint = std::sqrt((Real)1 - cost * cost);
    }
    Real random = rnd();
    Real phi = twoPi * random;
    Real cosp = std::cos(phi);
    Real sinp = std::sin(phi);
    Real denom = std::sqrt((Real)1 - vin[2] * vin[2]);
    if (denom > (Real)0.001f) {
      vout[0] = sint / denom * (vin[0] * vin[2] * cosp - vin[1] * sinp) + vin[0] * cost;
      vout[1] = sint / denom * (vin[1] * vin[2] * cosp + vin[0] * sinp) + vin[1] * cost;
      vout[2] = -sint * cosp * denom + vin[2] * cost;
    } else {
      vout[0] = sint * cosp;
      vout[1] = sint * sinp;
      vout[2] = (vin[2] >= (Real)0) ? cost : -cost;
    }
    bool n0 = !std::isnan(vout[0]), n1 = !std::isnan(vout[1]), n2 = !std::isnan(vout[2]);
    if (std::fabs(vout[0]) <= (Real)1 && std::fabs(vout[1]) <= (Real)1 &&
        std::fabs(vout[2]) <= (Real)1 && n0 && n1 && n2) {
      pk.dir.x = vout[0]; pk.dir.y = vout[1]; pk.dir.z = vout[2];
      return 0;
    }
    // Fortran precedence: A .or. B .or. (C .and. n0 .and. n1 .and. n2).  The
    // normalised vector is never written back (reference quirk, :2947-2952).
    if (std::fabs(vout[0]) >= (Real)1 || std::fabs(vout[1]) >= (Real)1 ||
        (std::fabs(vout[2]) >= (Real)1 && n0 && n1 && n2))
      return 0;
    return 1;
  }

  void escape(const Packet<Real> &pk) {
    if (!P.escapeRecord(pk.origin, pk.nuP, pk.dir.x, pk.dir.y, pk.dir.z, (double)deltaE)) { P.fail(MC_ERR_NAN, gpacket); return; }
    P.escaped.fetch_add(1, std::memory_order_relaxed);
  }

  // pathSegment, photon_mod.f90:1061-2872, mother grid only.  Returns true
  // when the packet was absorbed and must be re-emitted (reRun = 1); the new
  // type, position and cell go into (ptype, pos, cell).
  bool pathSegment(Packet<Real> &pk, PType &ptype, V3<Real> &posOut, int cell[3], int64_t &ncross) {
    const auto &xA = P.xA;
    const auto &yA = P.yA;
    const auto &zA = P.zA;
    const int nx = P.nx, ny = P.ny, nz = P.nz;
    auto X = [&](int i) { return xA[i - 1]; };
    auto Y = [&](int i) { return yA[i - 1]; };
    auto Z = [&](int i) { return zA[i - 1]; };

    if (pk.xP <= 0 || pk.xP > nx || pk.yP <= 0 || pk.yP > ny || pk.zP <= 0 || pk.zP > nz) {
      P.fail(MC_ERR_BOUNDS, gpacket); return false;
    }
    V3<Real> rVec = pk.pos;
    V3<Real> vHat = pk.dir;
    if (std::isnan(rVec.x) || std::isnan(vHat.x)) { P.fail(MC_ERR_NAN, gpacket); return false; }
    int xP = pk.xP, yP = pk.yP, zP = pk.zP;
    Real dSx = 0, dSy = 0, dSz = 0, dS = 0, dV, dx = 0, dy = 0, dz = 0;
    Real absTau = (Real)0;
    Real random = rnd();
    Real passProb = -std::log((Real)1 - random);
    const Real tiny = (Real)1.e-10f;
    const Real big = (Real)1.e35f;
    const int safeLimit = P.safeLimit;
    PType packetType = DIFFUSE;
    int i;
    for (i = 1; i <= safeLimit; ++i) {
      // the j loop runs once on a mother grid without sub-grids
      if (xP > nx || xP < 1 || yP > ny || yP < 1 || zP > nz || zP < 1) {
        P.fail(MC_ERR_BOUNDS, gpacket); return false;
      }
      if (P.act(xP, yP, zP) < 0) { P.fail(MC_ERR_UNSUPPORTED, gpacket); return false; }
      if (P.sym) {
        if (rVec.x <= X(1)) { if (vHat.x < (Real)0) vHat.x = -vHat.x; rVec.x = X(1); }
        if (rVec.y <= Y(1)) { if (vHat.y < (Real)0) vHat.y = -vHat.y; rVec.y = Y(1); }
        if (rVec.z <= Z(1)) { if (vHat.z < (Real)0) vHat.z = -vHat.z; rVec.z = Z(1); }
      }
      if (vHat.x > tiny) {
        if (xP < nx) {
          dSx = ((X(xP + 1) + X(xP)) / (Real)2 - rVec.x) / vHat.x;
          if (std::fabs(dSx) < tiny) { rVec.x = (X(xP + 1) + X(xP)) / (Real)2; xP = xP + 1; }
        } else {
          dSx = (X(nx) - rVec.x) / vHat.x;
          if (std::fabs(dSx) < tiny) { rVec.x = X(nx); P.silent.fetch_add(1); return false; }
        }
      } else if (vHat.x < -tiny) {
        if (xP > 1) {
          dSx = ((X(xP) + X(xP - 1)) / (Real)2 - rVec.x) / vHat.x;
          if (std::fabs(dSx) < tiny) { rVec.x = (X(xP) + X(xP - 1)) / (Real)2; xP = xP - 1; }
        } else {
          dSx = (X(1) - rVec.x) / vHat.x;
          if (std::fabs(dSx) < tiny) rVec.x = X(1);
        }
      } else {
        dSx = big;
      }
      if (std::isnan(dSx)) { P.fail(MC_ERR_NAN, gpacket); return false; }

      if (vHat.y > tiny) {
        if (yP < ny) {
          dSy = ((Y(yP + 1) + Y(yP)) / (Real)2 - rVec.y) / vHat.y;
          if (std::fabs(dSy) < tiny) { rVec.y = (Y(yP + 1) + Y(yP)) / (Real)2; yP = yP + 1; }
        } else {
          dSy = (Y(ny) - rVec.y) / vHat.y;
          if (std::fabs(dSy) < tiny) { rVec.y = Y(ny); P.silent.fetch_add(1); return false; }
        }
      } else if (vHat.y < -tiny) {
        if (yP > 1) {
          dSy = ((Y(yP) + Y(yP - 1)) / (Real)2 - rVec.y) / vHat.y;
          if (std::fabs(dSy) < tiny) { rVec.y = (Y(yP) + Y(yP - 1)) / (Real)2; yP = yP - 1; }
        } else {
          dSy = (Y(1) - rVec.y) / vHat.y;
          if (std::fabs(dSy) < tiny) rVec.y = Y(1);
        }
      } else {
        dSy = big;
      }
      if (std::isnan(dSy)) { P.fail(MC_ERR_NAN, gpacket); return false; }

      if (vHat.z > tiny) {
        if (zP < nz) {
          dSz = ((Z(zP + 1) + Z(zP)) / (Real)2 - rVec.z) / vHat.z;
          if (std::fabs(dSz) < tiny) { rVec.z = (Z(zP + 1) + Z(zP)) / (Real)2; zP = zP + 1; }
        } else {
          dSz = (Z(nz) - rVec.z) / vHat.z;
          if (std::fabs(dSz) < tiny) { rVec.z = Z(nz); P.silent.fetch_add(1); return false; }
        }
      } else if (vHat.z < -tiny) {
        if (zP > 1) {
          dSz = ((Z(zP) + Z(zP - 1)) / (Real)2 - rVec.z) / vHat.z;
          if (std::fabs(dSz) < tiny) { rVec.z = (Z(zP) + Z(zP - 1)) / (Real)2; zP = zP - 1; }
        } else {
          dSz = (Z(1) - rVec.z) / vHat.z;
          if (std::fabs(dSz) < tiny) rVec.z = Z(1);
        }
      } else {
        dSz = big;
      }
      if (std::isnan(dSz)) { P.fail(MC_ERR_NAN, gpacket); return false; }
      if (xP > nx || xP < 1 || yP > ny || yP < 1 || zP > nz || zP < 1) {
        P.fail(MC_ERR_BOUNDS, gpacket); return false;
      }
      // (active >= 0: leave the j loop)

      // cater for cells on cell wall (:1395-1397)
      if (std::fabs(dSx) < tiny) dSx = X(nx);
      if (std::fabs(dSy) < tiny) dSy = Y(ny);
      if (std::fabs(dSz) < tiny) dSz = Z(nz);
      dSx = std::fabs(dSx);
      dSy = std::fabs(dSy);
      dSz = std::fabs(dSz);
      if (dSx <= (Real)0) dS = std::min(dSy, dSz);
      else if (dSy <= (Real)0) dS = std::min(dSx, dSz);
      else if (dSz <= (Real)0) dS = std::min(dSx, dSy);
      else { dS = std::min(dSx, dSy); dS = std::min(dS, dSz); }
      if (dS <= (Real)0) { P.fail(MC_ERR_BOUNDS, gpacket); return false; }

      const int a = P.act(xP, yP, zP);
      const Real kap = P.opac(a, pk.nuP);
      Real tauCell = dS * kap;

      // cell volume (:1469-1512)
      if (xP > 1 && xP < nx) dx = std::fabs(X(xP + 1) - X(xP - 1)) / (Real)2;
      else if (xP == 1) dx = P.sym ? std::fabs(X(xP + 1) - X(xP)) / (Real)2 : std::fabs(X(xP + 1) - X(xP));
      else if (xP == nx) dx = std::fabs(X(xP) - X(xP - 1));
      if (yP > 1 && yP < ny) dy = std::fabs(Y(yP + 1) - Y(yP - 1)) / (Real)2;
      else if (yP == 1) dy = P.sym ? std::fabs(Y(yP + 1) - Y(yP)) / (Real)2 : std::fabs(Y(yP + 1) - Y(yP));
      else if (yP == ny) dy = std::fabs(Y(yP) - Y(yP - 1));
      if (zP > 1 && zP < nz) dz = std::fabs(Z(zP + 1) - Z(zP - 1)) / (Real)2;
      else if (zP == 1) dz = P.sym ? std::fabs(Z(zP + 1) - Z(zP)) / (Real)2 : std::fabs(Z(zP + 1) - Z(zP));
      else if (zP == nz) dz = std::fabs(Z(zP) - Z(zP - 1));
      dx = dx / (Real)1.e15f;
      dy = dy / (Real)1.e15f;
      dz = dz / (Real)1.e15f;
      dV = dx * dy * dz;

      ++ncross;
      if ((absTau + tauCell > passProb) && a > 0) {
        // the packet interacts in this cell (:1517-1815)
        Real dlLoc = (passProb - absTau) / kap;
        rVec.x = rVec.x + dlLoc * vHat.x;
        rVec.y = rVec.y + dlLoc * vHat.y;
        rVec.z = rVec.z + dlLoc * vHat.z;
        if (std::isnan(rVec.x) || std::isnan(rVec.y) || std::isnan(rVec.z)) {
          P.fail(MC_ERR_NAN, gpacket); return false;
        }
        if (P.sym) {
          if (rVec.x <= X(1)) { if (vHat.x < (Real)0) vHat.x = -vHat.x; rVec.x = X(1); }
          if (rVec.y <= Y(1)) { if (vHat.y < (Real)0) vHat.y = -vHat.y; rVec.y = Y(1); }
          if (rVec.z <= Z(1)) { if (vHat.z < (Real)0) vHat.z = -vHat.z; rVec.z = Z(1); }
        }
        Real contrib = dlLoc * deltaE / dV;
        if (pk.lgStellar || !P.debug) P.add(P.jste, a, pk.nuP, contrib);
        else P.add(P.jdif, a, pk.nuP, contrib);

        const Real e10 = (Real)1.e10f;
        Real rx = rVec.x / e10, ry = rVec.y / e10, rz = rVec.z / e10;
        if (std::sqrt(rx * rx + ry * ry + rz * rz) * e10 >= P.rOut && P.rOut > (Real)0) {
          escape(pk);
          return false;
        }
        if (P.dust) {
          Real probSca = P.scaOp(a, pk.nuP) / kap;
          Real rr = (Real)1 - rnd();
          bool lgScattered;
          if (rr > probSca) lgScattered = false;
          else if (rr <= probSca) lgScattered = true;
          else { P.fail(MC_ERR_NAN, gpacket); return false; }
          if (!lgScattered) {
            P.absorptions.fetch_add(1, std::memory_order_relaxed);
            packetType = P.gas ? DIFFUSE : DUSTEMI;
            break;
          }
          P.scatterings.fetch_add(1, std::memory_order_relaxed);
          // (grain sublimation checks :1722-1748 need Tdust: not on this path)
          pk.xP = xP; pk.yP = yP; pk.zP = zP;
          Packet<Real> np;
          if (!initPhotonPacket(np, pk.nuP, rVec, pk.dir, false, false, xP, yP, zP, true)) return false;
          pk = np;
          if (!P.iso && !pk.lgStellar) {
            int ihg;
            for (ihg = 1; ihg <= 10; ++ihg)
              if (hg(pk) == 0) break;
          }
          vHat = pk.dir;
          if (std::isnan(pk.dir.x)) { P.fail(MC_ERR_NAN, gpacket); return false; }
          absTau = (Real)0;
          random = rnd();
          passProb = -std::log((Real)1 - random);
        } else {
          P.absorptions.fetch_add(1, std::memory_order_relaxed);
          if (!P.gas) { P.fail(MC_ERR_ARG, gpacket); return false; }
          packetType = DIFFUSE;
          break;
        }
      } else {
        // full crossing (:1817-2731)
        Real contrib = dS * deltaE / dV;
        if (pk.lgStellar || !P.debug) P.add(P.jste, a, pk.nuP, contrib);
        else P.add(P.jdif, a, pk.nuP, contrib);
        absTau = absTau + tauCell;
        rVec.x = rVec.x + dS * vHat.x;
        rVec.y = rVec.y + dS * vHat.y;
        rVec.z = rVec.z + dS * vHat.z;

        if (dS == dSx && vHat.x > (Real)0) xP = xP + 1;
        else if (dS == dSx && vHat.x < (Real)0) xP = xP - 1;
        else if (dS == dSy && vHat.y > (Real)0) yP = yP + 1;
        else if (dS == dSy && vHat.y < (Real)0) yP = yP - 1;
        else if (dS == dSz && vHat.z > (Real)0) zP = zP + 1;
        else if (dS == dSz && vHat.z < (Real)0) zP = zP - 1;

        if (!P.sym) {
          bool lgReturn = false;
          if (rVec.y <= Y(1) - P.gcy || yP < 1) { yP = 1; lgReturn = true; }
          if (rVec.y > Y(ny) + P.gcy || yP > ny) { yP = ny; lgReturn = true; }
          if (rVec.x <= X(1) - P.gcx || xP < 1) { xP = 1; lgReturn = true; }
          if (rVec.x >= X(nx) + P.gcx || xP > nx) { xP = nx; lgReturn = true; }
          if (rVec.z <= Z(1) - P.gcz || zP < 1) { zP = 1; lgReturn = true; }
          if (rVec.z >= Z(nz) + P.gcz || zP > nz) { zP = nz; lgReturn = true; }
          if (lgReturn) { escape(pk); return false; }
        }
        if ((!P.sym && (rVec.x <= X(1) - P.gcx || rVec.y <= Y(1) - P.gcy || rVec.z <= Z(1) - P.gcz)) ||
            rVec.x >= X(nx) + P.gcx || rVec.y >= Y(ny) + P.gcy || rVec.z >= Z(nz) + P.gcz ||
            xP > nx || yP > ny || zP > nz) {
          escape(pk);
          return false;
        }
        if (P.sym) {
          if (rVec.x <= X(1) || xP < 1) { if (vHat.x < (Real)0) vHat.x = -vHat.x; xP = 1; rVec.x = X(1); }
          if (rVec.y <= Y(1) || yP < 1) { if (vHat.y < (Real)0) vHat.y = -vHat.y; yP = 1; rVec.y = Y(1); }
          if (rVec.z <= Z(1) || zP < 1) { if (vHat.z < (Real)0) vHat.z = -vHat.z; zP = 1; rVec.z = Z(1); }
        }
      }
      if (xP > nx || yP > ny || zP > nz) { escape(pk); return false; }
    }
    if (i >= safeLimit) { P.safeHits.fetch_add(1); return false; }
    ptype = packetType;
    posOut = rVec;
    cell[0] = xP; cell[1] = yP; cell[2] = zP;
    return true;
  }

  // energyPacketRun, photon_mod.f90:289-487.  Returns reRun.
  bool energyPacketRun(PType &ptype, V3<Real> &position, int cell[3], int64_t &ncross) {
    Packet<Real> pk;
    bool ok = true;
    if (ptype == STELLAR) {
      int nuP = getNu2([&](int i) { return (Real)src.spec_cdf[i - 1]; }, ok);
      if (!ok || nuP >= P.nb || nuP < 1) { P.fail(MC_ERR_BOUNDS, gpacket); return false; }
      if (P.act(cell[0], cell[1], cell[2]) < 0) { P.fail(MC_ERR_UNSUPPORTED, gpacket); return false; }
      if (!initPhotonPacket(pk, nuP, position, V3<Real>{0, 0, 0}, false, true, cell[0], cell[1], cell[2], false))
        return false;
      if (pk.nu > (Real)1) qphot += (double)(deltaE / ((Real)2.1799153e-11f * pk.nu));
    } else if (ptype == DIFFUSE) {
      if (!P.gas) { P.fail(MC_ERR_ARG, gpacket); return false; }
      int a = P.act(cell[0], cell[1], cell[2]);
      if (a <= 0) { P.fail(MC_ERR_BOUNDS, gpacket); return false; }
      Real random = (Real)1 - rnd();
      if (random <= (Real)P.g->total_lines[a]) {
        // line photon: escapes (no linePDF sampling off the debug path)
        if (!initPhotonPacket(pk, 0, position, V3<Real>{0, 0, 0}, true, false, cell[0], cell[1], cell[2], false))
          return false;
      } else {
        int nuP = getNu2([&](int i) { return P.recPDF(a, i); }, ok);
        if (!ok || nuP >= P.nb || nuP < 1) { P.fail(MC_ERR_BOUNDS, gpacket); return false; }
        if (!initPhotonPacket(pk, nuP, position, V3<Real>{0, 0, 0}, false, false, cell[0], cell[1], cell[2], false))
          return false;
      }
    } else {  // DUSTEMI
      if (!P.dust || P.gas) { P.fail(MC_ERR_ARG, gpacket); return false; }
      int a = P.act(cell[0], cell[1], cell[2]);
      if (a <= 0) { P.fail(MC_ERR_BOUNDS, gpacket); return false; }
      int nuP = getNu2([&](int i) { return P.dustPDF(a, i); }, ok);
      if (!ok || nuP >= P.nb || nuP < 1) { P.fail(MC_ERR_BOUNDS, gpacket); return false; }
      if (!initPhotonPacket(pk, nuP, position, V3<Real>{0, 0, 0}, false, false, cell[0], cell[1], cell[2], false))
        return false;
    }
    if (!P.dust && pk.nu < P.ionEdge1 && !pk.lgLine) {
      escape(pk);
      return false;
    }
    if (!pk.lgLine) return pathSegment(pk, ptype, position, cell, ncross);
    P.lines.fetch_add(1, std::memory_order_relaxed);
    return false;
  }

  // one resonance-line packet (energyPacketDriver :180-266): a "diffuse"
  // packet emitted at the node of cell c0 (xAxis(ix), yAxis(iy), zAxis(iz)),
  // followed through its re-emissions like any other history
  void res_history(int64_t p, int64_t gp, const int c0[3]) {
    gpacket = gp;
    d = Draws();
    d.k0 = k0;
    d.k1 = k1;
    d.packet = (uint64_t)p;
    PType ptype = DIFFUSE;
    V3<Real> position{P.xA[c0[0] - 1], P.yA[c0[1] - 1], P.zA[c0[2] - 1]};
    int cell[3] = {c0[0], c0[1], c0[2]};
    int64_t ncross = 0;
    int i;
    for (i = 1; i <= P.recursionLimit; ++i) {
      bool rerun = energyPacketRun(ptype, position, cell, ncross);
      if (d.exhausted) { P.fail(MC_ERR_REPLAY, gpacket); break; }
      if (!rerun) break;
    }
    if (i >= P.recursionLimit) P.trapped.fetch_add(1, std::memory_order_relaxed);
    P.crossings.fetch_add(ncross, std::memory_order_relaxed);
  }

  // Key / replay row of this source, set once per source.
  uint32_t k0 = 0, k1 = 0;
  const double *replay = nullptr;
  int64_t replayStride = 0;

  // one history of energyPacketDriver (:93-127); p is the packet index within
  // the source, gp the index over all sources (replay row, error reports).
  void history(int64_t p, int64_t gp) {
    gpacket = gp;
    d = Draws();
    d.k0 = k0;
    d.k1 = k1;
    d.packet = (uint64_t)p;
    if (replay) {
      d.replay = true;
      d.row = replay + gp * replayStride;
      d.stride = replayStride;
    }
    PType ptype = STELLAR;
    V3<Real> position{(Real)src.pos[0], (Real)src.pos[1], (Real)src.pos[2]};
    int cell[3] = {src.cell[0], src.cell[1], src.cell[2]};
    int64_t ncross = 0;
    int i;
    for (i = 1; i <= P.recursionLimit; ++i) {
      bool rerun = energyPacketRun(ptype, position, cell, ncross);
      if (d.exhausted) { P.fail(MC_ERR_REPLAY, gpacket); break; }
      if (!rerun) break;
    }
    if (i >= P.recursionLimit) P.trapped.fetch_add(1, std::memory_order_relaxed);
    P.crossings.fetch_add(ncross, std::memory_order_relaxed);
  }
};

template <typename Real, typename Acc>
int run(const mc_grid_t *g, const mc_source_t *src, int nsrc, const mc_run_opts_t *o,
        double *jste, double *jdif, double *esc, mc_stats_t *st, int nthreads, const int32_t *res_counts) {
  Problem<Real, Acc> P;
  P.g = g;
  P.nx = g->nx; P.ny = g->ny; P.nz = g->nz; P.nc = g->ncells; P.nb = g->nbins;
  P.xA.resize(P.nx); P.yA.resize(P.ny); P.zA.resize(P.nz);
  for (int i = 0; i < P.nx; ++i) P.xA[i] = (Real)g->x_axis[i];
  for (int i = 0; i < P.ny; ++i) P.yA[i] = (Real)g->y_axis[i];
  for (int i = 0; i < P.nz; ++i) P.zA[i] = (Real)g->z_axis[i];
  P.sym = g->flags & MC_FLAG_SYMMETRIC_XYZ;
  P.gas = g->flags & MC_FLAG_GAS;
  P.dust = g->flags & MC_FLAG_DUST;
  P.iso = g->flags & MC_FLAG_ISOTROPIC;
  P.debug = g->flags & MC_FLAG_DEBUG;
  P.multistars = g->flags & MC_FLAG_MULTISTARS;
  P.gcx = (Real)g->geo_corr[0]; P.gcy = (Real)g->geo_corr[1]; P.gcz = (Real)g->geo_corr[2];
  P.rOut = (Real)g->r_out;
  P.ionEdge1 = (Real)g->ion_edge1;
  P.recursionLimit = o->recursion_limit > 0 ? o->recursion_limit : 5000;
  P.safeLimit = o->safe_limit > 0 ? o->safe_limit : 500000;

  const int64_t nj = (int64_t)(P.nc + 1) * P.nb;
  if (P.setupViews()) return MC_ERR_ARG;
  const int64_t ne = (int64_t)(P.nc + 1) * (P.nb + 1) * (g->n_angle + 1);
  std::vector<Acc> aj, ad, ae;
  const bool direct = sizeof(Acc) == sizeof(double);
  if (direct) {
    P.jste = (Acc *)jste; P.jdif = (Acc *)jdif; P.esc = (Acc *)esc;
  } else {
    aj.assign(nj, (Acc)0); P.jste = aj.data();
    if (jdif) { ad.assign(nj, (Acc)0); P.jdif = ad.data(); } else P.jdif = nullptr;
    if (esc) { ae.assign(ne, (Acc)0); P.esc = ae.data(); } else P.esc = nullptr;
  }
  if (P.debug && !P.jdif) return MC_ERR_ARG;

  // resonance-line packets: the cell of each packet of a star's block, cells
  // in the reference's loop order (x outer, z inner), resLinePackets(cell)
  // packets each
  std::vector<int> res_cell;
  if (res_counts)
    for (int ix = 1; ix <= P.nx; ++ix)
      for (int iy = 1; iy <= P.ny; ++iy)
        for (int iz = 1; iz <= P.nz; ++iz) {
          const int a = g->active[(ix - 1) + (int64_t)P.nx * ((iy - 1) + (int64_t)P.ny * (iz - 1))];
          if (a <= 0) continue;
          for (int k = 0; k < res_counts[a]; ++k) {
            res_cell.push_back(ix);
            res_cell.push_back(iy);
            res_cell.push_back(iz);
          }
        }
  const int64_t nres = (int64_t)res_cell.size() / 3;
  int64_t total_stellar = 0;
  for (int s = 0; s < nsrc; ++s) total_stellar += src[s].n_packets;

  int64_t base = 0;
  double qphot = 0.0;
  for (int s = 0; s < nsrc; ++s) {
    const mc_source_t &S = src[s];
    uint32_t k0, k1;
    stream_key(o->seed, o->iteration, S.istar, k0, k1);
    const int64_t n = S.n_packets;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel reduction(+ : qphot)
    {
      Runner<Real, Acc> R(P, S);
      R.k0 = k0;
      R.k1 = k1;
      if (o->rng == MC_RNG_REPLAY) {
        R.replay = o->replay;
        R.replayStride = o->replay_stride;
      }
#pragma omp for schedule(dynamic, 64)
      for (int64_t p = 0; p < n; ++p) R.history(p, base + p);
      qphot += R.qphot;
    }
    base += n;
    if (nres > 0) {
      // this star's block of resonance-line packets, after its own packets,
      // drawn from the stream of star index istar | 0x80
      uint32_t r0, r1;
      stream_key(o->seed, o->iteration, S.istar | 0x80, r0, r1);
      const int64_t rbase = total_stellar + (int64_t)s * nres;
#pragma omp parallel
      {
        Runner<Real, Acc> R(P, S);
        R.k0 = r0;
        R.k1 = r1;
#pragma omp for schedule(dynamic, 64)
        for (int64_t p = 0; p < nres; ++p) R.res_history(p, rbase + p, &res_cell[3 * p]);
      }
    }
  }
  if (!direct) {
    for (int64_t i = 0; i < nj; ++i) jste[i] += (double)aj[i];
    if (jdif) for (int64_t i = 0; i < nj; ++i) jdif[i] += (double)ad[i];
    if (esc) for (int64_t i = 0; i < ne; ++i) esc[i] += (double)ae[i];
  }
  if (st) {
    st->crossings = P.crossings.load();
    st->absorptions = P.absorptions.load();
    st->scatterings = P.scatterings.load();
    st->escaped = P.escaped.load();
    st->lines = P.lines.load();
    st->trapped = P.trapped.load();
    st->silent_exits = P.silent.load();
    st->safe_limit_hits = P.safeHits.load();
    st->qphot = qphot;
    st->kernel_ms = 0.0;
    st->error_code = P.err.load();
    st->error_packet = (int32_t)P.errPacket.load();
  }
  return P.err.load();
}

}  // namespace

extern "C" {

// Runs the oracle over all sources.  precision = opts->precision; acc32 != 0
// accumulates the estimators in FP32 as the reference's `real` Jste does
// (FP32 march only).  nthreads <= 0 uses the OpenMP default.
int oracle_transport_run(const mc_grid_t *g, const mc_source_t *src, int32_t nsrc,
                         const mc_run_opts_t *o, double *jste, double *jdif, double *esc,
                         mc_stats_t *st, int32_t nthreads, int32_t acc32) {
  if (!g || !src || !o || !jste || nsrc < 0) return MC_ERR_ARG;
  if (g->n_angle < 0 || g->n_angle > 2 || (g->n_angle > 0 && (!g->view_theta || !g->view_phi))) return MC_ERR_ARG;
  if (o->rng == MC_RNG_REPLAY && (!o->replay || o->replay_stride <= 0)) return MC_ERR_ARG;
  if (o->precision == MC_PREC_FP64)
    return run<double, double>(g, src, nsrc, o, jste, jdif, esc, st, nthreads, nullptr);
  if (acc32) return run<float, float>(g, src, nsrc, o, jste, jdif, esc, st, nthreads, nullptr);
  return run<float, double>(g, src, nsrc, o, jste, jdif, esc, st, nthreads, nullptr);
}

// The same with resonance-line packets: res_counts [Nc+1] = resLinePackets
// per active cell, a block of them after each star's packets
// (energyPacketDriver :180-266).  Philox draws only.
int oracle_transport_run_res(const mc_grid_t *g, const mc_source_t *src, int32_t nsrc,
                             const mc_run_opts_t *o, double *jste, double *jdif, double *esc,
                             mc_stats_t *st, int32_t nthreads, const int32_t *res_counts) {
  if (!g || !src || !o || !jste || nsrc < 0 || !res_counts) return MC_ERR_ARG;
  if (o->rng != MC_RNG_PHILOX) return MC_ERR_ARG;
  if (g->n_angle < 0 || g->n_angle > 2 || (g->n_angle > 0 && (!g->view_theta || !g->view_phi))) return MC_ERR_ARG;
  if (o->precision == MC_PREC_FP64)
    return run<double, double>(g, src, nsrc, o, jste, jdif, esc, st, nthreads, res_counts);
  return run<float, double>(g, src, nsrc, o, jste, jdif, esc, st, nthreads, res_counts);
}

// Philox4x32-10 of one block, for the known-answer tests.
void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  Philox4 c;
  for (int i = 0; i < 4; ++i) c.v[i] = ctr[i];
  Philox4 r = philox10(c, key[0], key[1]);
  for (int i = 0; i < 4; ++i) out[i] = r.v[i];
}

// First n draws of one packet's stream (precision 0 = FP32, 1 = FP64).
void oracle_draws(uint64_t seed, uint32_t iteration, int32_t istar, uint64_t packet,
                  int32_t precision, int32_t n, double *out) {
  Draws d;
  stream_key(seed, iteration, istar, d.k0, d.k1);
  d.packet = packet;
  for (int i = 0; i < n; ++i)
    out[i] = precision == MC_PREC_FP64 ? d.next<double>() : (double)d.next<float>();
}

}  // extern "C"
