// transport_plain.cuh -- the plain GPU form of mocassin's packet transport.
//
// One thread owns one packet history from stellar emission through every
// re-emission until it escapes, becomes a line packet or is trapped
// (energyPacketDriver source/photon_mod.f90:93-127).  Within a history the
// arithmetic keeps the reference's order of operations so that the FP64
// instantiation, compiled without multiply-add contraction, reproduces the
// FP64 oracle on the same draws:
//   energyPacketRun  photon_mod.f90:289-487
//   newPhotonPacket  photon_mod.f90:768-1059 / initPhotonPacket :491-684
//   getNu2           photon_mod.f90:720-764 (binary search on the
//                    running-max CDF row == the linear scan)
//   pathSegment      photon_mod.f90:1061-2872 (mother grid only)
//   hg               photon_mod.f90:2875-3101
// Estimators go straight to FP64 global sums with atomics.
#pragma once

#include "mc_device.cuh"

namespace mcg {

template <typename Real> struct R3 {
  Real x, y, z;
};

enum PType { STELLAR = 0, DIFFUSE = 1, DUSTEMI = 2 };

template <typename Real> struct Pk {
  int nuP, xP, yP, zP, origin;
  Real nu;
  bool stellar, line;
  R3<Real> pos, dir;
};

template <typename Real> struct Axes {
  __device__ __forceinline__ static Real w(const DevGrid &g, int axis, int i);
};
template <> struct Axes<float> {
  __device__ __forceinline__ static float w(const DevGrid &g, int axis, int i) {
    return axis == 0 ? g.dx32[i] : (axis == 1 ? g.dy32[i] : g.dz32[i]);
  }
};
template <> struct Axes<double> {
  __device__ __forceinline__ static double w(const DevGrid &g, int axis, int i) {
    return axis == 0 ? g.dx64[i] : (axis == 1 ? g.dy64[i] : g.dz64[i]);
  }
};

struct LocalCounts {
  unsigned long long crossings = 0, absorptions = 0, scatterings = 0, escaped = 0, lines = 0,
                     trapped = 0, silent = 0, safe_hits = 0;
  double qphot = 0.0;
};

// Layout 0: emission CDF rows are contiguous per cell and monotone (the
// context's re-laid-out copy), sampled by binary search.  Layout 1: the
// caller's Fortran arrays recPDF(0:Nc, 1:nbins) (cell fastest), sampled by
// getNu2's own linear scan over a strided row.
template <typename Real, int Layout = 0> struct History {
  const DevGrid &g;
  const DevSource &src;
  DevCounters *cnt;
  Stream st;
  LocalCounts &lc;
  long long gpacket;
  unsigned long long t0;  // %globaltimer at kernel entry (watchdog)
  Real deltaE;
  bool failed;

  __device__ History(const DevGrid &g_, const DevSource &s_, DevCounters *c_, LocalCounts &lc_)
      : g(g_), src(s_), cnt(c_), lc(lc_), failed(false) {
    deltaE = (Real)s_.delta_e;
  }

  __device__ __forceinline__ void fail(int code) {
    if (!failed) raise_error(cnt, code, gpacket);
    failed = true;
  }
  __device__ __forceinline__ Real rnd() { return st.template next<Real>(); }
  __device__ __forceinline__ Real X(int i) const { return (Real)g.xa[i - 1]; }
  __device__ __forceinline__ Real Y(int i) const { return (Real)g.ya[i - 1]; }
  __device__ __forceinline__ Real Z(int i) const { return (Real)g.za[i - 1]; }
  __device__ __forceinline__ int act(int x, int y, int z) const {
    return __ldg(g.active + (x - 1) + (long long)g.nx * ((y - 1) + (long long)g.ny * (z - 1)));
  }

  // getNu2 on a monotone CDF row: the count c of leading entries <= random
  // gives nuP = max(c, 1), then +1 when below nbins-1.
  __device__ int getNu2(const float *row, long long stride) {
    Real random = rnd();
    int i;
    for (i = 1; i <= 10000; ++i) {
      if (random == (Real)0 || random == (Real)1 || random == (Real)0.9999999f) random = rnd();
      else break;
    }
    if (i >= 10000) { fail(MC_ERR_BOUNDS); return 0; }
    int nuP = 1;
    if constexpr (Layout == 0) {
      int lo = 0, hi = g.nb;  // first index with row[idx] > random
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (random >= (Real)__ldg(row + mid)) lo = mid + 1;
        else hi = mid;
      }
      nuP = lo < 1 ? 1 : lo;
    } else {
      for (int is = 1; is <= g.nb; ++is) {  // photon_mod.f90:746-753
        if (random >= (Real)__ldg(row + (long long)(is - 1) * stride)) nuP = is;
        else break;
      }
    }
    if (nuP < g.nb - 1) nuP = nuP + 1;
    return nuP;
  }

  __device__ R3<Real> randomUnitVector() {
    const Real r1 = rnd();
    const Real w = (Real)2 * r1 - (Real)1;
    const Real t = sqrt((Real)1 - w * w);
    const Real r2 = rnd();
    const Real ang = (Real)3.141592654 * ((Real)2 * r2 - (Real)1);
    Real s, c;
    s = sin(ang);
    c = cos(ang);
    return R3<Real>{t * c, t * s, w};
  }

  __device__ bool initPacket(Pk<Real> &pk, int nuP, R3<Real> position, R3<Real> direction, bool line,
                             bool stellar, int xP, int yP, int zP, bool lgHG) {
    pk.dir = direction;
    if (isnan(direction.x)) { fail(MC_ERR_NAN); return false; }
    pk.pos = position;
    pk.nuP = nuP;
    pk.stellar = stellar;
    if (line) { pk.nu = (Real)0; pk.line = true; }
    else { pk.nu = (Real)__ldg(g.nu + nuP - 1); pk.line = false; }
    pk.xP = xP; pk.yP = yP; pk.zP = zP;
    const bool iso = g.flags & MC_FLAG_ISOTROPIC;
    if (!lgHG || iso || pk.stellar) {
      for (int irep = 1; irep <= 1000000; ++irep) {
        pk.dir = randomUnitVector();
        if (isnan(pk.dir.x)) { fail(MC_ERR_NAN); return false; }
        if (pk.dir.x != (Real)0 && pk.dir.y != (Real)0 && pk.dir.z != (Real)0) break;
      }
      if ((g.flags & MC_FLAG_SYMMETRIC_XYZ) && pk.stellar && !(g.flags & MC_FLAG_MULTISTARS)) {
        if (pk.dir.x < (Real)0) pk.dir.x = -pk.dir.x;
        if (pk.dir.y < (Real)0) pk.dir.y = -pk.dir.y;
        if (pk.dir.z < (Real)0) pk.dir.z = -pk.dir.z;
      }
    }
    pk.origin = act(pk.xP, pk.yP, pk.zP);
    return true;
  }

  __device__ int hg(Pk<Real> &pk) {
    const Real twoPi = (Real)2 * (Real)3.141592654;
    const Real vin0 = pk.dir.x, vin1 = pk.dir.y, vin2 = pk.dir.z;
    Real v0, v1, v2;
    const Real hgg = (Real)__ldg(g.gsca + pk.nuP - 1);
    const Real random0 = rnd();
    const Real s = (Real)2 * random0 - (Real)1;
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
    const Real random = rnd();
    const Real phi = twoPi * random;
    const Real cosp = cos(phi);
    const Real sinp = sin(phi);
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
      pk.dir.x = v0; pk.dir.y = v1; pk.dir.z = v2;
      return 0;
    }
    if (fabs(v0) >= (Real)1 || fabs(v1) >= (Real)1 || (fabs(v2) >= (Real)1 && n0 && n1 && n2)) return 0;
    return 1;
  }

  __device__ __forceinline__ void escape(const Pk<Real> &pk) {
    int view = 0;
    if (g.n_angle > 0) {
      bool ok;
      view = escape_view<Real>(g, pk.dir.x, pk.dir.y, pk.dir.z, ok);
      if (!ok) { fail(MC_ERR_NAN); return; }
    }
    add_escape(g, pk.origin, pk.nuP, view, (double)deltaE);
    ++lc.escaped;
  }
  __device__ __forceinline__ void addJ(const Pk<Real> &pk, int a, Real v) {
    double *J = (pk.stellar || !(g.flags & MC_FLAG_DEBUG)) ? g.jste : g.jdif;
    atomicAdd(J + a + (long long)(g.nc + 1) * (pk.nuP - 1), (double)v);
  }

  // pathSegment; true = absorbed, re-emit as ptype from (posOut, cell).
  __device__ bool pathSegment(Pk<Real> &pk, int &ptype, R3<Real> &posOut, int cell[3]) {
    const int nx = g.nx, ny = g.ny, nz = g.nz;
    const bool sym = g.flags & MC_FLAG_SYMMETRIC_XYZ;
    if (pk.xP <= 0 || pk.xP > nx || pk.yP <= 0 || pk.yP > ny || pk.zP <= 0 || pk.zP > nz) {
      fail(MC_ERR_BOUNDS); return false;
    }
    R3<Real> r = pk.pos;
    R3<Real> v = pk.dir;
    if (isnan(r.x) || isnan(v.x)) { fail(MC_ERR_NAN); return false; }
    int xP = pk.xP, yP = pk.yP, zP = pk.zP;
    Real dSx = 0, dSy = 0, dSz = 0, dS;
    Real absTau = (Real)0;
    Real random = rnd();
    Real passProb = -log((Real)1 - random);
    const Real tiny = (Real)1.e-10f;
    const Real big = (Real)1.e35f;
    const Real gcx = (Real)g.gc[0], gcy = (Real)g.gc[1], gcz = (Real)g.gc[2];
    const Real X1 = X(1), Y1 = Y(1), Z1 = Z(1), Xn = X(nx), Yn = Y(ny), Zn = Z(nz);
    int packetType = DIFFUSE;
    int i;
    for (i = 1; i <= g.safe_limit; ++i) {
      if (xP > nx || xP < 1 || yP > ny || yP < 1 || zP > nz || zP < 1) { fail(MC_ERR_BOUNDS); return false; }
      if (sym) {
        if (r.x <= X1) { if (v.x < (Real)0) v.x = -v.x; r.x = X1; }
        if (r.y <= Y1) { if (v.y < (Real)0) v.y = -v.y; r.y = Y1; }
        if (r.z <= Z1) { if (v.z < (Real)0) v.z = -v.z; r.z = Z1; }
      }
      if (v.x > tiny) {
        if (xP < nx) {
          dSx = ((X(xP + 1) + X(xP)) / (Real)2 - r.x) / v.x;
          if (fabs(dSx) < tiny) { r.x = (X(xP + 1) + X(xP)) / (Real)2; xP = xP + 1; }
        } else {
          dSx = (Xn - r.x) / v.x;
          if (fabs(dSx) < tiny) { ++lc.silent; return false; }
        }
      } else if (v.x < -tiny) {
        if (xP > 1) {
          dSx = ((X(xP) + X(xP - 1)) / (Real)2 - r.x) / v.x;
          if (fabs(dSx) < tiny) { r.x = (X(xP) + X(xP - 1)) / (Real)2; xP = xP - 1; }
        } else {
          dSx = (X1 - r.x) / v.x;
          if (fabs(dSx) < tiny) r.x = X1;
        }
      } else {
        dSx = big;
      }
      if (v.y > tiny) {
        if (yP < ny) {
          dSy = ((Y(yP + 1) + Y(yP)) / (Real)2 - r.y) / v.y;
          if (fabs(dSy) < tiny) { r.y = (Y(yP + 1) + Y(yP)) / (Real)2; yP = yP + 1; }
        } else {
          dSy = (Yn - r.y) / v.y;
          if (fabs(dSy) < tiny) { ++lc.silent; return false; }
        }
      } else if (v.y < -tiny) {
        if (yP > 1) {
          dSy = ((Y(yP) + Y(yP - 1)) / (Real)2 - r.y) / v.y;
          if (fabs(dSy) < tiny) { r.y = (Y(yP) + Y(yP - 1)) / (Real)2; yP = yP - 1; }
        } else {
          dSy = (Y1 - r.y) / v.y;
          if (fabs(dSy) < tiny) r.y = Y1;
        }
      } else {
        dSy = big;
      }
      if (v.z > tiny) {
        if (zP < nz) {
          dSz = ((Z(zP + 1) + Z(zP)) / (Real)2 - r.z) / v.z;
          if (fabs(dSz) < tiny) { r.z = (Z(zP + 1) + Z(zP)) / (Real)2; zP = zP + 1; }
        } else {
          dSz = (Zn - r.z) / v.z;
          if (fabs(dSz) < tiny) { ++lc.silent; return false; }
        }
      } else if (v.z < -tiny) {
        if (zP > 1) {
          dSz = ((Z(zP) + Z(zP - 1)) / (Real)2 - r.z) / v.z;
          if (fabs(dSz) < tiny) { r.z = (Z(zP) + Z(zP - 1)) / (Real)2; zP = zP - 1; }
        } else {
          dSz = (Z1 - r.z) / v.z;
          if (fabs(dSz) < tiny) r.z = Z1;
        }
      } else {
        dSz = big;
      }
      if (isnan(dSx) || isnan(dSy) || isnan(dSz)) { fail(MC_ERR_NAN); return false; }
      if (xP > nx || xP < 1 || yP > ny || yP < 1 || zP > nz || zP < 1) { fail(MC_ERR_BOUNDS); return false; }

      if (fabs(dSx) < tiny) dSx = Xn;
      if (fabs(dSy) < tiny) dSy = Yn;
      if (fabs(dSz) < tiny) dSz = Zn;
      dSx = fabs(dSx);
      dSy = fabs(dSy);
      dSz = fabs(dSz);
      if (dSx <= (Real)0) dS = fmin(dSy, dSz);
      else if (dSy <= (Real)0) dS = fmin(dSx, dSz);
      else if (dSz <= (Real)0) dS = fmin(dSx, dSy);
      else { dS = fmin(dSx, dSy); dS = fmin(dS, dSz); }
      if (dS <= (Real)0) { fail(MC_ERR_BOUNDS); return false; }

      const int a = act(xP, yP, zP);
      const Real kap = (Real)__ldg(g.opacity + a + (long long)(g.nc + 1) * (pk.nuP - 1));
      const Real tauCell = dS * kap;
      const Real dV = Axes<Real>::w(g, 0, xP - 1) * Axes<Real>::w(g, 1, yP - 1) * Axes<Real>::w(g, 2, zP - 1);

      ++lc.crossings;
      if ((lc.crossings & 4095ull) == 0ull) {
        if (global_ns() - t0 > cnt->budget_ns) { fail(MC_ERR_TIMEOUT); return false; }
      }
      if ((absTau + tauCell > passProb) && a > 0) {
        const Real dlLoc = (passProb - absTau) / kap;
        r.x = r.x + dlLoc * v.x;
        r.y = r.y + dlLoc * v.y;
        r.z = r.z + dlLoc * v.z;
        if (isnan(r.x) || isnan(r.y) || isnan(r.z)) { fail(MC_ERR_NAN); return false; }
        if (sym) {
          if (r.x <= X1) { if (v.x < (Real)0) v.x = -v.x; r.x = X1; }
          if (r.y <= Y1) { if (v.y < (Real)0) v.y = -v.y; r.y = Y1; }
          if (r.z <= Z1) { if (v.z < (Real)0) v.z = -v.z; r.z = Z1; }
        }
        addJ(pk, a, dlLoc * deltaE / dV);
        const Real e10 = (Real)1.e10f;
        const Real rx = r.x / e10, ry = r.y / e10, rz = r.z / e10;
        const Real rout = (Real)g.rout;
        if (sqrt(rx * rx + ry * ry + rz * rz) * e10 >= rout && rout > (Real)0) {
          escape(pk);
          return false;
        }
        if (g.flags & MC_FLAG_DUST) {
          const Real probSca = (Real)__ldg(g.sca + a + (long long)(g.nc + 1) * (pk.nuP - 1)) / kap;
          const Real rr = (Real)1 - rnd();
          bool scattered;
          if (rr > probSca) scattered = false;
          else if (rr <= probSca) scattered = true;
          else { fail(MC_ERR_NAN); return false; }
          if (!scattered) {
            ++lc.absorptions;
            packetType = (g.flags & MC_FLAG_GAS) ? DIFFUSE : DUSTEMI;
            break;
          }
          ++lc.scatterings;
          Pk<Real> np;
          if (!initPacket(np, pk.nuP, r, pk.dir, false, false, xP, yP, zP, true)) return false;
          pk = np;
          if (!(g.flags & MC_FLAG_ISOTROPIC) && !pk.stellar) {
            for (int ihg = 1; ihg <= 10; ++ihg)
              if (hg(pk) == 0) break;
          }
          v = pk.dir;
          if (isnan(pk.dir.x)) { fail(MC_ERR_NAN); return false; }
          absTau = (Real)0;
          random = rnd();
          passProb = -log((Real)1 - random);
        } else {
          ++lc.absorptions;
          packetType = DIFFUSE;
          break;
        }
      } else {
        addJ(pk, a, dS * deltaE / dV);
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
        if (!sym) {
          bool ret = false;
          if (r.y <= Y1 - gcy || yP < 1) { yP = 1; ret = true; }
          if (r.y > Yn + gcy || yP > ny) { yP = ny; ret = true; }
          if (r.x <= X1 - gcx || xP < 1) { xP = 1; ret = true; }
          if (r.x >= Xn + gcx || xP > nx) { xP = nx; ret = true; }
          if (r.z <= Z1 - gcz || zP < 1) { zP = 1; ret = true; }
          if (r.z >= Zn + gcz || zP > nz) { zP = nz; ret = true; }
          if (ret) { escape(pk); return false; }
        }
        if ((!sym && (r.x <= X1 - gcx || r.y <= Y1 - gcy || r.z <= Z1 - gcz)) || r.x >= Xn + gcx ||
            r.y >= Yn + gcy || r.z >= Zn + gcz || xP > nx || yP > ny || zP > nz) {
          escape(pk);
          return false;
        }
        if (sym) {
          if (r.x <= X1 || xP < 1) { if (v.x < (Real)0) v.x = -v.x; xP = 1; r.x = X1; }
          if (r.y <= Y1 || yP < 1) { if (v.y < (Real)0) v.y = -v.y; yP = 1; r.y = Y1; }
          if (r.z <= Z1 || zP < 1) { if (v.z < (Real)0) v.z = -v.z; zP = 1; r.z = Z1; }
        }
      }
      if (xP > nx || yP > ny || zP > nz) { escape(pk); return false; }
    }
    if (i >= g.safe_limit) { ++lc.safe_hits; return false; }
    ptype = packetType;
    posOut = r;
    cell[0] = xP; cell[1] = yP; cell[2] = zP;
    return true;
  }

  __device__ bool energyPacketRun(int &ptype, R3<Real> &position, int cell[3]) {
    Pk<Real> pk;
    const R3<Real> zero{(Real)0, (Real)0, (Real)0};
    if (ptype == STELLAR) {
      const int nuP = getNu2(src.cdf, 1);
      if (failed || nuP >= g.nb || nuP < 1) { fail(MC_ERR_BOUNDS); return false; }
      if (!initPacket(pk, nuP, position, zero, false, true, cell[0], cell[1], cell[2], false)) return false;
      if (pk.nu > (Real)1) lc.qphot += (double)(deltaE / ((Real)2.1799153e-11f * pk.nu));
    } else {
      const int a = act(cell[0], cell[1], cell[2]);
      if (a <= 0) { fail(MC_ERR_BOUNDS); return false; }
      if (ptype == DIFFUSE) {
        const Real random = (Real)1 - rnd();
        if (random <= (Real)__ldg(g.total_lines + a)) {
          if (!initPacket(pk, 0, position, zero, true, false, cell[0], cell[1], cell[2], false)) return false;
        } else {
          const int nuP = Layout == 0 ? getNu2(g.rec_cdf + (long long)a * g.nb, 1)
                                      : getNu2(g.rec_cdf + a, (long long)g.nc + 1);
          if (failed || nuP >= g.nb || nuP < 1) { fail(MC_ERR_BOUNDS); return false; }
          if (!initPacket(pk, nuP, position, zero, false, false, cell[0], cell[1], cell[2], false)) return false;
        }
      } else {
        const int nuP = Layout == 0 ? getNu2(g.dust_cdf + (long long)a * g.nb, 1)
                                    : getNu2(g.dust_cdf + a, (long long)g.nc + 1);
        if (failed || nuP >= g.nb || nuP < 1) { fail(MC_ERR_BOUNDS); return false; }
        if (!initPacket(pk, nuP, position, zero, false, false, cell[0], cell[1], cell[2], false)) return false;
      }
    }
    if (!(g.flags & MC_FLAG_DUST) && pk.nu < (Real)g.ion_edge1 && !pk.line) {
      escape(pk);
      return false;
    }
    if (!pk.line) return pathSegment(pk, ptype, position, cell);
    ++lc.lines;
    return false;
  }

  __device__ void run(long long p) {
    if (global_ns() - t0 > cnt->budget_ns) { fail(MC_ERR_TIMEOUT); return; }
    int ptype = STELLAR;
    R3<Real> position{(Real)src.pos[0], (Real)src.pos[1], (Real)src.pos[2]};
    int cell[3] = {src.cell[0], src.cell[1], src.cell[2]};
    int i;
    for (i = 1; i <= g.recursion_limit; ++i) {
      const bool rerun = energyPacketRun(ptype, position, cell);
      if (st.exhausted) { fail(MC_ERR_REPLAY); break; }
      if (failed || !rerun) break;
    }
    if (i >= g.recursion_limit) ++lc.trapped;
  }
};

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ void flush_counts(DevCounters *c, LocalCounts &lc) {
  const unsigned long long a0 = warp_sum(lc.crossings), a1 = warp_sum(lc.absorptions),
                           a2 = warp_sum(lc.scatterings), a3 = warp_sum(lc.escaped),
                           a4 = warp_sum(lc.lines), a5 = warp_sum(lc.trapped), a6 = warp_sum(lc.silent),
                           a7 = warp_sum(lc.safe_hits);
  const double q = warp_sum(lc.qphot);
  if ((threadIdx.x & 31) == 0) {
    if (a0) atomicAdd(&c->crossings, a0);
    if (a1) atomicAdd(&c->absorptions, a1);
    if (a2) atomicAdd(&c->scatterings, a2);
    if (a3) atomicAdd(&c->escaped, a3);
    if (a4) atomicAdd(&c->lines, a4);
    if (a5) atomicAdd(&c->trapped, a5);
    if (a6) atomicAdd(&c->silent, a6);
    if (a7) atomicAdd(&c->safe_hits, a7);
    if (q != 0.0) atomicAdd(&c->qphot, q);
  }
}

// Persistent grid-stride kernel over all packets of all sources.
template <typename Real, int Layout = 0>
__global__ void __launch_bounds__(256) transport_plain_kernel(const __grid_constant__ DevGrid g,
                                                             const __grid_constant__ DevSources S,
                                                             const __grid_constant__ DevReplay rp,
                                                             DevCounters *cnt) {
  LocalCounts lc;
  const unsigned long long t0 = global_ns();
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long gp = (long long)blockIdx.x * blockDim.x + threadIdx.x; gp < S.total; gp += stride) {
    if (*(volatile int *)&cnt->error_code != 0) break;
    int s = 0;
    while (s + 1 < S.nsrc + S.nres && gp >= S.s[s + 1].base) ++s;
    const DevSource &src = S.s[s];
    History<Real, Layout> h(g, src, cnt, lc);
    h.gpacket = gp;
    h.t0 = t0;
    h.st.init(src.k0, src.k1, (unsigned long long)(gp - src.base), rp, gp);
    h.run(gp - src.base);
  }
  flush_counts(cnt, lc);
}

}  // namespace mcg
