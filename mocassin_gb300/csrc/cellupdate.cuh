// cellupdate.cuh -- the per-cell gas update kernel, templated on the
// arithmetic type; instantiated in cellupdate.cu (FP64, -fmad=false) and
// cellupdate_fp32.cu (FP32).
//
// One warp per cell (grid-stride over cells), following
//   iterateT      source/update_mod.f90:339-525: bracketed secant in Te,
//                 at most 25 steps, the 0.2 % bracket collapse after step 6;
//   calcAlpha     :1624-1654, radRecFit :1674-1780, dielectronic :1782-1834;
//   ionBalance    :1320-1622: photoionisation + collisional ionisation of
//                 H0 + charge exchange with H, ratios X(i+1)/X(i), up to 25
//                 passes until X(H0), X(He0), X(He+) move < 1 %;
//   thermBalance  :933-1258: H and He free-free and recombination cooling
//                 fits, H collisional excitation, forbidden-line cooling of
//                 every ion with data (equilibrium, emission_mod.f90:1913-2115,
//                 levels 1..10 summed), photo-heating from the Jste sums.
// The warp's lanes share the work that has width: lane b computes the
// recombination coefficient and the ionisation ratio of balance ion b (33
// ions: b and b + 32), lane k solves the level populations of line ion k
// (natural-spline collision strengths, the reference's Gaussian elimination
// without pivoting, in local memory).  Sums that the reference forms in one
// order (Ne, the cooling and heating totals) are formed by lane 0 in that
// order, so the FP64 instantiation (compiled with -fmad=false) follows the
// FP64 oracle operation by operation.  In a cell with grains the warp also
// runs the grain block of each T step (grains.cuh) between ionBalance and
// thermBalance, on the cell's Jste row staged once in shared memory.  Per
// cell and T step the work is
// ~1e4-1e5 operations, most of them in the level populations: the FP64 form
// is bound by GB300's FP64 rate, the FP32 form by issue and local memory.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "grains.cuh"
#include "mc_launch.h"

namespace mcg {

namespace {

constexpr int kW = 4;        // warps per block
constexpr int kNE = 7, kNS = 7, kNX = 8, kNB = 33, kNL = 18, kNT = 32;

template <typename Real> __device__ __forceinline__ const UpdTabs<Real> &tabs(const UpdArgs &a);
template <> __device__ __forceinline__ const UpdTabs<double> &tabs<double>(const UpdArgs &a) { return a.d; }
template <> __device__ __forceinline__ const UpdTabs<float> &tabs<float>(const UpdArgs &a) { return a.f; }

__device__ __forceinline__ int nion_of(int z) { return z < kNS - 1 ? z : kNS - 1; }
__device__ __forceinline__ int nstage_of(int z) { return z + 1 < kNS ? z + 1 : kNS; }

// dielectronic coefficient diRec(z, ion) of one element/stage at Te
// (dielectronic :1782-1834): the last matching row of dielectronic.dat whose
// temperature range applies (rows listed on the host in file order),
// replaced by the last matching Aldrovandi & Pequignot row above 60000 K or
// where it is zero
// (the last matching row is the one whose value stands, so the rows are
// scanned from the end and the first match ends the scan)
template <typename Real>
__device__ Real direc_of(const UpdArgs &a, const int *rows, int nrows, int arow, Real Te) {
  const UpdTabs<Real> &T = tabs<Real>(a);
  const Real t = Te / (Real)10000.;
  Real d = 0., al = 0.;
  for (int k = nrows - 1; k >= 0; --k) {
    const Real *r = T.direc + 8 * rows[k];
    const int g = (int)r[7];
    if (g == 0 || (g == 1 && Te < (Real)20000.) || (g == 2 && Te >= (Real)20000.)) {
      d = (Real)1e-12 * ((Real)r[2] / t + (Real)r[3] + (Real)r[4] * t + (Real)r[5] * t * t) * pow(t, (Real)-1.5) *
          exp(-(Real)r[6] / t);
      break;
    }
  }
  if (arow >= 0) {
    const Real *r = T.aldro + 6 * arow;
    al = (Real)r[2] * pow(Te, (Real)-1.5) * exp(-(Real)r[4] / Te) * ((Real)1. + (Real)r[3] * exp(-(Real)r[5] / Te));
  }
  if (Te > (Real)60000. || d == (Real)0.) d = al;
  return d;
}

template <typename Real>
__device__ Real alpha_of(const UpdArgs &a, const UpdIonT<Real> &b, Real Te) {
  const UpdTabs<Real> &T = tabs<Real>(a);
  const int z = b.z, n = b.nelec;
  Real v;
  if (n <= 3 || n == 11 || (z > 5 && z < 9) || z == 10 || (z == 26 && n > 11)) {
    const Real *rn = T.rnew;
    auto RN = [&](int i) { return (Real)rn[(i * 31 + z) * 31 + n]; };
    const Real tt = sqrt(Te / RN(2));
    v = RN(0) / (tt * pow(tt + (Real)1.0, (Real)1.0 - RN(1)) * pow((Real)1.0 + sqrt(Te / RN(3)), (Real)1.0 + RN(1)));
  } else {
    const Real tt = Te * (Real)1.e-4;
    v = T.rrec[(0 * 31 + z) * 31 + n] / pow(tt, T.rrec[(1 * 31 + z) * 31 + n]);
  }
  if (z >= 3) {
    Real d = direc_of<Real>(a, b.dr, b.ndr, b.ar, Te);
    if (d == (Real)0.) d = direc_of<Real>(a, b.dr8, b.ndr8, b.ar8, Te);
    v += d;
  }
  return v;
}

// forbidden-line cooling of line ion k per ion (equilibrium), levels 1..10
template <typename Real>
__device__ Real cel_cooling(const UpdArgs &a, int k, Real Te, Real Ne, Real up) {
  const UpdTabs<Real> &T = tabs<Real>(a);
  if (up != up) return (Real)0.;
  const UpdCelT<Real> &c = T.cel[k];
  const int n = c.nlev, nt = c.nt;
  const Real *logt = T.logt + (size_t)k * kNT;
  const Real *g = T.g + (size_t)k * kNL, *e = T.e + (size_t)k * kNL;
  const Real *A = T.A + (size_t)k * kNL * kNL;
  const Real *qq = T.qq + (size_t)k * kNL * kNL * kNT, *q2 = T.q2 + (size_t)k * kNL * kNL * kNT;
  const Real sqrTe = sqrt(Te), log10Te = log10(Te);
  Real alphaTotal[kNL];
  for (int j = 0; j < kNL; ++j) alphaTotal[j] = (Real)0.;
  for (int j = 2; j <= n; ++j) {
    if (c.br <= (Real)0.) break;
    alphaTotal[1] = (Real)1.;
    const Real br = (Real)c.br, zz = (Real)c.zz;
    const Real tz = Te * (Real)1.e-4 / (zz * zz), t4 = Te * (Real)1.e-4;
    alphaTotal[j] = (Real)1.e-13 * br * zz * (Real)c.ar[0] * pow(tz, (Real)c.ar[1]) /
                        ((Real)1. + (Real)c.ar[2] * pow(tz, (Real)c.ar[3])) +
                    (Real)1.0e-12 * br *
                        ((Real)c.ad[0] / t4 + (Real)c.ad[1] + (Real)c.ad[2] * t4 + (Real)c.ad[3] * t4 * t4) *
                        pow(t4, (Real)-1.5) * exp(-(Real)c.ad[4] * (Real)1.e4 / Te);
  }
  // the spline interval is the same for every transition of the ion
  int klo = 0, khi = nt - 1;
  const bool below = log10Te <= (Real)logt[0], above = log10Te >= (Real)logt[nt - 1];
  if (nt > 2 && !below && !above) {
    while (khi - klo > 1) {
      const int m = (khi + klo) / 2;
      if ((Real)logt[m] > log10Te) khi = m;
      else klo = m;
    }
  }
  // qeff(i, j) of every pair: excitation lo -> hi and de-excitation hi -> lo
  Real qeff[kNL][kNL];
  for (int lo = 1; lo < n; ++lo)
    for (int hi = lo + 1; hi <= n; ++hi) {
      const Real *y = qq + ((size_t)lo * kNL + hi) * kNT;
      Real cs;
      if (nt == 1) cs = (Real)y[0];
      else if (nt == 2)
        cs = (Real)y[0] + ((Real)y[1] - (Real)y[0]) / ((Real)logt[1] - (Real)logt[0]) * (log10Te - (Real)logt[0]);
      else if (below) cs = (Real)y[0];
      else if (above) cs = (Real)y[nt - 1];
      else {
        const Real *y2 = q2 + ((size_t)lo * kNL + hi) * kNT;
        const Real h = (Real)logt[khi] - (Real)logt[klo];
        const Real aa = ((Real)logt[khi] - log10Te) / h, bb = (log10Te - (Real)logt[klo]) / h;
        cs = aa * (Real)y[klo] + bb * (Real)y[khi] +
             ((aa * aa * aa - aa) * (Real)y2[klo] + (bb * bb * bb - bb) * (Real)y2[khi]) * (h * h) / (Real)6.;
      }
      const Real delTeK = ((Real)e[lo] - (Real)e[hi]) * (Real)1.4388463;
      qeff[lo][hi] = (Real)8.63e-6 * cs * exp(delTeK / Te) / ((Real)g[lo] * sqrTe);
      qeff[hi][lo] = (Real)8.63e-6 * cs / ((Real)g[hi] * sqrTe);
    }
  Real x[kNL][kNL], y[kNL];
  for (int i = 1; i <= n; ++i) {
    y[i] = (Real)0.;
    for (int j = 1; j <= n; ++j) x[i][j] = (Real)0.;
  }
  for (int j = 1; j <= n; ++j) x[1][j] = (Real)1.;
  y[1] = (Real)1.;
  for (int i = 2; i <= n; ++i) {
    for (int j = 1; j <= n; ++j) {
      if (j == i) continue;
      x[i][j] += Ne * qeff[j][i];
      x[i][i] -= Ne * qeff[i][j];
      if (j > i) x[i][j] += (Real)A[j * kNL + i];
      else x[i][i] -= (Real)A[i * kNL + j];
    }
    y[i] = -Ne * up * alphaTotal[i];
  }
  if (n > 1) {
    for (int i = 1; i <= n - 1; ++i)
      for (int kk = i + 1; kk <= n; ++kk) {
        const Real f = x[kk][i] / x[i][i];
        for (int j = i + 1; j <= n; ++j) x[kk][j] = x[kk][j] - x[i][j] * f;
      }
    for (int i = 1; i <= n - 1; ++i)
      for (int j = i + 1; j <= n; ++j) y[j] = y[j] - y[i] * x[j][i] / x[i][i];
    y[n] = y[n] / x[n][n];
    for (int i = 1; i <= n - 1; ++i) {
      const int kk = n - i;
      for (int j = kk + 1; j <= n; ++j) y[kk] = y[kk] - y[j] * x[kk][j];
      y[kk] = y[kk] / x[kk][kk];
    }
  } else {
    y[n] = y[n] / x[n][n];
  }
  Real sumN = (Real)0.;
  for (int i = 1; i <= n; ++i) sumN += y[i];
  Real cool = (Real)0.;
  const int top = n < 10 ? n : 10;
  for (int i = 1; i <= top - 1; ++i)
    for (int j = i + 1; j <= top; ++j)
      if (A[j * kNL + i] != (Real)0.) cool += (Real)A[j * kNL + i] * ((Real)e[j] - (Real)e[i]) * (y[j] / sumN);
  return cool;
}

// The same level populations with the matrix of lane k in shared memory
// (M, row-major with row length L, per-lane stride odd so the lanes' accesses
// fall in distinct banks), built pair by pair: each transition adds its
// collision and radiative rates to the rows of both of its levels.  The sums
// on the diagonal are formed in another order than the reference's row loop.
// top_levels = 10 gives thermBalance's cooling (transitions among levels
// 1..10).  With fscale > 0 each line is scaled by fscale and only lines above
// 1e-35 count: setDiffusePDF's normFor over forbiddenLines (all levels,
// emission_mod.f90:1151-1172).  With emis non-null the same populations also
// give that emission sum (over all levels, scaled by escale) in *emis.
template <typename Real>
__device__ Real cel_cooling_smem(const UpdArgs &a, int k, Real Te, Real Ne, Real up, Real *M, int L,
                                 int top_levels = 10, Real fscale = (Real)0., Real *emis = nullptr,
                                 Real escale = (Real)0.) {
  const UpdTabs<Real> &T = tabs<Real>(a);
  if (emis) *emis = (Real)0.;
  if (up != up) return (Real)0.;
  const UpdCelT<Real> &c = T.cel[k];
  const int n = c.nlev, nt = c.nt;
  const Real *logt = T.logt + (size_t)k * kNT;
  const Real *g = T.g + (size_t)k * kNL, *e = T.e + (size_t)k * kNL;
  const Real *A = T.A + (size_t)k * kNL * kNL;
  const Real *qq = T.qq + (size_t)k * kNL * kNL * kNT, *q2 = T.q2 + (size_t)k * kNL * kNL * kNT;
  const Real sqrTe = sqrt(Te), log10Te = log10(Te);
  auto X = [&](int i, int j) -> Real & { return M[(i - 1) * L + (j - 1)]; };
  Real y[kNL];
  Real alpha_j = (Real)0.;
  const bool rec = c.br > (Real)0.;
  Real arec = (Real)0.;
  if (rec) {
    const Real br = (Real)c.br, zz = (Real)c.zz;
    const Real tz = Te * (Real)1.e-4 / (zz * zz), t4 = Te * (Real)1.e-4;
    arec = (Real)1.e-13 * br * zz * (Real)c.ar[0] * pow(tz, (Real)c.ar[1]) /
               ((Real)1. + (Real)c.ar[2] * pow(tz, (Real)c.ar[3])) +
           (Real)1.0e-12 * br * ((Real)c.ad[0] / t4 + (Real)c.ad[1] + (Real)c.ad[2] * t4 + (Real)c.ad[3] * t4 * t4) *
               pow(t4, (Real)-1.5) * exp(-(Real)c.ad[4] * (Real)1.e4 / Te);
  }
  (void)alpha_j;
  for (int j = 1; j <= n; ++j) X(1, j) = (Real)1.;
  y[1] = (Real)1.;
  for (int i = 2; i <= n; ++i) {
    for (int j = 1; j <= n; ++j) X(i, j) = (Real)0.;
    y[i] = rec ? -Ne * up * arec : (Real)0.;
  }
  int klo = 0, khi = nt - 1;
  const bool below = log10Te <= (Real)logt[0], above = log10Te >= (Real)logt[nt - 1];
  if (nt > 2 && !below && !above) {
    while (khi - klo > 1) {
      const int m = (khi + klo) / 2;
      if ((Real)logt[m] > log10Te) khi = m;
      else klo = m;
    }
  }
  const Real h = (Real)logt[khi] - (Real)logt[klo];
  const Real aa = nt > 2 ? ((Real)logt[khi] - log10Te) / h : (Real)0.;
  const Real bb = nt > 2 ? (log10Te - (Real)logt[klo]) / h : (Real)0.;
  const Real ca = aa * aa * aa - aa, cb = bb * bb * bb - bb, h26 = h * h / (Real)6.;
  for (int lo = 1; lo < n; ++lo)
    for (int hi = lo + 1; hi <= n; ++hi) {
      const Real *yy = qq + ((size_t)lo * kNL + hi) * kNT;
      Real cs;
      if (nt == 1) cs = (Real)yy[0];
      else if (nt == 2)
        cs = (Real)yy[0] + ((Real)yy[1] - (Real)yy[0]) / ((Real)logt[1] - (Real)logt[0]) * (log10Te - (Real)logt[0]);
      else if (below) cs = (Real)yy[0];
      else if (above) cs = (Real)yy[nt - 1];
      else {
        const Real *y2 = q2 + ((size_t)lo * kNL + hi) * kNT;
        cs = aa * (Real)yy[klo] + bb * (Real)yy[khi] + (ca * (Real)y2[klo] + cb * (Real)y2[khi]) * h26;
      }
      const Real qex = (Real)8.63e-6 * cs * exp(((Real)e[lo] - (Real)e[hi]) * (Real)1.4388463 / Te) / ((Real)g[lo] * sqrTe);
      const Real qde = (Real)8.63e-6 * cs / ((Real)g[hi] * sqrTe);
      const Real Ahl = (Real)A[hi * kNL + lo];
      X(hi, lo) += Ne * qex;
      X(hi, hi) -= Ne * qde + Ahl;
      if (lo >= 2) {
        X(lo, hi) += Ne * qde + Ahl;
        X(lo, lo) -= Ne * qex;
      }
    }
  for (int i = 1; i <= n - 1; ++i) {
    const Real inv = (Real)1. / X(i, i);
    for (int kk = i + 1; kk <= n; ++kk) {
      const Real f = X(kk, i) * inv;
      for (int j = i + 1; j <= n; ++j) X(kk, j) = X(kk, j) - X(i, j) * f;
      y[kk] = y[kk] - y[i] * f;
    }
  }
  y[n] = y[n] / X(n, n);
  for (int kk = n - 1; kk >= 1; --kk) {
    for (int j = kk + 1; j <= n; ++j) y[kk] = y[kk] - y[j] * X(kk, j);
    y[kk] = y[kk] / X(kk, kk);
  }
  Real sumN = (Real)0.;
  for (int i = 1; i <= n; ++i) sumN += y[i];
  Real cool = (Real)0.;
  const int top = n < top_levels ? n : top_levels;
  const Real inv = (Real)1. / sumN;
  for (int i = 1; i <= top - 1; ++i)
    for (int j = i + 1; j <= top; ++j)
      if (A[j * kNL + i] != (Real)0.) {
        const Real line = (Real)A[j * kNL + i] * ((Real)e[j] - (Real)e[i]) * (y[j] * inv);
        if (!(fscale > (Real)0.)) cool += line;
        else if (line * fscale > (Real)1e-35) cool += line * fscale;
      }
  if (emis) {
    Real em = (Real)0.;
    for (int i = 1; i <= n - 1; ++i)
      for (int j = i + 1; j <= n; ++j)
        if (A[j * kNL + i] != (Real)0.) {
          const Real line = (Real)A[j * kNL + i] * ((Real)e[j] - (Real)e[i]) * (y[j] * inv) * escale;
          if (line > (Real)1e-35) em += line;
        }
    *emis = em;
  }
  return cool;
}

// The tables of one line ion as cel_cooling_reg reads them: straight from
// the device tables (CelTabGlobal), or from a warp's staged copy in shared
// memory (CelTabStaged: the N (N - 1) / 2 transitions' collision-strength
// rows, kNT apart, and A values packed by transition index).  Both give the
// same values.
struct CelTabGlobal {
  const float *logt_, *g_, *e_, *A, *qq, *q2;
  __device__ __forceinline__ CelTabGlobal(const UpdTabs<float> &T, int k)
      : logt_(T.logt + (size_t)k * kNT), g_(T.g + (size_t)k * kNL), e_(T.e + (size_t)k * kNL),
        A(T.A + (size_t)k * kNL * kNL), qq(T.qq + (size_t)k * kNL * kNL * kNT), q2(T.q2 + (size_t)k * kNL * kNL * kNT) {}
  __device__ __forceinline__ const float *logt() const { return logt_; }
  __device__ __forceinline__ const float *g() const { return g_; }
  __device__ __forceinline__ const float *e() const { return e_; }
  template <int N> __device__ __forceinline__ float a(int lo, int hi) const { return A[hi * kNL + lo]; }
  template <int N> __device__ __forceinline__ const float *y(int lo, int hi) const {
    return qq + ((size_t)lo * kNL + hi) * kNT;
  }
  template <int N> __device__ __forceinline__ const float *y2(int lo, int hi) const {
    return q2 + ((size_t)lo * kNL + hi) * kNT;
  }
};

// index of transition (lo, hi), 1 <= lo < hi <= N, in lo-major order
__host__ __device__ constexpr int cel_pair(int lo, int hi, int N) { return (lo - 1) * (2 * N - lo) / 2 + (hi - lo - 1); }

constexpr int kCelMaxPairs = 15 * 14 / 2;  // the register form's largest ion
// floats of one warp's staged tables: logt, g, e, A by transition, two rows
// of kNT collision strengths per transition
constexpr int kCelStage = kNT + 2 * kNL + kCelMaxPairs + 2 * kCelMaxPairs * kNT;

// one base pointer: every table sits at a fixed offset from it
struct CelTabStaged {
  const float *s;
  static constexpr int kG = kNT, kE = kNT + kNL, kA = kNT + 2 * kNL, kQ = kA + kCelMaxPairs,
                       kQ2 = kQ + kCelMaxPairs * kNT;
  __device__ __forceinline__ explicit CelTabStaged(const float *s_) : s(s_) {}
  __device__ __forceinline__ const float *logt() const { return s; }
  __device__ __forceinline__ const float *g() const { return s + kG; }
  __device__ __forceinline__ const float *e() const { return s + kE; }
  template <int N> __device__ __forceinline__ float a(int lo, int hi) const { return s[kA + cel_pair(lo, hi, N)]; }
  template <int N> __device__ __forceinline__ const float *y(int lo, int hi) const {
    return s + kQ + cel_pair(lo, hi, N) * kNT;
  }
  template <int N> __device__ __forceinline__ const float *y2(int lo, int hi) const {
    return s + kQ2 + cel_pair(lo, hi, N) * kNT;
  }
};

// the warp copies line ion k's tables (N levels, nt temperatures) into s
__device__ __forceinline__ void cel_stage(const UpdTabs<float> &T, int k, int N, int nt, float *s, int lane) {
  const CelTabGlobal G(T, k);
  float *logt = s, *g = s + CelTabStaged::kG, *e = s + CelTabStaged::kE, *A = s + CelTabStaged::kA;
  float *qq = s + CelTabStaged::kQ, *q2 = s + CelTabStaged::kQ2;
  if (lane < nt) logt[lane] = G.logt()[lane];
  if (lane <= N) { g[lane] = G.g()[lane]; e[lane] = G.e()[lane]; }
  int p = 0;
  for (int lo = 1; lo < N; ++lo)
    for (int hi = lo + 1; hi <= N; ++hi, ++p) {
      if (lane == 0) A[p] = G.A[hi * kNL + lo];
      if (lane < nt) {
        const size_t row = ((size_t)lo * kNL + hi) * kNT + lane;
        qq[p * kNT + lane] = G.qq[row];
        q2[p * kNT + lane] = G.q2[row];
      }
    }
}

// cel_cooling_smem in FP32 for an ion of N levels known at compile time:
// every loop unrolled, so the rate matrix, the right-hand side and the
// populations are registers (no per-thread matrix in local memory) and the
// table reads take constant offsets.  The same solve as cel_cooling_smem,
// with the rate factors 8.63e-6 / (g sqrt Te) and 1.4388463 / Te formed
// once per level (a few FP32 roundings apart from dividing per transition).
template <int N, typename Tab>
__device__ __forceinline__ float cel_cooling_reg(const UpdArgs &a, int k, const Tab &tb, float Te, float Ne, float up,
                                                 int top_levels, float fscale, float *emis, float escale) {
  const UpdTabs<float> &T = a.f;
  if (emis) *emis = 0.f;
  if (up != up) return 0.f;
  const UpdCelT<float> &c = T.cel[k];
  const int nt = c.nt;
  const float *logt = tb.logt(), *g = tb.g(), *e = tb.e();
  const float sqrTe = sqrtf(Te), log10Te = log10f(Te);
  float X[N][N], y[N];  // X[i][j] is row i + 1, column j + 1 of the 1-based system
  float arec = 0.f;
  const bool rec = c.br > 0.f;
  if (rec) {
    const float br = c.br, zz = c.zz;
    const float tz = Te * 1.e-4f / (zz * zz), t4 = Te * 1.e-4f;
    arec = 1.e-13f * br * zz * c.ar[0] * powf(tz, c.ar[1]) / (1.f + c.ar[2] * powf(tz, c.ar[3])) +
           1.0e-12f * br * (c.ad[0] / t4 + c.ad[1] + c.ad[2] * t4 + c.ad[3] * t4 * t4) * powf(t4, -1.5f) *
               expf(-c.ad[4] * 1.e4f / Te);
  }
#pragma unroll
  for (int j = 0; j < N; ++j) X[0][j] = 1.f;
  y[0] = 1.f;
#pragma unroll
  for (int i = 1; i < N; ++i) {
#pragma unroll
    for (int j = 0; j < N; ++j) X[i][j] = 0.f;
    y[i] = rec ? -Ne * up * arec : 0.f;
  }
  int klo = 0, khi = nt - 1;
  const bool below = log10Te <= logt[0], above = log10Te >= logt[nt - 1];
  if (nt > 2 && !below && !above) {
    while (khi - klo > 1) {
      const int m = (khi + klo) / 2;
      if (logt[m] > log10Te) khi = m;
      else klo = m;
    }
  }
  const float h = logt[khi] - logt[klo];
  const float aa = nt > 2 ? (logt[khi] - log10Te) / h : 0.f;
  const float bb = nt > 2 ? (log10Te - logt[klo]) / h : 0.f;
  const float ca = aa * aa * aa - aa, cb = bb * bb * bb - bb, h26 = h * h / 6.f;
  // the per-level factors of the rates, one division per level instead of
  // two per transition: 8.63e-6 / (g sqrt(Te)), and hc/k / Te
  const float ic = 1.4388463f / Te;
  const float i2 = nt == 2 ? (log10Te - logt[0]) / (logt[1] - logt[0]) : 0.f;
  float ig[N + 1];
#pragma unroll
  for (int l = 1; l <= N; ++l) ig[l] = 8.63e-6f / (g[l] * sqrTe);
#pragma unroll
  for (int lo = 1; lo < N; ++lo)
#pragma unroll
    for (int hi = lo + 1; hi <= N; ++hi) {
      const float *yy = tb.template y<N>(lo, hi);
      float cs;
      if (nt == 1) cs = yy[0];
      else if (nt == 2) cs = yy[0] + (yy[1] - yy[0]) * i2;
      else if (below) cs = yy[0];
      else if (above) cs = yy[nt - 1];
      else {
        const float *y2 = tb.template y2<N>(lo, hi);
        cs = aa * yy[klo] + bb * yy[khi] + (ca * y2[klo] + cb * y2[khi]) * h26;
      }
      const float qex = cs * expf((e[lo] - e[hi]) * ic) * ig[lo];
      const float qde = cs * ig[hi];
      const float Ahl = tb.template a<N>(lo, hi);
      X[hi - 1][lo - 1] += Ne * qex;
      X[hi - 1][hi - 1] -= Ne * qde + Ahl;
      if (lo >= 2) {
        X[lo - 1][hi - 1] += Ne * qde + Ahl;
        X[lo - 1][lo - 1] -= Ne * qex;
      }
    }
#pragma unroll
  for (int i = 0; i < N - 1; ++i) {
    const float inv = 1.f / X[i][i];
#pragma unroll
    for (int kk = i + 1; kk < N; ++kk) {
      const float f = X[kk][i] * inv;
#pragma unroll
      for (int j = i + 1; j < N; ++j) X[kk][j] = X[kk][j] - X[i][j] * f;
      y[kk] = y[kk] - y[i] * f;
    }
  }
  y[N - 1] = y[N - 1] / X[N - 1][N - 1];
#pragma unroll
  for (int kk = N - 2; kk >= 0; --kk) {
#pragma unroll
    for (int j = kk + 1; j < N; ++j) y[kk] = y[kk] - y[j] * X[kk][j];
    y[kk] = y[kk] / X[kk][kk];
  }
  float sumN = 0.f;
#pragma unroll
  for (int i = 0; i < N; ++i) sumN += y[i];
  float cool = 0.f;
  const int top = N < top_levels ? N : top_levels;
  const float inv = 1.f / sumN;
#pragma unroll
  for (int i = 1; i <= N - 1; ++i)
#pragma unroll
    for (int j = i + 1; j <= N; ++j) {
      const float Aji = tb.template a<N>(i, j);
      if (j <= top && Aji != 0.f) {
        const float line = Aji * (e[j] - e[i]) * (y[j - 1] * inv);
        if (!(fscale > 0.f)) cool += line;
        else if (line * fscale > 1e-35f) cool += line * fscale;
      }
    }
  if (emis) {
    float em = 0.f;
#pragma unroll
    for (int i = 1; i <= N - 1; ++i)
#pragma unroll
      for (int j = i + 1; j <= N; ++j) {
        const float Aji = tb.template a<N>(i, j);
        if (Aji != 0.f) {
          const float line = Aji * (e[j] - e[i]) * (y[j - 1] * inv) * escale;
          if (line > 1e-35f) em += line;
        }
      }
    *emis = em;
  }
  return cool;
}

// whether line ion k has a register form (the level counts the line ions of
// the atomic data have: 2, 3, 5, 6, 7, 9, 10, 12, 13, 15)
__device__ __forceinline__ bool cel_has_reg(int n) {
  return n == 2 || n == 3 || n == 5 || n == 6 || n == 7 || n == 9 || n == 10 || n == 12 || n == 13 || n == 15;
}

// the FP32 level populations of line ion k with the tables tb: the register
// form for its level count, cel_cooling_smem on the device tables and the
// scratch matrix M (L rows) otherwise
template <typename Tab>
__device__ __forceinline__ float cel_cooling_f32(const UpdArgs &a, int k, const Tab &tb, float Te, float Ne, float up,
                                                 float *M, int L, int top_levels, float fscale, float *emis = nullptr,
                                                 float escale = 0.f) {
  switch (a.f.cel[k].nlev) {
#define MC_CEL_CASE(n) \
  case n: return cel_cooling_reg<n>(a, k, tb, Te, Ne, up, top_levels, fscale, emis, escale);
    MC_CEL_CASE(2) MC_CEL_CASE(3) MC_CEL_CASE(5) MC_CEL_CASE(6) MC_CEL_CASE(7) MC_CEL_CASE(9) MC_CEL_CASE(10)
    MC_CEL_CASE(12) MC_CEL_CASE(13) MC_CEL_CASE(15)
#undef MC_CEL_CASE
    default: return cel_cooling_smem<float>(a, k, Te, Ne, up, M, L, top_levels, fscale, emis, escale);
  }
}

template <typename Real, bool Fast>
__global__ void __launch_bounds__(kW * 32) cell_update_kernel(const __grid_constant__ UpdArgs a) {
  extern __shared__ __align__(16) unsigned char cu_dyn[];
  __shared__ Real sX[kW][kNE][kNX];
  __shared__ Real sAl[kW][kNB + 1], sR[kW][kNB + 1], sCel[kW][32];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nw = gridDim.x * kW;
  const Real kB = (Real)1.380658e-16, hcRyd = (Real)2.1799153e-11, xMax = (Real)0.99999;
  const UpdTabs<Real> &T = tabs<Real>(a);
  for (int c = 1 + blockIdx.x * kW + w; c <= a.nc; c += nw) {
    const bool hit = a.mom[c] > 0.f;
    if (!hit) {
      if (lane == 0) { a.conv[c] = 0; a.niter[c] = 0; a.flags[c] = 0; a.dte[c] = -1.; }
      continue;
    }
    // grains: this cell's photon flux Jste x scale / (hcRyd nu) per bin
    const int ngr = a.g.nsizes;
    const size_t gnc1 = (size_t)a.nc + 1;
    Real *pf = (Real *)(cu_dyn + (Fast ? (size_t)kW * a.ncel * a.mat_stride * sizeof(Real) : 0)) + (size_t)w * a.g.nb;
    Real gvg = (Real)0., gpd = (Real)0., gcd = (Real)0., gtd = (Real)0., gheat = (Real)0., gcool = (Real)0.;
    bool gconv = true;
    if (ngr > 0) {
      for (int i = lane; i < a.g.nb; i += 32)
        pf[i] = (Real)((a.g.jste[(size_t)i * gnc1 + c] * a.g.jscale) / (2.1799153e-11 * (double)a.g.nu[i]));
      if (lane < ngr && a.g.tdust) gtd = (Real)a.g.tdust[(size_t)(1 + lane) * gnc1 + c];
    }
    double *Xc = a.X + (size_t)c * kNE * kNX;
    for (int i = lane; i < kNE * kNX; i += 32) sX[w][i / kNX][i % kNX] = (Real)Xc[i];
    const Real hden = (Real)a.hden[c];
    Real Te = (Real)a.te[c], Ne = (Real)a.ne[c];
    const Real Te0 = a.te_prev ? (Real)a.te_prev[c] : Te;
    Real P[2] = {(Real)0., (Real)0.}, Hh[2] = {(Real)0., (Real)0.};
    for (int r = 0; r < 2; ++r) {
      const int b = lane + 32 * r;
      if (b < kNB) {
        P[r] = (Real)a.mom[(size_t)(1 + b) * a.mstride + c] + (Real)1e-20;
        Hh[r] = (Real)a.mom[(size_t)(1 + kNB + b) * a.mstride + c];
      }
    }
    __syncwarp();
    const Real XOldHI = a.x_prev ? (Real)a.x_prev[(size_t)c * kNE * kNX + 1] : sX[w][0][1];
    int nIterT = 0, noTe = 0;
    bool ionConv = true, warm = a.x_prev != nullptr, grow = a.step_grow != 0, cold = false;
    Real thResHigh = 0., thResLow = 0., Thigh = 0., Tlow = 0.;
    Real fstep = (Real)a.step0;
    for (;;) {
      ++nIterT;
      for (int r = 0; r < 2; ++r) {
        const int b = lane + 32 * r;
        if (b < kNB) sAl[w][b] = alpha_of<Real>(a, T.bal[b], Te);
      }
      __syncwarp();
      // ionBalance
      int nIterX = 1;
      for (;;) {
        ionConv = true;
        Real expFact = (Real)157893.94 / Te;
        if (expFact > (Real)75.) expFact = (Real)75.;
        const Real collIon0 =
            (Real)2.75E-16 * Te * sqrt(Te) * ((Real)157893.94 / Te + (Real)2.) * exp(-expFact);
        const Real HIOld = sX[w][0][1], HeIOld = sX[w][1][1], HeIIOld = sX[w][1][2];
        const Real t4 = Te / (Real)10000.;
        for (int r = 0; r < 2; ++r) {
          const int b = lane + 32 * r;
          if (b >= kNB) continue;
          const UpdIonT<Real> &B = T.bal[b];
          Real ch = (Real)B.chex[0] * pow(t4, (Real)B.chex[1]) * ((Real)1. + (Real)B.chex[2] * exp((Real)B.chex[3] * t4));
          if (ch < (Real)0.) ch = (Real)0.;
          if (Te < (Real)6000. || Te > (Real)5.e4) ch = (Real)0.;
          Real revRate = (Real)0.;
          if (B.dek > (Real)1.)
            revRate = ch * ((Real)1. - HIOld) * hden * (Real)2. * exp(-(Real)B.dek / Te) / (Real)B.g0g1;
          const Real collIon = b == 0 ? collIon0 : (Real)0.;
          sR[w][b] = (P[r] + collIon + revRate) / (Ne * sAl[w][b] + ch * hden * HIOld);
        }
        __syncwarp();
        if (lane < kNE) {
          const int e = lane, z = a.bal_z[e], b0 = a.bal_first[e], ni = nion_of(z), ns = nstage_of(z);
          Real prod[kNS + 1];
          Real den = (Real)1.;
          for (int ion = 1; ion <= ni; ++ion) {
            Real p = (Real)1.;
            for (int i = 1; i <= ion; ++i) p *= sR[w][b0 + i - 1];
            prod[ion] = p;
          }
          for (int ion = 1; ion <= ni; ++ion) den += prod[ion];
          for (int ion = 1; ion <= ns; ++ion) {
            Real v = ion == 1 ? (Real)1.0 / den : prod[ion - 1] / den;
            if (v > xMax) v = xMax;
            if (v < (Real)1.e-20) v = (Real)1.e-20;
            sX[w][e][ion] = v;
          }
        }
        __syncwarp();
        Real ne = (Real)0.;
        if (lane == 0) {
          for (int e = 0; e < kNE; ++e) {
            const int ns = nstage_of(a.bal_z[e]);
            for (int ion = 2; ion <= ns; ++ion)
              if (sX[w][e][ion] >= (Real)1.e-10) ne += (Real)(ion - 1) * T.ab[e] * sX[w][e][ion];
          }
        }
        ne = __shfl_sync(0xffffffffu, ne, 0);
        Ne = ne * hden;
        if (Ne == (Real)0.) Ne = (Real)1.;
        const Real dHI = (sX[w][0][1] - HIOld) / HIOld, dHeI = (sX[w][1][1] - HeIOld) / HeIOld,
                   dHeII = (sX[w][1][2] - HeIIOld) / HeIIOld;
        const bool off = fabs(dHI) > (Real)0.01 || fabs(dHeI) > (Real)0.01 || fabs(dHeII) > (Real)0.01;
        if (off && nIterX < 25) { ++nIterX; continue; }
        if (off && nIterX == 25) ionConv = false;
        break;
      }
      if (ngr > 0) {
        __syncwarp();
        auto Xf = [&](int e, int s) -> Real { return sX[w][e][s]; };
        const GrainOut go = grain_step<Real>(a.g, a.bal_z, a.bal_first, T.ab, Te, Ne, hden, (Real)a.g.ndust[c], Xf, pf,
                                             gtd, lane, gvg, gpd, gcd);
        gheat = (Real)go.heat;
        gcool = (Real)go.cool;
        gconv = go.converged;
      }
      // thermBalance
      if (lane < a.ncel) {
        const UpdCelT<Real> &C = T.cel[lane];
        const Real up = C.ion < kNS ? sX[w][C.e][C.ion + 1] / sX[w][C.e][C.ion] : (Real)0.;
        if (Fast) {
          Real *M = (Real *)cu_dyn + ((size_t)w * a.ncel + lane) * a.mat_stride;
          sCel[w][lane] = cel_cooling_smem<Real>(a, lane, Te, Ne, up, M, a.mat_rows);
        } else {
          sCel[w][lane] = cel_cooling<Real>(a, lane, Te, Ne, up);
        }
      }
      __syncwarp();
      Real heatInt = 0., coolInt = 0.;
      if (lane == 0) {
        const Real log10Te = log10(Te), Te4 = Te / (Real)1.e4;
        auto poly4 = [](Real x, Real c0, Real c1, Real c2, Real c3, Real c4) {
          return c0 + c1 * x + c2 * x * x + c3 * x * x * x + c4 * x * x * x * x;
        };
        auto bff = [&](Real x) {
          return poly4(x, (Real)1.0108464E-11, (Real)9.7930778E-13, (Real)-6.6433144E-13, (Real)2.4793747E-13,
                       (Real)-2.3938215E-14);
        };
        auto brec = [&](Real x) {
          return poly4(x, (Real)9.4255985E-11, (Real)-4.04794384E-12, (Real)-1.0055237E-11, (Real)1.99266862E-12,
                       (Real)-1.06681387E-13);
        };
        Real Np = sX[w][0][2] * T.ab[0];
        Real coolFF = Np * Ne * bff(log10Te) * kB * Te / sqrt(Te);
        Real coolRec = Np * Ne * brec(log10Te) * kB * Te / sqrt(Te);
        Np = sX[w][1][3] * T.ab[1];
        const Real lts = log10(Te / (Real)4.);
        coolFF += Np * Ne * ((Real)2. * bff(lts)) * kB * Te / sqrt(Te / (Real)4.);
        coolRec += Np * Ne * ((Real)2. * brec(lts)) * kB * Te / sqrt(Te / (Real)4.);
        Np = sX[w][1][2] * T.ab[1];
        coolFF += Np * Ne *
                  ((Real)1.070073e-11 - (Real)2.5730207e-13 * log10Te + (Real)2.109134e-13 * log10Te * log10Te) * kB *
                  Te / sqrt(Te);
        coolRec += Np * Ne * brec(log10Te) * kB * Te / sqrt(Te);
        Real coolColl = (Real)0.;
        if (Te > (Real)5000.)
          coolColl = ((Real)2.47e-8 * exp((Real)-118338. / Te) * pow(Te4, (Real)-0.228) +
                      (Real)1.32e-8 * exp((Real)-140252. / Te) * pow(Te4, (Real)-0.460)) *
                     hcRyd * sX[w][0][1] * Ne;
        for (int k = 0; k < a.ncel; ++k) {
          const UpdCelT<Real> &C = T.cel[k];
          coolColl += sCel[w][k] * T.ab[C.e] * sX[w][C.e][C.ion] * (Real)1.9865e-16;
        }
        coolInt = coolFF + coolRec + coolColl;
        if (ngr > 0) coolInt = coolInt + gcool;
      }
      // heating: the sums live in the lanes' registers; gathered in order
      {
        Real hs = (Real)0.;
        for (int b = 0; b < kNB; ++b) {
          const int src = b & 31, r = b >> 5;
          const Real hb = __shfl_sync(0xffffffffu, r ? Hh[1] : Hh[0], src);
          if (lane == 0) {
            const UpdIonT<Real> &B = T.bal[b];
            hs += hb * sX[w][B.e][B.ion] * T.ab[B.e];
          }
        }
        if (lane == 0) heatInt = ngr > 0 ? hs + gheat : hs;
      }
      heatInt = __shfl_sync(0xffffffffu, heatInt, 0);
      coolInt = __shfl_sync(0xffffffffu, coolInt, 0);
      const Real thResidual = heatInt - coolInt;
      bool again = false;
      const bool first_warm = warm;
      if (warm) {
        warm = false;
        // a prediction far from balance: the cold solve from the state
        // before the prediction, with the full T-step allowance
        if (fabs(thResidual) >= (Real)a.near_res * heatInt) {
          const double *Xp = a.x_prev + (size_t)c * kNE * kNX;
          for (int i = lane; i < kNE * kNX; i += 32) sX[w][i / kNX][i % kNX] = (Real)Xp[i];
          Te = (Real)a.te_prev[c];
          Ne = (Real)a.ne_prev[c];
          fstep = (Real)1.2;
          grow = false;
          cold = true;
          nIterT = 0;
          __syncwarp();
          continue;
        }
      }
      if (fabs(thResidual) >= (first_warm ? (Real)a.accept_res : (Real)0.01) * heatInt) {
        if (nIterT < 25) {
          bool open = false;
          if (thResidual < (Real)0) {
            thResLow = thResidual;
            Tlow = Te;
            if (Thigh != (Real)0.) Te = Tlow - (Thigh - Tlow) * thResLow / (thResHigh - thResLow);
            else { Te = Te / fstep; open = true; }
          } else {
            thResHigh = thResidual;
            Thigh = Te;
            if (Tlow != (Real)0.) Te = Tlow - (Thigh - Tlow) * thResLow / (thResHigh - thResLow);
            else { Te = Te * fstep; open = true; }
          }
          if (open && grow) fstep = fstep - (Real)1. < (Real)0.1 ? (Real)1. + (Real)2. * (fstep - (Real)1.) : (Real)1.2;
          if (nIterT >= 6 && fabs(Thigh - Tlow) <= (Real)0.002 * (Thigh + Tlow)) {
            if (thResidual < (Real)0) { Te = Thigh - (Real)100.; Thigh = (Real)0.; }
            else { Te = Tlow + (Real)100.; Tlow = (Real)0.; }
          }
          if (Te <= (Real)0.) Te = (Real)1.;
          again = true;
        } else {
          if (Thigh == (Real)0.) Te = Tlow;
          else if (Tlow == (Real)0.) Te = Thigh;
          else Te = (Thigh + Tlow) * (Real)0.5;
          noTe = 1;
        }
      }
      __syncwarp();
      if (!again) break;
    }
    for (int i = lane; i < kNE * kNX; i += 32) Xc[i] = (double)sX[w][i / kNX][i % kNX];
    if (lane == 0) {
      a.te[c] = (double)Te;
      a.ne[c] = (double)Ne;
      if (a.forb_ok) a.forb_ok[c] = 0;  // this form keeps no line totals
      a.conv[c] = fabs((sX[w][0][1] - XOldHI) / XOldHI) <= (Real)a.xhi ? 1 : 0;
      a.niter[c] = nIterT;
      a.flags[c] = (noTe ? 1 : 0) | (ionConv ? 0 : 2) | (cold ? 4 : 0) | (gconv ? 0 : 8);
      a.dte[c] = fabs((double)Te - (double)Te0) / (double)Te0;
    }
    if (ngr > 0 && lane < ngr) {
      a.g.out[(size_t)lane * gnc1 + c] = (double)gvg;
      a.g.out[(size_t)(ngr + lane) * gnc1 + c] = (double)gpd;
      a.g.out[(size_t)(2 * ngr + lane) * gnc1 + c] = (double)gcd;
    }
    __syncwarp();
  }
}

}  // namespace

}  // namespace mcg
