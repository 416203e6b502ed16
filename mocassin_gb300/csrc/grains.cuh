// grains.cuh -- the grain terms of the cell update in a cell with gas and
// grains (lgPhotoelectric, on by default), for one T step of one cell, on
// one warp:
//   setGrainPotential      source/update_mod.f90:527-604: per size bin, a
//                          secant in the grain potential Vg [Ryd] from 0 on
//                          photoemission - recombination, steps at most 5 %
//                          of the threshold, until the two agree within
//                          0.5 % of their mean or after 100 evaluations;
//   getGrainEmission       :610-663: photoelectrons from the field above
//                          max(Vn + Vg, Vn), yield min(Y0 (1 - Vn/nu), Y1);
//   getGrainRecombination  :669-741: electron minus ion capture currents;
//   setPhotoelHeatCool     :745-806: grain cooling per size, gas heating;
//   setDustGasCollHeatCool :810-930: gas-grain collisions per size, gas
//                          cooling, every stage of every element, then
//                          electrons;
// called at :367-386 between ionBalance and thermBalance, which adds the gas
// heating and cooling (:1251-1254).  getDustT adds gasDustColl_d -
// photoelHeat_d of each size to its absorbed integral (:1886-1889).
//
// The warp's lanes split each sum over frequency (lane l adds the bins
// i = l mod 32 above the threshold, in ascending order, then the xor
// butterfly combines the 32 partial sums), the 33 ion currents of the
// recombination rate (ion pair b in lane b mod 32, same butterfly) and the
// collision terms (lane k: size k, stages in the reference's order).  The
// scalars of the secant are the same in every lane.  Per-bin factors that do
// not depend on Vg come from tables: this cell's photon flux
// Jste / (hcRyd nu) (shared memory), the yield Yn, nu - Vn and Qa = Cabs /
// (1e-8 a^2) per size (global, L1-resident).
#pragma once
#include <cuda_runtime.h>

#include <cmath>

#include "mc_launch.h"

namespace mcg {

namespace {

constexpr int kGrMaxSizes = 32;
constexpr int kGrWin = 64;  // suffix-sum entries kept per size (FP32 form)
constexpr int kGrNE = 7;  // elements H He C N O Ne S

__device__ __forceinline__ int gr_nstage(int z) { return z + 1 < 7 ? z + 1 : 7; }  // min(z + 1, nstages)

template <typename Real> struct GrConst {
  static constexpr double pi = 3.141592654, fourPi = 4. * 3.141592654, hcRyd = 2.1799153e-11;
  static constexpr double amu = 1.66053e-24, me = 9.109382e-28, ryd2erg = 2.1799e-11, kB = 1.380658e-16;
};

__device__ __forceinline__ double gr_aweight(int e) {
  switch (e) {  // H He C N O Ne S (grid_mod.f90:61)
    case 0: return 1.0080;
    case 1: return 4.0026;
    case 2: return 12.0111;
    case 3: return 14.0067;
    case 4: return 15.9994;
    case 5: return 20.179;
    default: return 32.06;
  }
}

template <typename Real> __device__ __forceinline__ Real gr_warp_total(Real p) {
  for (int o = 16; o; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
  return p;
}

// interpolation_mod locate (1-based) on the frequency grid, for an x that
// is the same in every lane: the first bin above x by two ballots (the
// segment of 32 whose last bin is above x, then the bin in it) where the
// grid has at most 1024 bins, by bisection otherwise
template <typename Real> __device__ __forceinline__ int gr_locate(const float *nu, int n, Real x, int lane) {
  if (x > (Real)nu[n - 1]) return n;
  if (x < (Real)nu[0]) return 0;
  int first;
  if (n <= 1024) {
    const int seg = (n + 31) >> 5;
    const int last = lane * seg + seg - 1 < n - 1 ? lane * seg + seg - 1 : n - 1;
    const unsigned m = __ballot_sync(0xffffffffu, lane * seg < n && (Real)nu[last] > x);
    if (!m) {
      first = n;
    } else {
      const int base = (__ffs(m) - 1) * seg;
      const unsigned m2 = __ballot_sync(0xffffffffu, lane < seg && base + lane < n && (Real)nu[base + lane] > x);
      first = base + __ffs(m2) - 1;
    }
  } else {
    int lo = 0, hi = n;
    while (lo < hi) {
      const int m = (lo + hi) >> 1;
      if ((Real)nu[m] > x) hi = m;
      else lo = m + 1;
    }
    first = lo;
  }
  return first == n ? 1 : (first > 1 ? first : 1);
}

template <typename Real> __device__ __forceinline__ const Real *gr_tab(const GrainArgs &g, int which);
template <> __device__ __forceinline__ const double *gr_tab<double>(const GrainArgs &g, int which) {
  return which == 0 ? g.yn_d : (which == 1 ? g.dnu_d : g.qa_d);
}
template <> __device__ __forceinline__ const float *gr_tab<float>(const GrainArgs &g, int which) {
  return which == 0 ? g.yn_f : (which == 1 ? g.dnu_f : g.qa_f);
}

struct GrainOut {
  double heat, cool;  // photoelHeat_g, gasDustColl_g (per H)
  bool converged;     // every size's potential converged
};

// The grain block of one T step of a cell.  bal_z / bal_first: the atomic
// number and first balance ion of each element.  pf: this cell's Jste x scale /
// (hcRyd nu) per bin (shared, the warp's own); X(e, s): ion fractions after
// ionBalance; tdust_k: this cell's grain temperatures of the previous
// iteration.  Lane k < nsizes keeps size k's potential, photoelHeat_d and
// gasDustColl_d in vg_k, pd_k, cd_k.
template <typename Real, class XF>
__device__ GrainOut grain_step(const GrainArgs &g, const int *bal_z, const int *bal_first, const Real *ab, Real Te, Real Ne,
                               Real hden, Real ndust, XF X, const Real *pf, Real tdust_k, int lane, Real &vg_k,
                               Real &pd_k, Real &cd_k) {
  using K = GrConst<Real>;
  const int nb = g.nb, ns = g.nsizes;
  const Real vn = (Real)g.vn;
  const Real *Yn = gr_tab<Real>(g, 0), *dnu = gr_tab<Real>(g, 1), *Qa = gr_tab<Real>(g, 2);
  const Real kT = (Real)6.336e-6 * Te, eightkT_pi = (Real)(1.1045e-15) * Te / (Real)K::pi;
  const Real ve = sqrt(eightkT_pi / (Real)K::me);
  // the ion pairs of the recombination rate: (element, stage 2..top) in the
  // reference's order, pair b in lane b mod 32: cpDen x vmean and the charge
  Real cv0 = (Real)0., z0 = (Real)0., cv1 = (Real)0., z1 = (Real)0.;
  {
    int b = 0;
    for (int e = 0; e < kGrNE; ++e) {
      const int top = gr_nstage(bal_z[e]);
      for (int s = 2; s <= top; ++s, ++b) {
        if ((b & 31) != lane) continue;
        const Real cpDen = X(e, s) * ab[e] * hden;
        const Real vmean = sqrt(eightkT_pi / ((Real)gr_aweight(e) * (Real)K::amu));
        if (b < 32) { cv0 = cpDen * vmean; z0 = (Real)(s - 1); }
        else { cv1 = cpDen * vmean; z1 = (Real)(s - 1); }
      }
    }
  }
  const bool two = lane == 0;  // pair 32 (S, stage 7)
  auto recomb = [&](Real Vg) -> Real {
    Real eta = -Vg / kT;
    eta = eta <= (Real)0. ? (Real)1. - eta : exp(-eta);
    const Real rec = (Real)0. + Ne * ve * (Real)1. * eta;
    Real et = z0 * Vg / kT;
    et = et <= (Real)0. ? (Real)1. - et : exp(-et);
    Real p = (Real)0.;
    p += cv0 * (Real)1. * et;
    if (two) {
      Real e1 = z1 * Vg / kT;
      e1 = e1 <= (Real)0. ? (Real)1. - e1 : exp(-e1);
      p += cv1 * (Real)1. * e1;
    }
    return rec - gr_warp_total<Real>(p);
  };
  // a cell with no photons above the grain threshold: every emission sum
  // from above Vn is a sum of exact zeros
  bool dark;
  {
    const int i0 = gr_locate<Real>(g.nu, nb, vn, lane);
    bool any = false;
    for (int i = i0 + lane; i < nb; i += 32) any |= pf[i] != (Real)0.;
    dark = !__any_sync(0xffffffffu, any);
  }
  const Real nu_top = (Real)g.nu[nb - 1];
  bool top_hit = false;  // locate's quirk at the top bin: the sum starts at bin 1
  auto emission = [&](int k, Real Vg) -> Real {
    const Real thres = fmax(vn + Vg, vn);
    if (dark && thres != nu_top) return (Real)0.;
    if (thres == nu_top) top_hit = true;
    const int ip = gr_locate<Real>(g.nu, nb, thres, lane);  // 0-based start of the loop from ip + 1
    const Real *q = Qa + (size_t)k * nb;
    Real p = (Real)0.;
    for (int i = ip + ((lane - ip) & 31); i < nb; i += 32) {
      const Real Yhat = Yn[i] * fmin((Real)1., fmax((Real)0., (Real)1. - Vg / dnu[i]));
      const Real photFlux = pf[i] * (Real)K::fourPi;
      p += Yhat * photFlux * q[i];
    }
    return gr_warp_total<Real>(p);
  };
  GrainOut o{0., 0., true};
  // setGrainPotential per size; `slope` (a `save` variable of the
  // reference) carries over the sizes of this T step, from 0.  In a dark
  // cell the sizes differ only in the emission, zero for all of them, so
  // each size repeats the secant of size 0 step by step (its first step
  // sets the slope unless that step's change of the currents is exactly 0):
  // size 0's result stands for all.
  Real slope = (Real)0.;
  bool same = dark;
  Real vg0 = (Real)0.;
  for (int k = 0; k < ns; ++k) {
    if (k > 0 && same) {
      if (lane == k) vg_k = vg0;
      continue;
    }
    const Real errorLim = (Real)0.005, dm = (Real)0.05;
    Real Vg = (Real)0., VgOld = (Real)0.;
    Real emiOld = emission(k, (Real)0.), recOld = recomb((Real)0.);
    Vg = VgOld + (Real)0.05;
    bool convk = true;
    for (int n = 1;; ++n) {
      const Real threshold = fmax(vn + Vg, vn);
      const Real emi = emission(k, Vg), rec = recomb(Vg);
      Real delta = emi - rec;
      Real delta1 = fabs(delta / ((Real)0.5 * fmax((Real)1.e-35, emi + rec)));
      if (delta1 < errorLim) break;
      if (Vg != VgOld) {
        const Real fac = (emi - emiOld) - (rec - recOld);
        if (fac != (Real)0.) slope = fac / (Vg - VgOld);
        else if (n == 1) same = false;
      } else if (n == 1) {
        same = false;
      }
      VgOld = Vg;
      recOld = rec;
      emiOld = emi;
      delta1 = -delta / slope;
      delta = fabs(delta1);
      delta = fmin(delta, dm * threshold);
      delta = copysign(delta, delta1);
      Vg = Vg + delta;
      if (n >= 100) { convk = false; break; }
    }
    if (!convk) o.converged = false;
    if (k == 0) {
      vg0 = Vg;
      if (top_hit) same = false;
    }
    if (lane == k) vg_k = Vg;
  }
  // setPhotoelHeatCool
  Real heat = (Real)0.;
  for (int k = 0; k < ns; ++k) {
    const Real Vg = __shfl_sync(0xffffffffu, vg_k, k);
    const Real th = fmax(vn + Vg, vn);
    int thP = gr_locate<Real>(g.nu, nb, th, lane);
    if (thP <= 0) thP = 1;
    const int i0 = thP - 1;
    const float *xs = g.xs + (size_t)k * nb;
    const Real abun = (Real)g.abundance, wk = (Real)g.weight[k];
    Real sd = (Real)0., sg = (Real)0.;
    for (int i = i0 + ((lane - i0) & 31); i < nb; i += 32) {
      const Real Yhat = Yn[i] * fmin((Real)1., fmax((Real)0., (Real)1. - Vg / dnu[i]));
      const Real d = dnu[i];
      const Real EY = Yn[i] * (Real)0.5 * fmin(d, fmax((Real)0., (d * d - Vg * Vg) / d));
      const Real Qf = (Real)xs[i] * pf[i];
      sd += Qf * EY * (Real)K::hcRyd / (Real)K::pi;
      sg += Qf * (EY - Yhat * Vg) * abun * wk;
    }
    sd = gr_warp_total<Real>(sd);
    sg = gr_warp_total<Real>(sg);
    if (lane == k) pd_k = sd;
    heat = heat + sg;
  }
  heat = heat * ndust * (Real)K::hcRyd / hden;
  // setDustGasCollHeatCool: lane k, size k
  Real cg = (Real)0.;
  if (lane < ns) {
    const int k = lane;
    const Real r = (Real)g.radius_um[k], Vg = vg_k, Td = tdust_k;
    const Real abun = (Real)g.abundance, wk = (Real)g.weight[k], msurf = (Real)g.msurf;
    Real cd = (Real)0.;
    Real IPerg = (Real)0.;  // of H0: an unset local in the reference
    for (int e = 0; e < kGrNE; ++e) {
      const int top = gr_nstage(bal_z[e]);
      for (int s = 1; s <= top; ++s) {
        const Real Z = (Real)(s - 1);
        const Real mcp = (Real)gr_aweight(e) * (Real)K::amu;
        const Real vmean = sqrt(eightkT_pi / mcp);
        if (s > 1) IPerg = (Real)g.ion_nu[bal_first[e] + s - 2] * (Real)K::ryd2erg;
        const Real S = s == 1 ? (Real)2. * mcp * msurf / ((mcp + msurf) * (mcp + msurf)) : (Real)1.;
        const Real psi = Z * Vg / kT;
        Real eta, xi;
        if (psi <= (Real)0.) { eta = (Real)1. - psi; xi = (Real)1. - psi / (Real)2.; }
        else { eta = exp(-psi); xi = ((Real)1. + psi / (Real)2.) * eta; }
        const Real x = X(e, s);
        cd = cd + x * ab[e] * hden * (Real)K::pi * r * r * (Real)1.e-8 * S * vmean *
                      ((Real)2. * kT * (Real)K::ryd2erg * xi -
                       eta * (Z * Vg * (Real)K::ryd2erg - IPerg + (Real)2. * (Real)K::kB * Td));
        cg = cg + x * wk * abun * ndust * ab[e] * (Real)K::pi * r * r * (Real)1.e-8 * S * vmean *
                      ((Real)2. * kT * (Real)K::ryd2erg * xi - eta * (Real)2. * (Real)K::kB * Td);
      }
    }
    {
      const Real S = (Real)1., Z = (Real)-1.;
      const Real psi = Z * Vg / kT;
      Real eta, xi;
      if (psi <= (Real)0.) { eta = (Real)1. - psi; xi = (Real)1. - psi / (Real)2.; }
      else { eta = exp(-psi); xi = ((Real)1. + psi / (Real)2.) * eta; }
      cd = cd + Ne * (Real)K::pi * r * r * (Real)1.e-8 * S * ve *
                    ((Real)2. * kT * (Real)K::ryd2erg * xi - eta * (Z * Vg * (Real)K::ryd2erg));
      cg = cg + Ne * wk * abun * ndust * (Real)K::pi * r * r * (Real)1.e-8 * S * ve *
                    ((Real)2. * kT * (Real)K::ryd2erg * xi) / hden;
    }
    cd_k = cd / (Real)K::fourPi;
  }
  Real cool = (Real)0.;
  for (int k = 0; k < ns; ++k) cool = cool + __shfl_sync(0xffffffffu, cg, k);
  cool = cool / (Real)K::fourPi;
  o.heat = (double)heat;
  o.cool = (double)cool;
  return o;
}

// The FP32 form of the grain block (wave_grain_kernel): the same secant,
// sums and collision terms in 4-byte floats, regrouped so that each secant
// step costs a few operations instead of a sum over bins and ions:
//   potentials     the sizes' secants side by side, lane k for size k
//                  (each with its own `slope`);
//   photoemission  from suffix sums over the bins above Vn, built once per
//                  T step in shared memory (sfx, nsizes x 2 x kGrWin floats:
//                  the first kGrWin bins above Vn) of t(i) = Yn pf 4 pi Qa
//                  and t(i) / (nu - Vn):
//                  above max(Vn + Vg, Vn) the yield factor is 1 - Vg / (nu -
//                  Vn) (Vg > 0) or 1, so the sum is SF - Vg SG or SF;
//   recombination  the ion currents grouped by charge Z = 1..6 once per T
//                  step (C_Z = sum of cpDen vmean over the stages of charge
//                  Z), so that Ne ve eta_e - sum_Z C_Z eta_Z needs one exp:
//                  eta_Z = exp(-Vg/kT)^Z above 0 and 1 - Z Vg/kT below;
//   collisions     eta and xi of each charge once per size;
//   divisions by kT and by nu - Vn as products with reciprocals, exp as
//                  __expf.
// Results follow the FP64 form within the rounding of 4-byte floats.
template <class XF>
__device__ GrainOut grain_step_fast(const GrainArgs &g, const int *bal_z, const int *bal_first, const float *ab,
                                    float Te, float Ne, float hden, float ndust, XF X, const float *pf, float *sfx,
                                    float tdust_k, int lane, float &vg_k, float &pd_k, float &cd_k) {
  using K = GrConst<float>;
  const int nb = g.nb, ns = g.nsizes, ivn = g.ivn, nsf = nb - ivn + 1;
  const float vn = (float)g.vn;
  const float *Yn = g.yn_f, *idnu = g.idnu_f, *dnu = g.dnu_f, *Qa = g.qa_f;
  const float kT = 6.336e-6f * Te, ikT = 1.f / kT;
  const float ekp = 1.1045e-15f * Te / (float)K::pi, sq = sqrtf(ekp);
  const float ve = sq * 3.313260193e13f;  // sqrt(ekp / me)
  auto rsqm = [](int e) -> float {        // 1 / sqrt(aWeight amu) of H He C N O Ne S
    switch (e) {
      case 0: return 7.729410466e11f;
      case 1: return 3.878872830e11f;
      case 2: return 2.239160609e11f;
      case 3: return 2.073522362e11f;
      case 4: return 1.940103007e11f;
      case 5: return 1.727534848e11f;
      default: return 1.370549981e11f;
    }
  };
  // ion currents per unit eta, by charge
  float C[7] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  for (int e = 0; e < kGrNE; ++e) {
    const int top = gr_nstage(bal_z[e]);
    const float vm = sq * rsqm(e);
    for (int s = 2; s <= top; ++s) C[s - 1] += X(e, s) * ab[e] * hden * vm;
  }
  const float S0 = C[1] + C[2] + C[3] + C[4] + C[5] + C[6];
  const float S1 = C[1] + 2.f * C[2] + 3.f * C[3] + 4.f * C[4] + 5.f * C[5] + 6.f * C[6];
  const float NeVe = Ne * ve;
  auto recomb = [&](float Vg) -> float {
    const float x = Vg * ikT;
    if (x >= 0.f) {
      const float t = __expf(-x);
      const float ions = t * (C[1] + t * (C[2] + t * (C[3] + t * (C[4] + t * (C[5] + t * C[6])))));
      return NeVe * (1.f + x) - ions;
    }
    return NeVe * __expf(x) - (S0 - x * S1);
  };
  // dark cell: no photons above the grain threshold
  bool dark;
  {
    bool any = false;
    for (int i = ivn + lane; i < nb; i += 32) any |= pf[i] != 0.f;
    dark = !__any_sync(0xffffffffu, any);
  }
  // suffix sums of every size from the first kGrWin bins above Vn (the
  // thresholds a potential below ~3 Ryd reaches on a 600-bin grid):
  // sfx [ns][2][kGrWin], chunks of 32 bins from the top
  if (!dark)
    for (int k = 0; k < ns; ++k) {
      const float *q = Qa + (size_t)k * nb;
      float *sf = sfx + (size_t)k * 2 * kGrWin, *sg = sf + kGrWin;
      float cf = 0.f, cgs = 0.f;
      const int nchunk = (nsf - 1 + 31) >> 5;
      for (int ch = nchunk - 1; ch >= 0; --ch) {
        const int i = ivn + ch * 32 + lane;
        float tf = 0.f, tg = 0.f;
        if (i < nb) {
          tf = Yn[i] * pf[i] * (float)K::fourPi * q[i];
          tg = tf * idnu[i];
        }
        for (int o = 1; o < 32; o <<= 1) {
          const float xf = __shfl_down_sync(0xffffffffu, tf, o), xg = __shfl_down_sync(0xffffffffu, tg, o);
          if (lane + o < 32) { tf += xf; tg += xg; }
        }
        tf += cf;
        tg += cgs;
        if (i < nb && i - ivn < kGrWin) { sf[i - ivn] = tf; sg[i - ivn] = tg; }
        cf = __shfl_sync(0xffffffffu, tf, 0);
        cgs = __shfl_sync(0xffffffffu, tg, 0);
      }
    }
  __syncwarp();
  // the photoemission of this lane's size (lane < ns)
  const float nu_top = g.nu[nb - 1];
  auto emission = [&](int k, float Vg) -> float {
    if (dark) return 0.f;
    const float thres = fmaxf(vn + Vg, vn);
    int ip;  // locate (1-based) = the 0-based first bin above thres
    if (thres > nu_top) {
      ip = nb;
    } else if (thres < g.nu[0]) {
      ip = 0;
    } else {
      int lo = 0, hi = nb;
      while (lo < hi) {
        const int m = (lo + hi) >> 1;
        if (g.nu[m] > thres) hi = m;
        else lo = m + 1;
      }
      ip = lo == nb ? 1 : (lo > 1 ? lo : 1);
    }
    const float *q = Qa + (size_t)k * nb;
    if (ip >= nb) return 0.f;
    if (ip >= ivn && ip - ivn < kGrWin) {
      const float *sf = sfx + (size_t)k * 2 * kGrWin;
      const int j = ip - ivn;
      return Vg > 0.f ? sf[j] - Vg * sf[kGrWin + j] : sf[j];
    }
    // a threshold above the window, or locate's quirk at the top bin: the
    // literal sum from bin ip
    float p = 0.f;
    for (int i = ip; i < nb; ++i) p += Yn[i] * fminf(1.f, fmaxf(0.f, 1.f - Vg / dnu[i])) * pf[i] * (float)K::fourPi * q[i];
    return p;
  };
  // setGrainPotential: every size's secant at once, lane k for size k (each
  // lane keeps its own `slope`, from 0); a dark cell's sizes share one
  GrainOut o{0., 0., true};
  {
    const int k = dark ? 0 : lane;
    const bool mine = dark ? true : lane < ns;
    float Vg = 0.f, VgOld = 0.f, slope = 0.f;
    float emiOld = 0.f, recOld = 0.f;
    bool run = mine, conv = true;
    if (mine) {
      emiOld = emission(k, 0.f);
      recOld = recomb(0.f);
      Vg = 0.05f;
    }
    for (int n = 1; __any_sync(0xffffffffu, run); ++n) {
      if (!run) continue;
      const float threshold = fmaxf(vn + Vg, vn);
      const float emi = emission(k, Vg), rec = recomb(Vg);
      float delta = emi - rec;
      float delta1 = fabsf(delta / (0.5f * fmaxf(1.e-35f, emi + rec)));
      if (delta1 < 0.005f) { run = false; continue; }
      if (Vg != VgOld) {
        const float fac = (emi - emiOld) - (rec - recOld);
        if (fac != 0.f) slope = fac / (Vg - VgOld);
      }
      VgOld = Vg;
      recOld = rec;
      emiOld = emi;
      delta1 = -delta / slope;
      delta = fminf(fabsf(delta1), 0.05f * threshold);
      Vg = Vg + copysignf(delta, delta1);
      if (n >= 100) { run = false; conv = false; }
    }
    if (!__all_sync(0xffffffffu, conv || !mine)) o.converged = false;
    vg_k = Vg;
  }
  // setPhotoelHeatCool
  float heat = 0.f;
  for (int k = 0; k < ns; ++k) {
    const float Vg = __shfl_sync(0xffffffffu, vg_k, k);
    int thP = gr_locate<float>(g.nu, nb, fmaxf(vn + Vg, vn), lane);
    if (thP <= 0) thP = 1;
    const int i0 = thP - 1;
    const float *xs = g.xs + (size_t)k * nb;
    float sd = 0.f, sg = 0.f;
    if (!dark || i0 < ivn)
      for (int i = i0 + ((lane - i0) & 31); i < nb; i += 32) {
        const float d = dnu[i], id = idnu[i];
        const float Yhat = Yn[i] * fminf(1.f, fmaxf(0.f, 1.f - Vg * id));
        const float EY = Yn[i] * 0.5f * fminf(d, fmaxf(0.f, (d * d - Vg * Vg) * id));
        const float Qf = xs[i] * pf[i];
        sd += Qf * EY;
        sg += Qf * (EY - Yhat * Vg);
      }
    sd = gr_warp_total<float>(sd) * (float)(K::hcRyd / K::pi);
    sg = gr_warp_total<float>(sg) * (float)g.abundance * (float)g.weight[k];
    if (lane == k) pd_k = sd;
    heat += sg;
  }
  heat = heat * ndust * (float)K::hcRyd / hden;
  // setDustGasCollHeatCool: lane k, size k; eta and xi of each charge once
  float cg = 0.f;
  if (lane < ns) {
    const int k = lane;
    const float r = (float)g.radius_um[k], Vg = vg_k, Td = tdust_k, msurf = (float)g.msurf;
    const float geo = (float)K::pi * r * r * 1.e-8f;
    const float wk = (float)g.weight[k] * (float)g.abundance * ndust;
    const float x = Vg * ikT;
    float eta[7], xi[7];
    const float t = x > 0.f ? __expf(-x) : 1.f;
    float tz = 1.f;
    for (int Z = 0; Z < 7; ++Z) {
      const float psi = (float)Z * x;
      if (psi <= 0.f) { eta[Z] = 1.f - psi; xi[Z] = 1.f - 0.5f * psi; }
      else { eta[Z] = tz; xi[Z] = (1.f + 0.5f * psi) * tz; }
      tz *= t;
    }
    const float twokT = 2.f * kT * (float)K::ryd2erg, twokTd = 2.f * (float)K::kB * Td;
    float cd = 0.f, cgk = 0.f, IPerg = 0.f;  // IPerg of H0: an unset local in the reference
    for (int e = 0; e < kGrNE; ++e) {
      const int top = gr_nstage(bal_z[e]);
      const float mcp = (float)(gr_aweight(e) * 1.66053e-24);
      const float vm = sq * rsqm(e);
      for (int s = 1; s <= top; ++s) {
        const int Z = s - 1;
        if (s > 1) IPerg = (float)g.ion_nu[bal_first[e] + s - 2] * (float)K::ryd2erg;
        const float S = s == 1 ? 2.f * mcp * msurf / ((mcp + msurf) * (mcp + msurf)) : 1.f;
        const float n = X(e, s) * ab[e] * S * vm;
        cd += n * hden * (twokT * xi[Z] - eta[Z] * ((float)Z * Vg * (float)K::ryd2erg - IPerg + twokTd));
        cgk += n * (twokT * xi[Z] - eta[Z] * twokTd);
      }
    }
    // electrons (charge -1)
    float eta_e, xi_e;
    if (x >= 0.f) { eta_e = 1.f + x; xi_e = 1.f + 0.5f * x; }
    else { eta_e = __expf(x); xi_e = (1.f - 0.5f * x) * eta_e; }
    cd += Ne * ve * (twokT * xi_e - eta_e * (-Vg * (float)K::ryd2erg));
    cgk = cgk * wk + Ne * wk * ve * twokT * xi_e / hden;
    cd_k = cd * geo / (float)K::fourPi;
    cg = cgk * geo;
  }
  float cool = 0.f;
  for (int k = 0; k < ns; ++k) cool += __shfl_sync(0xffffffffu, cg, k);
  o.heat = (double)heat;
  o.cool = (double)(cool / (float)K::fourPi);
  return o;
}

}  // namespace

}  // namespace mcg
