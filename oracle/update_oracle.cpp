// update_oracle.cpp -- TEST INFRASTRUCTURE ONLY: CPU restatement (FP64) of
// mocassin's per-cell gas update, used to check the GPU cell-update kernel.
// Nothing in the product links or calls this file.
//
// Follows, for a cell with the debug field off (nPhotoDif unused):
//   updateCell     source/update_mod.f90:15-335 (lgHit, state set-up)
//   iterateT       source/update_mod.f90:339-525 (bracketed secant in Te)
//   ionBalance     source/update_mod.f90:1320-1622 (photo + collisional
//                  ionisation, charge exchange, recombination; up to 25
//                  passes until X(H0), X(He0), X(He+) change < 1 %)
//   calcAlpha      source/update_mod.f90:1624-1654
//   radRecFit      source/update_mod.f90:1674-1780
//   dielectronic   source/update_mod.f90:1782-1834 (`direc` in the `where`
//                  is diRec: Fortran names are case-insensitive)
//   thermBalance   source/update_mod.f90:933-1258 (H/He free-free and
//                  recombination fits, H collisional excitation, forbidden
//                  lines over levels 1..10, photo-heating)
//   forLines       source/update_mod.f90:1263-1318
//   equilibrium    source/emission_mod.f90:1913-2115 (level populations)
//   luSlv          source/emission_mod.f90:2119-2190 (no pivoting)
//   spline/splint  source/interpolation_mod.f90:182-311 (natural spline)
//   getOuterShell  source/hydro_mod.f90:89-182 (statistical weights)
// and, in a cell with gas and grains (lgPhotoelectric, the default):
//   setGrainPotential / getGrainEmission / getGrainRecombination
//                  source/update_mod.f90:527-741 (grain charge balance)
//   setPhotoelHeatCool      :745-806 (photoelectric gas heating, grain cooling)
//   setDustGasCollHeatCool  :810-930 (gas-grain collisions)
//   called per T step at :367-386 and added in thermBalance :1251-1254
// for the elements H, He, C, N, O, Ne, S (nstages = 7).  The reference
// computes in 4-byte `real` with a few double-precision arrays; this is the
// FP64 restatement.  Photoionisation sums nPhotoSte (without the 1e-20
// floor added here) and the heating sums per unit ion density are inputs:
// they are moments of Jste over frequency.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int kNE = 7;       // elements H He C N O Ne S
constexpr int kNS = 7;       // nstages
constexpr int kLev = 18;     // nForLevels + 1 (1-based)
constexpr int kNT = 32;
const int kZ[kNE] = {1, 2, 6, 7, 8, 10, 16};

}  // namespace

extern "C" {

struct upd_tables_t {
  const double *rrec;   // [2][31][31]
  const double *rnew;   // [4][31][31]
  const double *direc;  // [ndirec][8]: elem n a b c d f g
  int32_t ndirec;
  const double *aldro;  // [naldro][6]: elem n a b t0 t1
  int32_t naldro;
  int32_t ncel;
  const int32_t *cel_key;    // [ncel][2] (Z, ion)
  const int32_t *cel_nlev;
  const int32_t *cel_ntemp;
  const double *cel_logt;    // [ncel][32]
  const double *cel_qom;     // [ncel][32][18][18]
  const double *cel_a;       // [ncel][18][18], a[j][i] = A(j -> i)
  const double *cel_g;       // [ncel][18]
  const double *cel_e;       // [ncel][18] 1/cm
  const double *cel_br, *cel_z;
  const double *cel_ar;      // [ncel][4]
  const double *cel_ad;      // [ncel][5]
};

// The grains of a dusty gas cell (one species in nsizes size bins), for the
// photoelectric and gas-grain collision terms of the update.
struct upd_grains_t {
  int32_t nsizes, nbins;
  const double *nu;         // [nbins] frequency grid [Ryd]
  const double *xs_abs;     // [nsizes][nbins] absorption cross-section per grain [cm^2]
  const double *radius_um;  // [nsizes] grainRadius [um]
  const double *weight;     // [nsizes] grainWeight
  double abundance;         // grainAbun of the species
  double vn;                // grainVn [Ryd]
  double msurf;             // MsurfAtom
  const double *ion_nu;     // [33] threshold energy of each balance ion [Ryd]
};

}  // extern "C"

namespace {

struct Cell {
  const upd_tables_t *t;
  const double *ab;   // number abundance per element
  double hden;
  const double *photo;  // [33] nPhotoSte - 1e-20
  const double *heat;   // [33] sum xs J (nu - nuIP) / nu
  double Te, Ne;
  double X[kNE][kNS + 1];  // ionDen(elem, 1..7)
  double alphaTot[kNE][kNS + 1];
  int nIterT = 0, nIterX = 0;
  double thResHigh = 0, thResLow = 0, Thigh = 0, Tlow = 0;
  bool ionConv = true;
  int noTeBal = 0, noIonBal = 0;
  // grains (null: a gas-only cell): this cell's Jste x scale [nbins], grains
  // per cm^3, the grain temperatures of the previous iteration [nsizes]
  const upd_grains_t *g = nullptr;
  const double *J = nullptr;
  double ndust = 0.;
  const double *tdust = nullptr;
  double photoG = 0., collG = 0.;       // photoelHeat_g, gasDustColl_g
  double vg[32], photoD[32], collD[32];  // grainPot, photoelHeat_d, gasDustColl_d
  bool gcConv = true;                   // every grain potential converged (last T step)

  static int nion(int e) { return std::min(kZ[e], kNS - 1); }  // ion 1..min(elem, nstages-1)
  static int nstage(int e) { return std::min(kZ[e] + 1, kNS); }
  // index of (e, ion) in the 33 balance ions
  static int bidx(int e, int ion) {
    int k = 0;
    for (int i = 0; i < e; ++i) k += nion(i);
    return k + ion - 1;
  }

  double radRecFit(int z, int n) const {
    auto RN = [&](int i) { return t->rnew[(i * 31 + z) * 31 + n]; };
    auto RR = [&](int i) { return t->rrec[(i * 31 + z) * 31 + n]; };
    if (n <= 3 || n == 11 || (z > 5 && z < 9) || z == 10 || (z == 26 && n > 11)) {
      const double tt = std::sqrt(Te / RN(2));
      return RN(0) / (tt * std::pow(tt + 1.0, 1.0 - RN(1)) * std::pow(1.0 + std::sqrt(Te / RN(3)), 1.0 + RN(1)));
    }
    const double tt = Te * 1.e-4;
    return RR(0) / std::pow(tt, RR(1));
  }

  void calcAlpha() {
    double diRec[31][kNS + 1], aldro[31][kNS + 1];
    std::memset(diRec, 0, sizeof diRec);
    std::memset(aldro, 0, sizeof aldro);
    for (int e = 0; e < kNE; ++e)
      for (int ion = 1; ion <= nion(e); ++ion) alphaTot[e][ion] = radRecFit(kZ[e], kZ[e] - ion + 1);
    const double t4 = Te / 10000.;
    for (int i = 0; i < t->ndirec; ++i) {
      const double *r = t->direc + 8 * i;
      const int el = (int)r[0], n = (int)r[1], g = (int)r[7];
      const int ion = el + 1 - n;
      if (ion > kNS || el > 30 || ion < 1) continue;
      const double v =
          1e-12 * (r[2] / t4 + r[3] + r[4] * t4 + r[5] * t4 * t4) * std::pow(t4, -1.5) * std::exp(-r[6] / t4);
      if (g == 0 || (g == 1 && Te < 20000.) || (g == 2 && Te >= 20000.)) diRec[el][ion] = v;
    }
    for (int i = 0; i < t->naldro; ++i) {
      const double *r = t->aldro + 6 * i;
      const int el = (int)r[0], n = (int)r[1];
      const int ion = el + 1 - n;
      const double a = r[2] * std::pow(Te, -1.5) * std::exp(-r[4] / Te) * (1. + r[3] * std::exp(-r[5] / Te));
      if (ion <= kNS && ion >= 1 && el <= 30) aldro[el][ion] = a;
    }
    for (int el = 0; el <= 30; ++el)
      for (int ion = 1; ion <= kNS; ++ion)
        if (Te > 60000. || diRec[el][ion] == 0.) diRec[el][ion] = aldro[el][ion];
    for (int e = 2; e < kNE; ++e)
      for (int ion = 1; ion <= nion(e); ++ion) {
        double d = diRec[kZ[e]][ion];
        if (d == 0.) d = diRec[8][ion];
        alphaTot[e][ion] += d;
      }
  }

  // charge-exchange fit coefficients chex(elem, ion, 1:4) (ionBalance :1400-1460)
  static void chexCoeff(int z, int ion, double c[4]) {
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

  // statistical weights g0 / g1 of getOuterShell for z <= 20
  static double g0g1(int nElec) {
    static const int gl[30] = {2, 1, 2, 1, 6, 9, 4, 9, 6, 1, 2, 1, 6, 9, 4, 9, 6, 1, 2, 1,
                               10, 21, 28, 7, 6, 25, 28, 21, 2, 1};
    const int g0 = gl[nElec - 1];
    const int g1 = nElec == 1 ? 1 : gl[nElec - 2];
    return (double)g0 / (double)g1;
  }

  // one pass of ionBalance; returns after the recursion (iteration) ends
  void ionBalance() {
    const double xMax = 0.99999;  // constants_mod.f90:58
    for (;;) {
      ionConv = true;
      double expFact = 157893.94 / Te;
      if (expFact > 75.) expFact = 75.;
      double collIon = 2.75E-16 * Te * std::sqrt(Te) * (157893.94 / Te + 2.) * std::exp(-expFact);
      const double HIOld = X[0][1], HeIOld = X[1][1], HeIIOld = X[1][2];
      const double t4 = Te / 10000.;
      double ionRatio[kNE][kNS + 1] = {}, ionProd[kNE][kNS + 1];
      for (int e = 0; e < kNE; ++e)
        for (int s = 0; s <= kNS; ++s) ionProd[e][s] = 1.;
      for (int e = 0; e < kNE; ++e) {
        for (int ion = 1; ion <= nion(e); ++ion) {
          double c[4];
          chexCoeff(kZ[e], ion, c);
          double ch = c[0] * std::pow(t4, c[1]) * (1. + c[2] * std::exp(c[3] * t4));
          if (ch < 0.) ch = 0.;
          if (Te < 6000. || Te > 5.e4) ch = 0.;
          const int nElec = kZ[e] - ion + 1;
          double dEk = 0.;
          if (kZ[e] == 7 && ion == 1) dEk = 10863.;
          if (kZ[e] == 8 && ion == 1) dEk = 2205.;
          double revRate = 0.;
          if (dEk > 1.) revRate = ch * (1. - X[0][1]) * hden * 2. * std::exp(-dEk / Te) / g0g1(nElec);
          if (kZ[e] > 1 || ion > 1) collIon = 0.;
          const double P = photo[bidx(e, ion)] + 1e-20;
          ionRatio[e][ion] = (P + collIon + revRate) / (Ne * alphaTot[e][ion] + ch * hden * X[0][1]);
        }
      }
      double denom[kNE];
      for (int e = 0; e < kNE; ++e) {
        for (int ion = 1; ion <= nion(e); ++ion)
          for (int i = 1; i <= ion; ++i) ionProd[e][ion] *= ionRatio[e][i];
        denom[e] = 1.;
        for (int ion = 1; ion <= nion(e); ++ion) denom[e] += ionProd[e][ion];
      }
      for (int e = 0; e < kNE; ++e)
        for (int ion = 1; ion <= nstage(e); ++ion) {
          double v = ion == 1 ? 1.0 / denom[e] : ionProd[e][ion - 1] / denom[e];
          if (v > xMax) v = xMax;
          if (v < 1.e-20) v = 1.e-20;
          X[e][ion] = v;
        }
      double ne = 0.;
      for (int e = 0; e < kNE; ++e)
        for (int ion = 2; ion <= nstage(e); ++ion)
          if (X[e][ion] >= 1.e-10) ne += (ion - 1) * ab[e] * X[e][ion];
      Ne = ne * hden;
      if (Ne == 0.) Ne = 1.;
      const double dHI = (X[0][1] - HIOld) / HIOld, dHeI = (X[1][1] - HeIOld) / HeIOld,
                   dHeII = (X[1][2] - HeIIOld) / HeIIOld;
      const bool off = std::fabs(dHI) > 0.01 || std::fabs(dHeI) > 0.01 || std::fabs(dHeII) > 0.01;
      if (off && nIterX < 25) { ++nIterX; continue; }
      if (off && nIterX == 25) ionConv = false;
      return;
    }
  }

  // forbidden-line emissivities of one ion (equilibrium), summed over the
  // transitions among levels 1..10 that thermBalance adds up [erg/s per ion]
  // Forbidden-line cooling of line ion k: sum over the transitions among
  // levels 1..top of A(j,i) (E_j - E_i) n_j (thermBalance, top = 10).  With
  // fscale > 0 every line is scaled by fscale and only lines above 1e-35
  // count (setDiffusePDF's normFor over forbiddenLines, top = all levels).
  double celCooling(int k, double ionDenUp, int top_levels = 10, double fscale = 0.) const {
    if (ionDenUp != ionDenUp) return 0.;
    const int n = t->cel_nlev[k], nt = t->cel_ntemp[k];
    const double *logt = t->cel_logt + (size_t)k * kNT;
    auto QOM = [&](int it, int i, int j) { return t->cel_qom[(((size_t)k * kNT + it) * kLev + i) * kLev + j]; };
    auto A = [&](int j, int i) { return t->cel_a[((size_t)k * kLev + j) * kLev + i]; };
    const double *g = t->cel_g + (size_t)k * kLev, *e = t->cel_e + (size_t)k * kLev;
    const double br = t->cel_br[k], z = t->cel_z[k];
    const double *a_r = t->cel_ar + 4 * k, *a_d = t->cel_ad + 5 * k;
    const double sqrTe = std::sqrt(Te), log10Te = std::log10(Te);
    double alphaTotal[kLev] = {};
    for (int j = 2; j <= n; ++j) {
      if (br <= 0.) break;
      alphaTotal[1] = 1.;
      const double tz = Te * 1.e-4 / (z * z), t4 = Te * 1.e-4;
      alphaTotal[j] = 1.e-13 * br * z * a_r[0] * std::pow(tz, a_r[1]) / (1. + a_r[2] * std::pow(tz, a_r[3])) +
                      1.0e-12 * br * (a_d[0] / t4 + a_d[1] + a_d[2] * t4 + a_d[3] * t4 * t4) * std::pow(t4, -1.5) *
                          std::exp(-a_d[4] * 1.e4 / Te);
    }
    double qeff[kLev][kLev] = {};
    for (int i = 2; i <= n; ++i)
      for (int j = i; j <= n; ++j) {
        double qq[kNT], qomInt;
        for (int it = 0; it < nt; ++it) qq[it] = QOM(it, i - 1, j);
        if (nt == 1) {
          qomInt = qq[0];
        } else if (nt == 2) {
          qomInt = qq[0] + (qq[1] - qq[0]) / (logt[1] - logt[0]) * (log10Te - logt[0]);
        } else {
          // natural cubic spline (spline with yp1 = ypn = 1e30, then splint)
          double y2[kNT], u[kNT];
          y2[0] = 0.;
          u[0] = 0.;
          for (int m = 1; m < nt - 1; ++m) {
            const double sig = (logt[m] - logt[m - 1]) / (logt[m + 1] - logt[m - 1]);
            const double p = sig * y2[m - 1] + 2.;
            y2[m] = (sig - 1.) / p;
            double um = qq[m + 1];
            um = um - qq[m];
            um = um / (logt[m + 1] - logt[m]);
            um = um - (qq[m] - qq[m - 1]) / (logt[m] - logt[m - 1]);
            u[m] = (6. * um / (logt[m + 1] - logt[m - 1]) - sig * u[m - 1]) / p;
          }
          y2[nt - 1] = (0. - 0. * u[nt - 2]) / (0. * y2[nt - 2] + 1.);
          for (int m = nt - 2; m >= 0; --m) y2[m] = y2[m] * y2[m + 1] + u[m];
          if (log10Te <= logt[0]) {
            qomInt = qq[0];
          } else if (log10Te >= logt[nt - 1]) {
            qomInt = qq[nt - 1];
          } else {
            int klo = 0, khi = nt - 1;
            while (khi - klo > 1) {
              const int m = (khi + klo) / 2;
              if (logt[m] > log10Te) khi = m;
              else klo = m;
            }
            const double h = logt[khi] - logt[klo];
            const double a = (logt[khi] - log10Te) / h, b = (log10Te - logt[klo]) / h;
            qomInt = a * qq[klo] + b * qq[khi] + ((a * a * a - a) * y2[klo] + (b * b * b - b) * y2[khi]) * (h * h) / 6.;
          }
        }
        const double delTeK = (e[i - 1] - e[j]) * 1.4388463;
        const double expFac = std::exp(delTeK / Te);
        qeff[i - 1][j] = 8.63e-6 * qomInt * expFac / (g[i - 1] * sqrTe);
        qeff[j][i - 1] = 8.63e-6 * qomInt / (g[j] * sqrTe);
      }
    double x[kLev][kLev] = {}, y[kLev] = {};
    for (int j = 1; j <= n; ++j) x[1][j] = 1.;
    y[1] = 1.;
    for (int i = 2; i <= n; ++i) {
      for (int j = 1; j <= n; ++j) {
        if (j == i) continue;
        x[i][j] += Ne * qeff[j][i];
        x[i][i] -= Ne * qeff[i][j];
        if (j > i) x[i][j] += A(j, i);
        else x[i][i] -= A(i, j);
      }
      y[i] = -Ne * ionDenUp * alphaTotal[i];
    }
    // luSlv: lured + reslv, no pivoting
    if (n > 1) {
      for (int i = 1; i <= n - 1; ++i)
        for (int kk = i + 1; kk <= n; ++kk) {
          const double f = x[kk][i] / x[i][i];
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
    double sumN = 0.;
    for (int i = 1; i <= n; ++i) sumN += y[i];
    double cool = 0.;
    const int top = std::min(n, top_levels);
    for (int i = 1; i <= top - 1; ++i)
      for (int j = i + 1; j <= top; ++j)
        if (A(j, i) != 0.) {
          const double line = A(j, i) * (e[j] - e[i]) * (y[j] / sumN);
          if (fscale <= 0.) cool += line;
          else if (line * fscale > 1e-35) cool += line * fscale;
        }
    return cool;
  }

  // ---- grains: setGrainPotential, getGrainEmission, getGrainRecombination,
  // setPhotoelHeatCool, setDustGasCollHeatCool (update_mod.f90:527-930)
  //
  // Sums over frequency are formed in the order of the GPU's warp (lane l
  // adds the terms of the bins i = l mod 32, i >= i0, in ascending order,
  // then the 32 partial sums are combined by the xor butterfly over offsets
  // 16, 8, 4, 2, 1), and so is the sum of the 33 ion currents in the
  // recombination rate (ion pair b in lane b mod 32); the sums over grain
  // sizes of the two gas terms go size by size after each size's own sum.
  // The reference adds the same terms one by one; only the rounding differs.
  template <class F>
  static double warpSum(int i0, int n, F term) {
    double p[32], q[32];
    for (int l = 0; l < 32; ++l) {
      p[l] = 0.;
      for (int i = i0 + ((l - i0) & 31); i < n; i += 32) p[l] += term(i);
    }
    for (int o = 16; o; o >>= 1) {
      for (int l = 0; l < 32; ++l) q[l] = p[l] + p[l ^ o];
      std::memcpy(p, q, sizeof p);
    }
    return p[0];
  }

  // interpolation_mod locate (1-based): n above the grid, 0 below it, else
  // the last entry <= x, and 1 where no entry exceeds x
  static int locate(const double *xa, int n, double x) {
    if (x > xa[n - 1]) return n;
    if (x < xa[0]) return 0;
    int lo = 0, hi = n;  // first index with xa > x (0-based), n if none
    while (lo < hi) {
      const int m = (lo + hi) >> 1;
      if (xa[m] > x) hi = m;
      else lo = m + 1;
    }
    return lo == n ? 1 : (lo > 1 ? lo : 1);
  }

  static constexpr double kPi = 3.141592654, kFourPi = 4. * 3.141592654, kHcRyd = 2.1799153e-11;
  static constexpr double kY0 = 0.5, kY1 = 0.2, kAmu = 1.66053e-24, kMe = 9.109382e-28;
  static constexpr double kRyd2erg = 2.1799e-11, kBoltz = 1.380658e-16;
  static double aWeight(int e) {
    static const double w[kNE] = {1.0080, 4.0026, 12.0111, 14.0067, 15.9994, 20.179, 32.06};
    return w[e];
  }

  // getGrainEmission (:610-663): photoelectrons per second from a grain of
  // size k at potential Vg [Ryd], the field above max(Vn + Vg, Vn)
  double grainEmission(int k, double Vg) const {
    const double vn = g->vn, *nu = g->nu, *xs = g->xs_abs + (size_t)k * g->nbins;
    const double r = g->radius_um[k], qden = 1.e-8 * (r * r);
    const double thres = std::max(vn + Vg, vn);
    const int ip = locate(nu, g->nbins, thres);  // the loop starts at ip + 1 (1-based)
    return warpSum(ip, g->nbins, [&](int i) {
      const double Yn = std::min(kY0 * (1. - vn / nu[i]), kY1);
      const double Yhat = Yn * std::min(1., std::max(0., 1. - Vg / (nu[i] - vn)));
      double photFlux = J[i] / (kHcRyd * nu[i]);
      photFlux = photFlux * kFourPi;
      const double Qa = xs[i] / qden;
      return Yhat * photFlux * Qa;
    });
  }

  // getGrainRecombination (:669-741): electron minus ion capture rate at Vg
  double grainRecombination(double Vg) const {
    const double kT = 6.336e-6 * Te, eightkT_pi = (1.1045e-15) * Te / kPi;
    double vmean = std::sqrt(eightkT_pi / kMe);
    double eta = -Vg / kT;
    eta = eta <= 0. ? 1. - eta : std::exp(-eta);
    const double rec = 0. + Ne * vmean * 1. * eta;
    double term[33];
    int b = 0;
    for (int e = 0; e < kNE; ++e)
      for (int s = 2; s <= nstage(e); ++s, ++b) {
        const double cpDen = X[e][s] * ab[e] * hden;
        const double mcp = aWeight(e) * kAmu;
        vmean = std::sqrt(eightkT_pi / mcp);
        const double Z = (double)(s - 1);
        double et = Z * Vg / kT;
        et = et <= 0. ? 1. - et : std::exp(-et);
        term[b] = cpDen * vmean * 1. * et;
      }
    return rec - warpSum(0, 33, [&](int i) { return term[i]; });
  }

  // setGrainPotential (:527-604) as a loop: from Vg = 0 a secant in Vg on
  // emission - recombination, steps at most 5 % of the threshold, until the
  // two agree within 0.5 % of their mean or after maxIterateGC = 100
  // evaluations.  `slope` is a `save` variable in the reference; here it
  // carries over the sizes of one T step of one cell, starting at 0.
  double grainPotential(int k, double &slope, bool &conv) const {
    const double errorLim = 0.005, dm = 0.05, vn = g->vn;
    double Vg = 0., VgOld = 0., emiOld = grainEmission(k, 0.), recOld = grainRecombination(0.);
    Vg = VgOld + 0.05;
    for (int n = 1;; ++n) {
      const double threshold = std::max(vn + Vg, vn);
      const double emi = grainEmission(k, Vg), rec = grainRecombination(Vg);
      double delta = emi - rec;
      double delta1 = std::fabs(delta / (0.5 * std::max(1.e-35, emi + rec)));
      if (delta1 < errorLim) return Vg;
      if (Vg != VgOld) {
        const double fac = (emi - emiOld) - (rec - recOld);
        if (fac != 0.) slope = fac / (Vg - VgOld);
      }
      VgOld = Vg;
      recOld = rec;
      emiOld = emi;
      delta1 = -delta / slope;
      delta = std::fabs(delta1);
      delta = std::min(delta, dm * threshold);
      delta = std::copysign(delta, delta1);
      Vg = Vg + delta;
      if (n >= 100) { conv = false; return Vg; }
    }
  }

  // setPhotoelHeatCool (:745-806): the grains' photoelectric cooling per
  // size and the gas heating per H
  void photoelHeatCool() {
    const double vn = g->vn, *nu = g->nu;
    photoG = 0.;
    for (int k = 0; k < g->nsizes; ++k) {
      const double Vg = vg[k], *xs = g->xs_abs + (size_t)k * g->nbins;
      const double th = std::max(vn + Vg, vn);
      int thP = locate(nu, g->nbins, th);
      if (thP <= 0) thP = 1;
      auto pieces = [&](int i, double &Qflux, double &EY, double &Yhat) {
        const double Yn = std::min(kY0 * (1. - vn / nu[i]), kY1);
        Yhat = Yn * std::min(1., std::max(0., 1. - Vg / (nu[i] - vn)));
        const double photFlux = J[i] / (kHcRyd * nu[i]);
        const double Qa = xs[i];
        const double d = nu[i] - vn;
        EY = Yn * 0.5 * std::min(d, std::max(0., (d * d - Vg * Vg) / d));
        Qflux = Qa * photFlux;
      };
      photoD[k] = warpSum(thP - 1, g->nbins, [&](int i) {
        double Qf, EY, Yh;
        pieces(i, Qf, EY, Yh);
        return Qf * EY * kHcRyd / kPi;
      });
      const double gk = warpSum(thP - 1, g->nbins, [&](int i) {
        double Qf, EY, Yh;
        pieces(i, Qf, EY, Yh);
        return Qf * (EY - Yh * Vg) * g->abundance * g->weight[k];
      });
      photoG = photoG + gk;
    }
    photoG = photoG * ndust * kHcRyd / hden;
  }

  // setDustGasCollHeatCool (:810-930): collisions of the gas particles
  // (every stage of every element, then electrons) with the grains.  IPerg
  // of a neutral stage is the value left from the element before it, as in
  // the reference (an unset local there for H0, taken as 0 here).
  void dustGasColl() {
    const int ns = g->nsizes;
    const double kT = 6.336e-6 * Te, eightkT_pi = (1.1045e-15) * Te / kPi;
    double cg[32];
    for (int k = 0; k < ns; ++k) { collD[k] = 0.; cg[k] = 0.; }
    double IPerg = 0.;
    for (int e = 0; e < kNE; ++e)
      for (int s = 1; s <= nstage(e); ++s) {
        const double Z = (double)(s - 1);
        const double mcp = aWeight(e) * kAmu;
        const double vmean = std::sqrt(eightkT_pi / mcp);
        if (s > 1) IPerg = g->ion_nu[bidx(e, s - 1)] * kRyd2erg;
        const double S = s == 1 ? 2. * mcp * g->msurf / ((mcp + g->msurf) * (mcp + g->msurf)) : 1.;
        for (int k = 0; k < ns; ++k) {
          const double r = g->radius_um[k], Vg = vg[k], Td = tdust ? tdust[k] : 0.;
          const double psi = Z * Vg / kT;
          double eta, xi;
          if (psi <= 0.) { eta = 1. - psi; xi = 1. - psi / 2.; }
          else { eta = std::exp(-psi); xi = (1. + psi / 2.) * eta; }
          collD[k] = collD[k] + X[e][s] * ab[e] * hden * kPi * r * r * 1.e-8 * S * vmean *
                                    (2. * kT * kRyd2erg * xi - eta * (Z * Vg * kRyd2erg - IPerg + 2. * kBoltz * Td));
          cg[k] = cg[k] + X[e][s] * g->weight[k] * g->abundance * ndust * ab[e] * kPi * r * r * 1.e-8 * S * vmean *
                              (2. * kT * kRyd2erg * xi - eta * 2. * kBoltz * Td);
        }
      }
    const double vmean = std::sqrt(eightkT_pi / kMe);
    for (int k = 0; k < ns; ++k) {
      const double r = g->radius_um[k], Vg = vg[k];
      const double S = 1., Z = -1.;
      const double psi = Z * Vg / kT;
      double eta, xi;
      if (psi <= 0.) { eta = 1. - psi; xi = 1. - psi / 2.; }
      else { eta = std::exp(-psi); xi = (1. + psi / 2.) * eta; }
      collD[k] = collD[k] + Ne * kPi * r * r * 1.e-8 * S * vmean * (2. * kT * kRyd2erg * xi - eta * (Z * Vg * kRyd2erg));
      cg[k] = cg[k] + Ne * g->weight[k] * g->abundance * ndust * kPi * r * r * 1.e-8 * S * vmean *
                          (2. * kT * kRyd2erg * xi) / hden;
    }
    collG = 0.;
    for (int k = 0; k < ns; ++k) collG = collG + cg[k];
    for (int k = 0; k < ns; ++k) collD[k] = collD[k] / kFourPi;
    collG = collG / kFourPi;
  }

  // the grain block of one T step (iterateT :367-386)
  void grainTerms() {
    double slope = 0.;
    gcConv = true;
    for (int k = 0; k < g->nsizes; ++k) vg[k] = grainPotential(k, slope, gcConv);
    photoelHeatCool();
    dustGasColl();
  }

  void thermBalance(double &heatInt, double &coolInt) {
    const double kB = 1.380658e-16, hcRyd = 2.1799153e-11;
    const double log10Te = std::log10(Te), Te4 = Te / 1.e4;
    auto poly4 = [](double x, const double c[5]) {
      return c[0] + c[1] * x + c[2] * x * x + c[3] * x * x * x + c[4] * x * x * x * x;
    };
    const double cFF[5] = {1.0108464E-11, 9.7930778E-13, -6.6433144E-13, 2.4793747E-13, -2.3938215E-14};
    const double cRec[5] = {9.4255985E-11, -4.04794384E-12, -1.0055237E-11, 1.99266862E-12, -1.06681387E-13};
    double Np = X[0][2] * ab[0];
    double coolFF = Np * Ne * poly4(log10Te, cFF) * kB * Te / std::sqrt(Te);
    double coolRec = Np * Ne * poly4(log10Te, cRec) * kB * Te / std::sqrt(Te);
    Np = X[1][3] * ab[1];
    const double lts = std::log10(Te / 4.);
    coolFF += Np * Ne * (2. * poly4(lts, cFF)) * kB * Te / std::sqrt(Te / 4.);
    coolRec += Np * Ne * (2. * poly4(lts, cRec)) * kB * Te / std::sqrt(Te / 4.);
    Np = X[1][2] * ab[1];
    coolFF += Np * Ne * (1.070073e-11 - 2.5730207e-13 * log10Te + 2.109134e-13 * log10Te * log10Te) * kB * Te /
              std::sqrt(Te);
    coolRec += Np * Ne * poly4(log10Te, cRec) * kB * Te / std::sqrt(Te);
    double coolColl = 0.;
    if (Te > 5000.)
      coolColl = (2.47e-8 * std::exp(-118338. / Te) * std::pow(Te4, -0.228) +
                  1.32e-8 * std::exp(-140252. / Te) * std::pow(Te4, -0.460)) *
                 hcRyd * X[0][1] * Ne;
    for (int k = 0; k < t->ncel; ++k) {
      const int z = t->cel_key[2 * k], ion = t->cel_key[2 * k + 1];
      int e = 0;
      while (e < kNE && kZ[e] != z) ++e;
      if (e == kNE || ion > nstage(e)) continue;
      const double up = ion < kNS ? X[e][ion + 1] / X[e][ion] : 0.;
      coolColl += celCooling(k, up) * ab[e] * X[e][ion] * 1.9865e-16;
    }
    double heatSte = 0.;
    for (int e = 0; e < kNE; ++e)
      for (int ion = 1; ion <= nion(e); ++ion) heatSte += heat[bidx(e, ion)] * X[e][ion] * ab[e];
    heatInt = heatSte;
    coolInt = coolFF + coolRec + coolColl;
    if (g) {
      coolInt = coolInt + collG;
      heatInt = heatInt + photoG;
    }
  }

  // iterateT as a loop (the recursion re-enters with the new TeUsed)
  void iterateT() {
    for (;;) {
      ++nIterT;
      calcAlpha();
      nIterX = 1;
      ionBalance();
      if (g) grainTerms();
      double heatInt, coolInt;
      thermBalance(heatInt, coolInt);
      const double thResidual = heatInt - coolInt;
      if (std::fabs(thResidual) >= 0.01 * heatInt) {
        if (nIterT < 25) {
          if (thResidual < 0) {
            thResLow = thResidual;
            Tlow = Te;
            if (Thigh != 0.) Te = Tlow - (Thigh - Tlow) * thResLow / (thResHigh - thResLow);
            else Te = Te / 1.2;
          } else {
            thResHigh = thResidual;
            Thigh = Te;
            if (Tlow != 0.) Te = Tlow - (Thigh - Tlow) * thResLow / (thResHigh - thResLow);
            else Te = Te * 1.2;
          }
          if (nIterT >= 6 && std::fabs(Thigh - Tlow) <= 0.002 * (Thigh + Tlow)) {
            if (thResidual < 0) { Te = Thigh - 100.; Thigh = 0.; }
            else { Te = Tlow + 100.; Tlow = 0.; }
          }
          if (Te <= 0.) Te = 1.;
          continue;
        }
        if (Thigh == 0.) Te = Tlow;
        else if (Tlow == 0.) Te = Thigh;
        else Te = (Thigh + Tlow) * 0.5;
        ++noTeBal;
      }
      if (!ionConv) ++noIonBal;
      return;
    }
  }
};

}  // namespace

extern "C" {

// Updates cells 1..ncells in place.  ionden: [Nc+1][7][8] (elements H He C N
// O Ne S, stage index 1..7); photo / heat: [Nc+1][33] balance-ion sums (Jste
// normalised, nPhotoSte without the 1e-20 floor); hit: cell was reached by a
// packet.  Outputs per cell: te, ne, ionden, conv (|dX(H0)/X(H0)| <= xhi_limit),
// niter (T iterations), flags (1 = no T balance, 2 = no ion balance, 8 = a
// grain potential did not converge in the last T step).
//
// With grains (g non-null): jste [nbins][Nc+1] is the normalised Jste
// (x scale), ndust [Nc+1] the grains per cm^3, tdust [nsizes][Nc+1] the
// grain temperatures of the previous iteration (null: 0 K); gout
// [3][nsizes][Nc+1] receives each cell's grain potential [Ryd],
// photoelHeat_d and gasDustColl_d of its last T step.
static void update_cells_impl(const upd_tables_t *t, int32_t ncells, const double *abund, const double *hden,
                              const double *photo, const double *heat, const int32_t *hit, double xhi_limit,
                              double *te, double *ne, double *ionden, int32_t *conv, int32_t *niter, int32_t *flags,
                              int32_t nthreads, const upd_grains_t *g, const double *jste, const double *ndust,
                              const double *tdust, double *gout) {
  const size_t nc1 = (size_t)ncells + 1;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
  for (int c = 1; c <= ncells; ++c) {
    if (!hit[c]) { conv[c] = 0; niter[c] = 0; flags[c] = 0; continue; }
    Cell C;
    C.t = t;
    C.ab = abund;
    C.hden = hden[c];
    C.photo = photo + (size_t)c * 33;
    C.heat = heat + (size_t)c * 33;
    C.Te = te[c];
    C.Ne = ne[c];
    std::vector<double> jrow, trow;
    if (g) {
      jrow.resize(g->nbins);
      for (int i = 0; i < g->nbins; ++i) jrow[i] = jste[(size_t)i * nc1 + c];
      trow.assign(g->nsizes, 0.);
      if (tdust)
        for (int k = 0; k < g->nsizes; ++k) trow[k] = tdust[(size_t)k * nc1 + c];
      C.g = g;
      C.J = jrow.data();
      C.ndust = ndust[c];
      C.tdust = trow.data();
    }
    double *X = ionden + (size_t)c * kNE * (kNS + 1);
    for (int e = 0; e < kNE; ++e)
      for (int s = 0; s <= kNS; ++s) C.X[e][s] = X[e * (kNS + 1) + s];
    const double XOldHI = C.X[0][1];
    C.iterateT();
    te[c] = C.Te;
    ne[c] = C.Ne;
    for (int e = 0; e < kNE; ++e)
      for (int s = 0; s <= kNS; ++s) X[e * (kNS + 1) + s] = C.X[e][s];
    conv[c] = std::fabs((C.X[0][1] - XOldHI) / XOldHI) <= xhi_limit ? 1 : 0;
    niter[c] = C.nIterT;
    flags[c] = (C.noTeBal ? 1 : 0) | (C.noIonBal ? 2 : 0) | (g && !C.gcConv ? 8 : 0);
    if (g)
      for (int k = 0; k < g->nsizes; ++k) {
        gout[((size_t)0 * g->nsizes + k) * nc1 + c] = C.vg[k];
        gout[((size_t)1 * g->nsizes + k) * nc1 + c] = C.photoD[k];
        gout[((size_t)2 * g->nsizes + k) * nc1 + c] = C.collD[k];
      }
  }
}

int oracle_update_cells(const upd_tables_t *t, int32_t ncells, const double *abund, const double *hden,
                        const double *photo, const double *heat, const int32_t *hit, double xhi_limit, double *te,
                        double *ne, double *ionden, int32_t *conv, int32_t *niter, int32_t *flags, int32_t nthreads) {
  update_cells_impl(t, ncells, abund, hden, photo, heat, hit, xhi_limit, te, ne, ionden, conv, niter, flags,
                    nthreads, nullptr, nullptr, nullptr, nullptr, nullptr);
  return 0;
}

int oracle_update_cells_grains(const upd_tables_t *t, int32_t ncells, const double *abund, const double *hden,
                               const double *photo, const double *heat, const int32_t *hit, double xhi_limit,
                               double *te, double *ne, double *ionden, int32_t *conv, int32_t *niter,
                               int32_t *flags, int32_t nthreads, const upd_grains_t *g, const double *jste,
                               const double *ndust, const double *tdust, double *gout) {
  if (!g || g->nsizes < 1 || g->nsizes > 32 || !jste || !ndust || !gout) return 1;
  update_cells_impl(t, ncells, abund, hden, photo, heat, hit, xhi_limit, te, ne, ionden, conv, niter, flags,
                    nthreads, g, jste, ndust, tdust, gout);
  return 0;
}

// The grain block at a fixed state of one cell (Te, Ne, ionden [7][8],
// Jste x scale [nbins], tdust [nsizes]): out[0][k] potential, out[1][k]
// photoelHeat_d, out[2][k] gasDustColl_d; gas[0] photoelHeat_g, gas[1]
// gasDustColl_g, gas[2] 1 if every potential converged; emi_rec[k][2] the
// emission and recombination rates at each size's final potential.
int oracle_grain_pieces(const upd_grains_t *g, const double *abund, double hden, double te, double ne,
                        const double *ionden, const double *jrow, double ndust, const double *tdust, double *out,
                        double *gas, double *emi_rec) {
  if (!g || g->nsizes < 1 || g->nsizes > 32) return 1;
  Cell C;
  C.t = nullptr;
  C.ab = abund;
  C.hden = hden;
  C.photo = nullptr;
  C.heat = nullptr;
  C.Te = te;
  C.Ne = ne;
  for (int e = 0; e < kNE; ++e)
    for (int s = 0; s <= kNS; ++s) C.X[e][s] = ionden[e * (kNS + 1) + s];
  C.g = g;
  C.J = jrow;
  C.ndust = ndust;
  C.tdust = tdust;
  C.grainTerms();
  for (int k = 0; k < g->nsizes; ++k) {
    out[k] = C.vg[k];
    out[g->nsizes + k] = C.photoD[k];
    out[2 * g->nsizes + k] = C.collD[k];
    emi_rec[2 * k] = C.grainEmission(k, C.vg[k]);
    emi_rec[2 * k + 1] = C.grainRecombination(C.vg[k]);
  }
  gas[0] = C.photoG;
  gas[1] = C.collG;
  gas[2] = C.gcConv ? 1. : 0.;
  return 0;
}

// Pieces of the update at a fixed state, for pinning against an independent
// restatement: alphaTot [33], the cooling of each line ion [ncel] per ion
// (equilibrium, levels 1..10), and heat / cool of thermBalance.
int oracle_update_pieces(const upd_tables_t *t, const double *abund, double hden, const double *photo,
                         const double *heat, double te, double ne, const double *ionden, double *alpha_out,
                         double *cel_out, double *heat_cool) {
  Cell C;
  C.t = t;
  C.ab = abund;
  C.hden = hden;
  C.photo = photo;
  C.heat = heat;
  C.Te = te;
  C.Ne = ne;
  for (int e = 0; e < kNE; ++e)
    for (int s = 0; s <= kNS; ++s) C.X[e][s] = ionden[e * (kNS + 1) + s];
  C.calcAlpha();
  for (int e = 0; e < kNE; ++e)
    for (int ion = 1; ion <= Cell::nion(e); ++ion) alpha_out[Cell::bidx(e, ion)] = C.alphaTot[e][ion];
  for (int k = 0; k < t->ncel; ++k) {
    const int z = t->cel_key[2 * k], ion = t->cel_key[2 * k + 1];
    int e = 0;
    while (e < kNE && kZ[e] != z) ++e;
    const double up = ion < kNS ? C.X[e][ion + 1] / C.X[e][ion] : 0.;
    cel_out[k] = C.celCooling(k, up);
  }
  C.thermBalance(heat_cool[0], heat_cool[1]);
  return 0;
}

// setDiffusePDF's forbidden-line totals (forLines, emission_mod.f90:837-903,
// and normFor, :1151-1172): per line ion k, the sum of its line
// emissivities [1e-25 erg/s per H] at Te, Ne and the ionic fractions, lines
// above 1e-35 only.  Ne below 1e-5 is taken as 1e-5 (emissionDriver :86-88).
int oracle_forbidden_lines(const upd_tables_t *t, const double *abund, double te, double ne, const double *ionden,
                           double *out) {
  Cell C;
  C.t = t;
  C.ab = abund;
  C.hden = 0.;
  C.photo = nullptr;
  C.heat = nullptr;
  C.Te = te;
  C.Ne = ne < 1e-5 ? 1e-5 : ne;
  for (int e = 0; e < kNE; ++e)
    for (int s = 0; s <= kNS; ++s) C.X[e][s] = ionden[e * (kNS + 1) + s];
  for (int k = 0; k < t->ncel; ++k) {
    const int z = t->cel_key[2 * k], ion = t->cel_key[2 * k + 1];
    int e = 0;
    while (e < kNE && kZ[e] != z) ++e;
    const double up = ion < kNS ? C.X[e][ion + 1] / C.X[e][ion] : 0.;
    out[k] = C.celCooling(k, up, 1 << 20, abund[e] * C.X[e][ion] * 1.9865e9);
  }
  return 0;
}

}  // extern "C"
