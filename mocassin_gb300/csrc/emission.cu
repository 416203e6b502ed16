// emission.cu -- the diffuse-emission CDF of every cell (recPDF row and
// totalLines) from its Te, Ne and ionic fractions, on the GPU, in FP32.
//
// The reference builds it per cell on the host before each transport
// (emissionDriver -> fb_ff, twoPhoton, RecLinesEmission, forLines,
// setDiffusePDF; emission_mod.f90:32-1311).  Here two kernels cover all
// cells of the resident state:
//   emission_forb_kernel  one thread per (line ion, cell): the level
//                         populations of the ion (equilibrium,
//                         emission_mod.f90:1913-2115) and the sum of its
//                         line emissivities above 1e-35 (forLines, normFor);
//                         the lanes of a warp are cells of one ion;
//   emission_cdf_kernel   one block per cell: the per-cell coefficients
//                         (Te interpolation of the gamma tables, the Gaunt
//                         expansion, two-photon rates, recombination lines)
//                         in shared memory, then one thread per frequency bin
//                         for the f-b, f-f, two-photon and heavy-ion
//                         continua, a block scan for the cumulative row, the
//                         normalisation and the 0.999998 snap; the row is
//                         written in place into the transport's CDF rows.
#include <algorithm>

#include "cellupdate.cuh"

namespace mcg {

namespace {

constexpr float kHcRydK = 157893.94f;
constexpr float kFourPi = 4.f * 3.141592654f;
constexpr int kEmiThreads = 128;

// the cells whose line totals do not belong to their state (ok[c] == 0)
__global__ void emission_stale_kernel(int nc, const int *ok, int *list, int *count) {
  for (int c = 1 + blockIdx.x * blockDim.x + threadIdx.x; c <= nc; c += gridDim.x * blockDim.x)
    if (!ok[c]) list[atomicAdd(count, 1)] = c;
}
__global__ void emission_fresh_kernel(const int *list, const int *count, int *ok) {
  const int n = *count;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) ok[list[i]] = 1;
}

__global__ void __launch_bounds__(128) emission_forb_kernel(const __grid_constant__ UpdArgs a, float *forb,
                                                            const int *list, const int *count) {
  const UpdTabs<float> &T = a.f;
  const int nc = a.nc, n = *count;
  const long long total = (long long)n * a.ncel;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
       q += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(q / n), c = list[q % n];
    const UpdCelT<float> &C = T.cel[k];
    const float Te = (float)a.te[c];
    const float Ne = fmaxf((float)a.ne[c], 1e-5f);
    const double *Xc = a.X + (size_t)c * kNE * kNX;
    const float xi = (float)Xc[C.e * kNX + C.ion];
    const float up = C.ion < kNS ? (float)Xc[C.e * kNX + C.ion + 1] / xi : 0.f;
    float x[kNL * kNL];
    forb[(size_t)k * (nc + 1) + c] =
        cel_cooling_f32(a, k, CelTabGlobal(T, k), Te, Ne, up, x, a.mat_rows, kNL, T.ab[C.e] * xi * 1.9865e9f);
  }
}

__device__ __forceinline__ float pow10f(float x) { return exp10f(x); }

// getFlux(energy, T, 'blackbody') (continuum_mod.f90:359-394): the Planck
// function over h, with the Wien and Rayleigh-Jeans branches
__device__ __forceinline__ float planck_over_h(float nu, float T) {
  const float hp = 6.6262e-27f, constant = 0.5250229f / hp;
  const float u = kHcRydK * nu / T;
  if (u > 86.f) return constant * nu * nu * nu * expf(-u);
  const float den = expf(u) - 1.f;
  if (den <= 0.f) return 3.32154e-6f * nu * nu * T / hp;
  return constant * nu * nu * nu / den;
}

__global__ void __launch_bounds__(kEmiThreads) emission_cdf_kernel(const __grid_constant__ EmiArgs E) {
  extern __shared__ float s_row[];  // [nb]
  __shared__ float s_lg[3][kEmiMaxLim], s_afit[3][kEmiMaxLim / 2], s_gc[2][8], s_w[kEmiMaxHeavy];
  __shared__ float s_scan[kEmiThreads / 32];
  __shared__ float s_par[16];
  __shared__ float s_td[kEmiMaxSizes];
  const int nb = E.nb, t = threadIdx.x;
  const int chunk = (nb + kEmiThreads - 1) / kEmiThreads;
  for (int c = 1 + blockIdx.x; c <= E.nc; c += gridDim.x) {
    const double *Xc = E.gas ? E.X + (size_t)c * kNE * kNX : nullptr;
    const float Te = E.gas ? (float)E.te[c] : 1e4f;
    const float Ne = E.gas ? fmaxf((float)E.ne[c], 1e-5f) : 1.f;
    const float sq = sqrtf(Te), l10 = log10f(Te), t4 = Te * 1e-4f, kT = kHcRydK / Te;
    const bool dust = E.nsizes > 0 && E.tdust != nullptr;
    if (dust && t < E.nsizes) s_td[t] = E.tdust[(size_t)(1 + t) * (E.nc + 1) + c];
    if (!E.gas) {
      // dust-only grid: setDustPDF (emission_mod.f90:1313-1387)
      __syncthreads();
      for (int b = t; b < nb; b += kEmiThreads) {
        const float nu = E.nu[b];
        float sd = 0.f;
        for (int ai = 0; ai < E.nsizes; ++ai) {
          const float T = s_td[ai];
          if (T > 0.f && T < E.t_sub)
            sd += E.xs_abs[(size_t)ai * nb + b] * planck_over_h(nu, T) * E.widflx[b] * E.gw[ai];
        }
        s_row[b] = sd;
      }
    }
    // ---- per-cell coefficients ----
    if (!E.gas) {
    } else if (t < E.nlim[0] + E.nlim[1] + E.nlim[2]) {
      int sidx = 0, i = t;
      while (i >= E.nlim[sidx]) { i -= E.nlim[sidx]; ++sidx; }
      const float *lg = E.lg[sidx];
      const int nl = E.nlim[sidx];
      float v;
      if (Te <= E.tk[0]) v = lg[i];
      else if (Te >= E.tk[E.ntk - 1]) v = lg[(E.ntk - 1) * nl + i];
      else {
        int k = 0;
        while (k + 1 < E.ntk - 1 && E.tk[k + 1] <= Te) ++k;
        const float afit = (lg[(k + 1) * nl + i] - lg[k * nl + i]) / log10f(E.tk[k + 1] / E.tk[k]);
        v = lg[k * nl + i] + afit * log10f(Te / E.tk[k]);
      }
      s_lg[sidx][i] = v;
    } else if (t >= 64 && t < 80) {
      // Gaunt factor expansion in gamma^2 (getGauntFF, ionization_mod.f90:249-276)
      const int z = (t - 64) >> 3, j = (t - 64) & 7;
      const float xlrkt = 5.1983649f - fminf(fmaxf(l10, 2.5f), 8.f);
      const float txg = 0.66666667f * (2.f * (z ? 0.30103f : 0.f) + xlrkt);
      float b[13];
      b[11] = E.gaunt_d[j * 11 + 10];
      b[10] = txg * b[11] + E.gaunt_d[j * 11 + 9];
      b[12] = 0.f;
      for (int ir = 9; ir >= 1; --ir) b[ir] = txg * b[ir + 1] - b[ir + 2] + E.gaunt_d[j * 11 + ir - 1];
      s_gc[z][j] = 0.25f * (b[1] - b[3]);
    } else if (t >= 80 && t < 96) {
      for (int h = t - 80; h < E.nheavy; h += 16)
        s_w[h] = E.h_g[h] * (float)Xc[E.h_e[h] * kNX + E.h_stage[h]] * E.ab[E.h_e[h]];
    } else if (t >= 96) {
      // warp 3: recombination lines (RecLinesEmission, :744-832), the
      // forbidden-line totals, then lane 0 the remaining per-cell rates
      const int lane = t - 96;
      const float abH = E.ab[0], abHe = E.ab[1];
      const float xH2 = (float)Xc[2], xHe2 = (float)Xc[kNX + 2], xHe3 = (float)Xc[kNX + 3];
      const float nn = Ne;
      const int den = nn <= 100.f ? 0 : (nn <= 1e4f ? 1 : (nn <= 1e6f ? 2 : 3));
      float part = 0.f;
      for (int l = lane; l < 34; l += 32) {
        const float *co = E.hei_rec + l * 12;
        auto fit = [&](int k) { return co[k * 4] * powf(t4, co[k * 4 + 1]) * expf(co[k * 4 + 2] / t4); };
        if (den == 1 || den == 2) {
          const float x1 = fit(den - 1), x2 = fit(den);
          const float p0 = den == 1 ? 100.f : 1e4f, p1 = den == 1 ? 1e4f : 1e6f;
          part += x1 + (x2 - x1) * (nn - p0) / (p1 - p0);
        } else {
          part += fit(den == 0 ? 0 : 2);
        }
      }
      float fo = lane < E.ncel ? E.forb[(size_t)lane * (E.nc + 1) + c] : 0.f;
      for (int o = 16; o; o >>= 1) {
        part += __shfl_xor_sync(0xffffffffu, part, o);
        fo += __shfl_xor_sync(0xffffffffu, fo, o);
      }
      if (lane == 0) {
        const float hbeta = pow10f(-0.870f * l10 + 3.57f) * Ne * xH2 * abH;
        const float lalpha = pow10f(-0.897f * l10 + 5.05f);
        float rec = hbeta * E.hi_rec_sum + abH * xH2 * Ne * lalpha;
        const float h4686 = pow10f(-0.997f * l10 + 5.16f) * Ne * abHe * xHe3;
        rec += h4686 * E.heii_rec_sum;
        rec += part * nn * abHe * xHe2;
        s_par[0] = rec + fo;
        // HeI 2^3S line into the HeI sum and the HeII Lyman lines (:996-1039)
        s_par[1] = 27.2f * powf(t4, -0.678f) * Ne * abHe * xHe2 * 1.45673f * 2.1799153e-11f * 1e11f;
        const float lya = pow10f(-0.792f * l10 + 6.01f) * Ne * xHe3 * abHe;
        for (int i = 0; i < 4; ++i) s_par[2 + i] = i == 3 ? lya : E.ly_data[i] * lya;
        // two-photon rates (hydro2phot, HeI2photSub)
        float q;
        if (Te <= 10000.f) q = 5.31e-4f;
        else if (Te >= 20000.f) q = 4.71e-4f;
        else q = pow10f(log10f(5.31e-4f) + log10f(4.71e-4f / 5.31e-4f) / log10f(2.f) * log10f(Te / 10000.f));
        s_par[6] = 0.8368f * powf(t4, -0.723f) / (1.f + Ne * q / 8.23f);
        float ahe;
        if (Te <= 5000.f) ahe = 6.161f;
        else if (Te >= 30000.f) ahe = 2.035f;
        else if (Te <= 10000.f) ahe = pow10f(log10f(6.161f) + log10f(4.091f / 6.161f) / log10f(2.f) * log10f(Te / 5000.f));
        else if (Te <= 15000.f) ahe = pow10f(log10f(4.091f) + log10f(3.189f / 4.091f) / log10f(1.5f) * log10f(Te / 10000.f));
        else ahe = pow10f(log10f(3.189f) + log10f(2.035f / 3.189f) / log10f(2.f) * log10f(Te / 15000.f));
        s_par[7] = ahe;
        s_par[8] = 6.23f * powf(t4, -0.827f);
      }
    }
    __syncthreads();
    if (E.gas && t < (E.nlim[0] + E.nlim[1] + E.nlim[2]) / 2) {
      int sidx = 0, p = t;
      while (p >= E.nlim[sidx] / 2) { p -= E.nlim[sidx] / 2; ++sidx; }
      const int iup = E.edge[sidx][2 * p + 1], ilow = E.edge[sidx][2 * p];
      s_afit[sidx][p] = (s_lg[sidx][2 * p + 1] - s_lg[sidx][2 * p]) / (E.nu[iup] - E.nu[ilow]);
    }
    __syncthreads();
    // ---- one thread per bin ----
    // the thermal grain emission of a gas grid (sumDiffuseDust, :1042-1105)
    const float dfac = dust && E.gas ? 6.6262e-27f * 4.f * 3.141592654f * 1e25f * 3.2898423e15f * E.ndust[c] / (float)E.hden[c]
                            : 0.f;
    const float xH2 = E.gas ? (float)Xc[2] : 0.f, xHe2 = E.gas ? (float)Xc[kNX + 2] : 0.f;
    const float xHe3 = E.gas ? (float)Xc[kNX + 3] : 0.f;
    const float abH = E.gas ? E.ab[0] : 0.f, abHe = E.gas ? E.ab[1] : 0.f;
    const float fH = abH * xH2 * Ne, fHeI = abHe * xHe2 * Ne, fHeII = abHe * xHe3 * Ne;
    const float xlrkt = 5.1983649f - fminf(fmaxf(l10, 2.5f), 8.f);
    const float con = 0.72727273f * xlrkt + 0.90909091f;
    float gam2[2];
    for (int z = 0; z < 2; ++z) gam2[z] = pow10f(0.66666667f * (2.f * (z ? 0.30103f : 0.f) + xlrkt) * 1.5f);
    const float cm = E.milne_c / (Te * sq);
    for (int b = t; E.gas && b < nb; b += kEmiThreads) {
      const float nu = E.nu[b];
      const float nu3 = nu * nu * nu;
      float g[3];
      for (int sidx = 0; sidx < 3; ++sidx) {
        const int p = E.pair[sidx * nb + b];
        g[sidx] = p >= 0 ? pow10f(s_lg[sidx][2 * p + 1] + s_afit[sidx][p] * (nu - E.nu[E.edge[sidx][2 * p + 1]])) : 0.f;
      }
      if (b >= E.p_from[0]) {
        float ff[2];
        const float lx = E.lnu[b];
        for (int z = 0; z < 2; ++z) {
          const float txu = 0.72727273f * lx + con;
          const float u = pow10f((txu - 0.90909091f) / 0.72727273f);
          float gf = 0.f;
          if (fabsf(txu) <= 2.f) {
            float bb[10];
            bb[8] = s_gc[z][7];
            bb[9] = 0.f;
            bb[7] = txu * bb[8] + s_gc[z][6];
            for (int ir = 6; ir >= 1; --ir) bb[ir] = txu * bb[ir + 1] - bb[ir + 2] + s_gc[z][ir - 1];
            gf = bb[1] - bb[3];
          } else if (log10f(u) < -4.f) {
            gf = gam2[z] < 0.3f ? 0.551329f * logf(2.24593f / u) : 0.551329f * logf(0.944931f / u / sqrtf(gam2[z]));
          } else if (txu > 2.f) {
            const float lg2 = log10f(gam2[z]);
            if (lg2 < -3.f) gf = sqrtf(0.9549297f / u);
            else if (lg2 < 0.f) {
              const float slope = (sqrtf(12.f * gam2[z] / u) - sqrtf(0.9549297f / u)) / 3.f;
              gf = sqrtf(12.f * gam2[z] / u) + slope * lg2;
            } else gf = fminf(1.05f, sqrtf(12.f * gam2[z] / u));
          }
          ff[z] = kFourPi * 54.43f * (z ? 4.f : 1.f) * gf * expf(-nu * kT) / sq;
        }
        const float f3 = nu3 * cm;
        g[0] = E.xs_h[b] * 2.f * f3 * expf((E.nu[E.p_milne[0]] - nu) * kT) + ff[0];
        if (b >= E.p_from[1]) {
          g[1] = E.xs_hei[b] * 0.5f * f3 * expf((E.nu[E.p_milne[1]] - nu) * kT) + ff[0];
          if (b >= E.p_from[2]) g[2] = E.xs_heii[b] * 2.f * f3 * expf((E.nu[E.p_milne[2]] - nu) * kT) + ff[1];
        }
      }
      float heavy = 0.f;
      for (int h = 0; h < E.nheavy; ++h)
        if (b >= E.h_ip[h] && b < E.h_hi[h])
          heavy += expf((E.h_nuip[h] - nu) * kT) * E.xs_outer[(size_t)h * nb + b] * s_w[h];
      heavy *= nu3 * cm;
      float eHI = (g[0] + s_par[6] * E.tp_hi[b]) * fH + heavy * Ne;
      float eHeI = (g[1] + s_par[8] * E.tp_hei[b]) * fHeI;
      float eHeII = (g[2] + s_par[7] * E.tp_heii[b]) * fHeII;
      if (eHI < 1e-15f) eHI = 0.f;
      if (eHeI < 1e-15f) eHeI = 0.f;
      if (eHeII < 1e-15f) eHeII = 0.f;
      const float w = E.wid[b];
      float sHeI = w * eHeI, sHeII = w * eHeII;
      if (b == E.j2) sHeI += s_par[1];
      for (int i = 0; i < 4; ++i)
        if (b == E.ly_bin[i]) sHeII += s_par[2 + i];
      float sd = 0.f;
      if (dust) {
        for (int ai = 0; ai < E.nsizes; ++ai) {
          const float T = s_td[ai];
          if (T < E.t_sub && T > 0.f)
            sd += E.xs_abs[(size_t)ai * nb + b] * planck_over_h(nu, T) * E.widflx[b] * E.gw[ai];
        }
        sd *= dfac;
      }
      s_row[b] = w * eHI + sHeI + sHeII + sd;
    }
    __syncthreads();
    // ---- cumulative row: sequential within a chunk, scanned across chunks ----
    const int b0 = t * chunk, b1 = min(b0 + chunk, nb);
    float run = 0.f;
    for (int b = b0; b < b1; ++b) { run += s_row[b]; s_row[b] = run; }
    const int lane = t & 31, wid = t >> 5;
    float incl = run;
    for (int o = 1; o < 32; o <<= 1) {
      const float v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    if (lane == 31) s_scan[wid] = incl;
    __syncthreads();
    float off = incl - run;
    for (int k = 0; k < wid; ++k) off += s_scan[k];
    for (int b = b0; b < b1; ++b) s_row[b] += off;
    // the chunk offsets are sums in another order than the running sums, so
    // a chunk may start one rounding below the end of the previous one: a
    // running maximum across chunks keeps the row non-decreasing, as the
    // reference's sequential sum is
    float last = b1 > b0 ? s_row[b1 - 1] : -INFINITY;
    float mx = last;
    for (int o = 1; o < 32; o <<= 1) {
      const float v = __shfl_up_sync(0xffffffffu, mx, o);
      if (lane >= o) mx = fmaxf(mx, v);
    }
    __syncthreads();
    if (lane == 31) s_scan[wid] = mx;
    __syncthreads();
    float before = __shfl_up_sync(0xffffffffu, mx, 1);
    if (lane == 0) before = -INFINITY;
    for (int k = 0; k < wid; ++k) before = fmaxf(before, s_scan[k]);
    for (int b = b0; b < b1; ++b) s_row[b] = fmaxf(s_row[b], before);
    __syncthreads();
    const float total = s_row[nb - 1];
    const bool ok = total > 0.f && total < INFINITY;
    float *out = (E.gas ? E.rec_cdf : E.dust_cdf) + (size_t)c * nb;
    for (int b = t; b < nb; b += kEmiThreads) {
      float v = ok ? s_row[b] / total : 1.f;
      if (b == nb - 1 || (E.gas && v > 0.999998f)) v = 1.f;
      out[b] = v;
    }
    if (E.gas && t == 0) {
      const float lines = s_par[0], all = (ok ? total : 0.f) + lines;
      E.total_lines[c] = all > 0.f ? lines / all : 0.f;
    }
    __syncthreads();
  }
}

}  // namespace

cudaError_t launch_emission(const UpdArgs &a, const EmiArgs &E, float *forb, int *ok, int *list, int *count,
                            int num_sms, cudaStream_t s) {
  if (E.nb > kEmiMaxBins || E.nheavy > kEmiMaxHeavy || E.nsizes > kEmiMaxSizes || E.nlim[0] > kEmiMaxLim || E.nlim[1] > kEmiMaxLim ||
      E.nlim[2] > kEmiMaxLim || E.nlim[0] + E.nlim[1] + E.nlim[2] > 64)
    return cudaErrorInvalidValue;
  if (a.ncel > 0) {
    // only the cells whose totals the update did not leave
    cudaError_t e = cudaFuncSetAttribute(emission_forb_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
    if (e == cudaSuccess) e = cudaMemsetAsync(count, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    emission_stale_kernel<<<num_sms * 4, 256, 0, s>>>(a.nc, ok, list, count);
    emission_forb_kernel<<<num_sms * 32, 128, 0, s>>>(a, forb, list, count);
    emission_fresh_kernel<<<num_sms * 4, 256, 0, s>>>(list, count, ok);
  }
  emission_cdf_kernel<<<num_sms * 12, kEmiThreads, (size_t)E.nb * sizeof(float), s>>>(E);
  return cudaGetLastError();
}

}  // namespace mcg
