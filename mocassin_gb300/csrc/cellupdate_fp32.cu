// cellupdate_fp32.cu -- the FP32 form of the cell update as T-step
// wavefronts over all cells (the reference's own updateCell arithmetic is
// 4-byte `real`); compiled with the default contraction into FMA.
//
// The FP64 form (cellupdate.cuh, one warp per cell) follows the oracle
// operation by operation.  This form runs the same per-cell algorithm --
// iterateT's bracketed secant around ionBalance and thermBalance
// (update_mod.f90:339-1622) -- but batched across cells one T step at a
// time, so every lane of a warp does the same work:
//   wave_ion_kernel    one thread per active cell: calcAlpha and the
//                      ionBalance passes (at most 25) at the cell's Te;
//   wave_grain_kernel  (cells with grains) one warp per active cell: the
//                      grain potentials, photoelectric and collision terms
//                      of the T step (grains.cuh) at the new ion fractions;
//   wave_cel_kernel    one thread per (line ion, active cell): the level
//                      populations and forbidden-line cooling of that ion
//                      (equilibrium, emission_mod.f90:1913-2115); the 32
//                      lanes of a warp are 32 cells of one ion, so the level
//                      count and every loop bound are uniform;
//   wave_therm_kernel  one thread per active cell: the heating and cooling
//                      totals, the residual test and the secant step; a cell
//                      that is done writes its state, the others go on to
//                      the next T step's active list.
// State between the kernels is structure-of-arrays over cells (coalesced).
// The host issues the 25 possible T steps without synchronising: each
// kernel reads the active count from device memory.
#include <algorithm>

#include "cellupdate.cuh"
#include "tc_util.cuh"

namespace mcg {

namespace {

constexpr int kX = kNE * kNX;  // 56 ion slots per cell

struct WaveArgs {
  UpdArgs a;
  float *Xs;          // [56][nc+1] ion fractions, slot-major
  float *Te, *Ne;     // [nc+1]
  float *sec;         // [5][nc+1]: Thigh, Tlow, resHigh, resLow, fstep
  int *nit, *flags;   // [nc+1]: T steps, bit 1 = ion balance not converged in the last step
  float *cool;        // [ncel][nc+1] forbidden-line cooling per H
  float *gheat, *gcool;  // [nc+1] grains: photoelectric heating and collisional cooling of the gas per H
  float *gpf;            // [nc+1][nbp] grains: each cell's photon flux Jste x scale / (hcRyd nu) per bin
  int *act[2];        // active lists
  int *count;         // [2] their lengths
  unsigned int *cel_ctr;  // the level-population kernel's task counter (reset each T step)
};

__device__ __forceinline__ float &XS(const WaveArgs &w, int slot, int c) {
  return w.Xs[(size_t)slot * (w.a.nc + 1) + c];
}

__global__ void wave_init_kernel(const __grid_constant__ WaveArgs w) {
  const UpdArgs &a = w.a;
  const size_t nc1 = (size_t)a.nc + 1;
  for (int c = 1 + blockIdx.x * blockDim.x + threadIdx.x; c <= a.nc; c += gridDim.x * blockDim.x) {
    if (!(a.mom[c] > 0.f)) {
      a.conv[c] = 0; a.niter[c] = 0; a.flags[c] = 0; a.dte[c] = -1.;
      continue;
    }
    const double *Xc = a.X + (size_t)c * kX;
    for (int i = 0; i < kX; ++i) w.Xs[i * nc1 + c] = (float)Xc[i];
    w.Te[c] = (float)a.te[c];
    w.Ne[c] = (float)a.ne[c];
    for (int k = 0; k < 4; ++k) w.sec[k * nc1 + c] = 0.f;
    w.sec[4 * nc1 + c] = (float)a.step0;
    w.nit[c] = 0;
    w.flags[c] = 0;
    w.act[0][atomicAdd(&w.count[0], 1)] = c;
  }
}

// calcAlpha and ionBalance of every active cell at its current Te.  The
// per-ion terms that stay fixed through the passes (photoionisation rate,
// charge-exchange reverse rate, recombination coefficient, charge-exchange
// rate x Hden) sit in shared memory, one column per thread, so the passes
// keep only the ion fractions in registers.
constexpr int kIonThreads = 64;
__global__ void __launch_bounds__(kIonThreads) wave_ion_kernel(const __grid_constant__ WaveArgs w, int cur) {
  extern __shared__ float ion_sm[];
  float *sP = ion_sm, *sRev = ion_sm + kNB * kIonThreads, *sAl = ion_sm + 2 * kNB * kIonThreads,
        *sChh = ion_sm + 3 * kNB * kIonThreads;
  const int t = threadIdx.x;
  const UpdArgs &a = w.a;
  const UpdTabs<float> &T = a.f;
  const int n = w.count[cur];
  const float xMax = 0.99999f;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int c = w.act[cur][k];
    const float Te = w.Te[c], hden = (float)a.hden[c];
    float X[kNE][kNX];
    for (int e = 0; e < kNE; ++e)
      for (int s = 0; s < kNX; ++s) X[e][s] = XS(w, e * kNX + s, c);
    float Ne = w.Ne[c];
    float expFact = 157893.94f / Te;
    if (expFact > 75.f) expFact = 75.f;
    const float collIon0 = 2.75E-16f * Te * sqrtf(Te) * (157893.94f / Te + 2.f) * expf(-expFact);
    const float t4 = Te / 10000.f;
    // the charge-exchange rates depend on Te only
    for (int b = 0; b < kNB; ++b) {
      const UpdIonT<float> &B = T.bal[b];
      float x = B.chex[0] * powf(t4, B.chex[1]) * (1.f + B.chex[2] * expf(B.chex[3] * t4));
      if (x < 0.f) x = 0.f;
      if (Te < 6000.f || Te > 5.e4f) x = 0.f;
      sChh[b * kIonThreads + t] = x * hden;
      sRev[b * kIonThreads + t] = B.dek > 1.f ? x * hden * 2.f * expf(-B.dek / Te) / B.g0g1 : 0.f;
      sAl[b * kIonThreads + t] = alpha_of<float>(a, B, Te);
      sP[b * kIonThreads + t] = a.mom[(size_t)(1 + b) * a.mstride + c] + 1e-20f + (b == 0 ? collIon0 : 0.f);
    }
    bool conv = true;
    for (int pass = 1;; ++pass) {
      conv = true;
      const float HIOld = X[0][1], HeIOld = X[1][1], HeIIOld = X[1][2];
      float ne = 0.f;
      for (int e = 0; e < kNE; ++e) {
        const int z = a.bal_z[e], b0 = a.bal_first[e], ni = nion_of(z), ns = nstage_of(z);
        float prod[kNS + 1];
        float p = 1.f, den = 1.f;
        for (int ion = 1; ion <= ni; ++ion) {
          const int b = (b0 + ion - 1) * kIonThreads + t;
          p *= (sP[b] + sRev[b] * (1.f - HIOld)) / (Ne * sAl[b] + sChh[b] * HIOld);
          prod[ion] = p;
          den += p;
        }
        for (int ion = 1; ion <= ns; ++ion) {
          float v = ion == 1 ? 1.f / den : prod[ion - 1] / den;
          v = fminf(fmaxf(v, 1.e-20f), xMax);
          X[e][ion] = v;
          if (ion >= 2 && v >= 1.e-10f) ne += (float)(ion - 1) * T.ab[e] * v;
        }
      }
      Ne = ne * hden;
      if (Ne == 0.f) Ne = 1.f;
      const bool off = fabsf((X[0][1] - HIOld) / HIOld) > 0.01f || fabsf((X[1][1] - HeIOld) / HeIOld) > 0.01f ||
                       fabsf((X[1][2] - HeIIOld) / HeIIOld) > 0.01f;
      if (off && pass < 25) continue;
      if (off) conv = false;
      break;
    }
    for (int e = 0; e < kNE; ++e)
      for (int s = 1; s < kNX; ++s) XS(w, e * kNX + s, c) = X[e][s];
    w.Ne[c] = Ne;
    w.flags[c] = (w.flags[c] & 4) | (conv ? 0 : 2);
  }
}

// each cell's photon flux per bin for the grain block, once per update:
// Jste [nb][nc+1] (bin-major) -> gpf [nc+1][nbp] (cell-major), through 32 x
// 32 tiles in shared memory so that both sides are coalesced
__global__ void grain_flux_kernel(const __grid_constant__ WaveArgs w) {
  __shared__ float tile[32][33];
  const GrainArgs &g = w.a.g;
  const int nc1 = w.a.nc + 1, nb = g.nb, nbp = (nb + 1) & ~1;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
  const int tiles_c = (nc1 + 31) / 32, tiles_b = (nb + 31) / 32;
  for (int t = blockIdx.x; t < tiles_c * tiles_b; t += gridDim.x) {
    const int c0 = (t % tiles_c) * 32, b0 = (t / tiles_c) * 32;
    for (int r = ty; r < 32; r += 8) {
      const int b = b0 + r, c = c0 + tx;
      float v = 0.f;
      // FP32 form: Jste rounded by integer operations, times the bin's
      // jscale / (hcRyd nu) in FP32 (no FP64 arithmetic per element)
      if (b < nb && c < nc1) v = f64_to_f32_rn(g.jste[(size_t)b * nc1 + c]) * (float)(g.jscale * g.inv_hnu[b]);
      tile[r][tx] = v;
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
      const int c = c0 + r, b = b0 + tx;
      if (c < nc1 && b < nb) w.gpf[(size_t)c * nbp + b] = tile[tx][r];
    }
    __syncthreads();
  }
}

// the grain block of every active cell at its current Te and ion fractions
// (one warp per cell; the cell's photon flux per bin staged in shared memory)
__global__ void __launch_bounds__(128) wave_grain_kernel(const __grid_constant__ WaveArgs w, int cur) {
  extern __shared__ __align__(16) float gr_pf[];
  const UpdArgs &a = w.a;
  const GrainArgs &g = a.g;
  const int n = w.count[cur], ns = g.nsizes, nb = g.nb;
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const size_t nc1 = (size_t)a.nc + 1;
  const int nbp = (nb + 1) & ~1;
  float *pf = gr_pf + (size_t)wid * nbp;
  float *sfx = gr_pf + 4 * (size_t)nbp + (size_t)wid * ns * 2 * kGrWin;
  for (int k = blockIdx.x * 4 + wid; k < n; k += gridDim.x * 4) {
    const int c = w.act[cur][k];
    for (int i = lane; i < nb; i += 32) pf[i] = w.gpf[(size_t)c * nbp + i];
    const float td = (lane < ns && g.tdust) ? g.tdust[(size_t)(1 + lane) * nc1 + c] : 0.f;
    __syncwarp();
    auto Xf = [&](int e, int s) -> float { return XS(w, e * kNX + s, c); };
    float vg = 0.f, pd = 0.f, cd = 0.f;
    const GrainOut go = grain_step_fast(g, a.bal_z, a.bal_first, a.f.ab, w.Te[c], w.Ne[c], (float)a.hden[c],
                                        g.ndust[c], Xf, pf, sfx, td, lane, vg, pd, cd);
    if (lane == 0) {
      w.gheat[c] = (float)go.heat;
      w.gcool[c] = (float)go.cool;
      w.flags[c] = (w.flags[c] & ~8) | (go.converged ? 0 : 8);
    }
    if (lane < ns) {
      g.out[(size_t)lane * nc1 + c] = (double)vg;
      g.out[(size_t)(ns + lane) * nc1 + c] = (double)pd;
      g.out[(size_t)(2 * ns + lane) * nc1 + c] = (double)cd;
    }
    __syncwarp();
  }
}

// forbidden-line cooling per H of line ion `ion` in every active cell.  The
// level-population matrix of each thread is in local memory with the row
// length of the largest ion (mat_rows): the fewer bytes a thread touches, the
// more of the resident threads' matrices stay in the L1.
__global__ void __launch_bounds__(128) wave_cel_kernel(const __grid_constant__ WaveArgs w, int cur) {
  extern __shared__ float cel_stage_smem[];
  const UpdArgs &a = w.a;
  const UpdTabs<float> &T = a.f;
  const int n = w.count[cur];
  const int lane = threadIdx.x & 31;
  // tasks of 32 active cells of one line ion, ion-major, handed out by a
  // counter: the warps move through the list together, so a warp's next
  // task is mostly of the ion whose tables it has staged
  const unsigned int nchunk = (unsigned int)(n + 31) / 32u;
  const unsigned int total = nchunk * (unsigned int)a.ncel;
  float *stage = cel_stage_smem + (threadIdx.x >> 5) * kCelStage;
  int staged = -1;
  float x[kNL * kNL];
  while (true) {
    unsigned int t = 0;
    if (lane == 0) t = atomicAdd(w.cel_ctr, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= total) break;
    const int k = (int)(t / nchunk), ci = (int)(t % nchunk) * 32 + lane;
    const UpdCelT<float> &C = T.cel[k];
    const bool reg = cel_has_reg(C.nlev);
    if (reg && k != staged) {
      __syncwarp();
      cel_stage(T, k, C.nlev, C.nt, stage, lane);
      __syncwarp();
      staged = k;
    }
    if (ci >= n) continue;
    const int c = w.act[cur][ci];
    const float Te = w.Te[c], Ne = w.Ne[c];
    const float xi = XS(w, C.e * kNX + C.ion, c);
    const float up = C.ion < kNS ? XS(w, C.e * kNX + C.ion + 1, c) / xi : 0.f;
    float emis = 0.f;
    const float es = T.ab[C.e] * xi * 1.9865e9f;
    const float cool = reg ? cel_cooling_f32(a, k, CelTabStaged(stage), Te, Ne, up, x, a.mat_rows, 10, 0.f,
                                             a.forb_out ? &emis : nullptr, es)
                           : cel_cooling_smem<float>(a, k, Te, Ne, up, x, a.mat_rows, 10, 0.f,
                                                     a.forb_out ? &emis : nullptr, es);
    w.cool[(size_t)k * (a.nc + 1) + c] = cool * T.ab[C.e] * xi * 1.9865e-16f;
    if (a.forb_out) a.forb_out[(size_t)k * (a.nc + 1) + c] = emis;
  }
}

// heating and cooling totals, the residual test and the secant step
__global__ void __launch_bounds__(128) wave_therm_kernel(const __grid_constant__ WaveArgs w, int cur) {
  const UpdArgs &a = w.a;
  const UpdTabs<float> &T = a.f;
  const int n = w.count[cur];
  const size_t nc1 = (size_t)a.nc + 1;
  const float kB = 1.380658e-16f, hcRyd = 2.1799153e-11f;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
    const int c = w.act[cur][k];
    float Te = w.Te[c];
    const float Ne = w.Ne[c];
    const float log10Te = log10f(Te), Te4 = Te / 1.e4f;
    auto poly4 = [](float x, float c0, float c1, float c2, float c3, float c4) {
      return c0 + x * (c1 + x * (c2 + x * (c3 + x * c4)));
    };
    auto bff = [&](float x) { return poly4(x, 1.0108464E-11f, 9.7930778E-13f, -6.6433144E-13f, 2.4793747E-13f, -2.3938215E-14f); };
    auto brec = [&](float x) { return poly4(x, 9.4255985E-11f, -4.04794384E-12f, -1.0055237E-11f, 1.99266862E-12f, -1.06681387E-13f); };
    const float xH1 = XS(w, 1, c), xH2 = XS(w, 2, c), xHe2 = XS(w, kNX + 2, c), xHe3 = XS(w, kNX + 3, c);
    float Np = xH2 * T.ab[0];
    float coolFF = Np * Ne * bff(log10Te) * kB * Te / sqrtf(Te);
    float coolRec = Np * Ne * brec(log10Te) * kB * Te / sqrtf(Te);
    Np = xHe3 * T.ab[1];
    const float lts = log10f(Te / 4.f);
    coolFF += Np * Ne * (2.f * bff(lts)) * kB * Te / sqrtf(Te / 4.f);
    coolRec += Np * Ne * (2.f * brec(lts)) * kB * Te / sqrtf(Te / 4.f);
    Np = xHe2 * T.ab[1];
    coolFF += Np * Ne * (1.070073e-11f - 2.5730207e-13f * log10Te + 2.109134e-13f * log10Te * log10Te) * kB * Te / sqrtf(Te);
    coolRec += Np * Ne * brec(log10Te) * kB * Te / sqrtf(Te);
    float coolColl = 0.f;
    if (Te > 5000.f)
      coolColl = (2.47e-8f * expf(-118338.f / Te) * powf(Te4, -0.228f) + 1.32e-8f * expf(-140252.f / Te) * powf(Te4, -0.460f)) *
                 hcRyd * xH1 * Ne;
    for (int i = 0; i < a.ncel; ++i) coolColl += w.cool[(size_t)i * nc1 + c];
    float heat = 0.f;
    for (int b = 0; b < kNB; ++b) {
      const UpdIonT<float> &B = T.bal[b];
      heat += a.mom[(size_t)(1 + kNB + b) * a.mstride + c] * XS(w, B.e * kNX + B.ion, c) * T.ab[B.e];
    }
    float cool = coolFF + coolRec + coolColl;
    if (a.g.nsizes > 0) {
      cool += w.gcool[c];
      heat += w.gheat[c];
    }
    const float res = heat - cool;
    float Thigh = w.sec[0 * nc1 + c], Tlow = w.sec[1 * nc1 + c];
    float resHigh = w.sec[2 * nc1 + c], resLow = w.sec[3 * nc1 + c], fstep = w.sec[4 * nc1 + c];
    int nIterT = ++w.nit[c];
    bool again = false, noTe = false;
    const bool first_warm = a.x_prev && nIterT == 1 && !(w.flags[c] & 4);
    if (first_warm && fabsf(res) >= (float)a.near_res * heat) {
      // a prediction far from balance: the cold solve from the state before
      // the prediction, with the full T-step allowance (one extra T step)
      const double *Xp = a.x_prev + (size_t)c * kX;
      for (int i = 0; i < kX; ++i) XS(w, i, c) = (float)Xp[i];
      w.Te[c] = (float)a.te_prev[c];
      w.Ne[c] = (float)a.ne_prev[c];
      for (int k = 0; k < 4; ++k) w.sec[k * nc1 + c] = 0.f;
      w.sec[4 * nc1 + c] = 1.2f;
      w.nit[c] = 0;
      w.flags[c] |= 4;
      w.act[cur ^ 1][atomicAdd(&w.count[cur ^ 1], 1)] = c;
      continue;
    }
    if (fabsf(res) >= (first_warm ? (float)a.accept_res : 0.01f) * heat) {
      if (nIterT < 25) {
        bool open = false;
        if (res < 0.f) {
          resLow = res;
          Tlow = Te;
          if (Thigh != 0.f) Te = Tlow - (Thigh - Tlow) * resLow / (resHigh - resLow);
          else { Te = Te / fstep; open = true; }
        } else {
          resHigh = res;
          Thigh = Te;
          if (Tlow != 0.f) Te = Tlow - (Thigh - Tlow) * resLow / (resHigh - resLow);
          else { Te = Te * fstep; open = true; }
        }
        if (open && a.step_grow && !(w.flags[c] & 4)) fstep = fstep - 1.f < 0.1f ? 1.f + 2.f * (fstep - 1.f) : 1.2f;
        if (nIterT >= 6 && fabsf(Thigh - Tlow) <= 0.002f * (Thigh + Tlow)) {
          if (res < 0.f) { Te = Thigh - 100.f; Thigh = 0.f; }
          else { Te = Tlow + 100.f; Tlow = 0.f; }
        }
        if (Te <= 0.f) Te = 1.f;
        again = true;
      } else {
        if (Thigh == 0.f) Te = Tlow;
        else if (Tlow == 0.f) Te = Thigh;
        else Te = (Thigh + Tlow) * 0.5f;
        noTe = true;
      }
    }
    if (again) {
      w.Te[c] = Te;
      w.sec[0 * nc1 + c] = Thigh; w.sec[1 * nc1 + c] = Tlow;
      w.sec[2 * nc1 + c] = resHigh; w.sec[3 * nc1 + c] = resLow; w.sec[4 * nc1 + c] = fstep;
      w.act[cur ^ 1][atomicAdd(&w.count[cur ^ 1], 1)] = c;
      continue;
    }
    // done: the state goes back to the cell arrays (which still hold the
    // state the update started from: the convergence test compares with it)
    double *Xc = a.X + (size_t)c * kX;
    const double te0 = a.te_prev ? a.te_prev[c] : a.te[c];
    const double x0 = a.x_prev ? a.x_prev[(size_t)c * kX + 1] : Xc[1];
    for (int e = 0; e < kNE; ++e)
      for (int s = 1; s < kNX; ++s) Xc[e * kNX + s] = (double)XS(w, e * kNX + s, c);
    a.te[c] = (double)Te;
    a.ne[c] = (double)Ne;
    // the last T step's line totals belong to this state unless Te was moved
    // after them (no balance) or the emission would clamp Ne
    if (a.forb_ok) a.forb_ok[c] = (!noTe && Ne >= 1e-5f) ? 1 : 0;
    const double xh = (double)xH1;
    a.conv[c] = fabs((xh - x0) / x0) <= a.xhi ? 1 : 0;
    a.niter[c] = nIterT;
    a.flags[c] = (noTe ? 1 : 0) | (w.flags[c] & 14);
    a.dte[c] = fabs((double)Te - te0) / te0;
  }
}

__global__ void wave_reset_kernel(int *count, int slot, unsigned int *cel_ctr) {
  count[slot] = 0;
  *cel_ctr = 0u;
}

}  // namespace

// wave_cel_kernel: 2 blocks of 4 warps per SM (255 registers), each warp
// with its staged tables in shared memory
constexpr int kCelBlocksPerSm = 2;
static size_t cel_smem() { return (size_t)4 * kCelStage * sizeof(float); }

// shared memory of wave_grain_kernel: per warp the cell's photon flux per
// bin and each size's two suffix sums over the bins above grainVn
static size_t grain_smem(const GrainArgs &g) {
  const size_t nbp = (size_t)((g.nb + 1) & ~1);
  return 4 * nbp * sizeof(float) + 4 * (size_t)g.nsizes * 2 * kGrWin * sizeof(float);
}

cudaError_t cell_update_fp32_prepare(const UpdArgs &a) {
  if (a.g.nsizes > 0) {
    cudaError_t e = raise_smem_limit((const void *)wave_grain_kernel, (int)grain_smem(a.g));
    if (e != cudaSuccess) return e;
  }
  cudaError_t e = raise_smem_limit((const void *)wave_cel_kernel, (int)cel_smem());
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(wave_cel_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
}

size_t cell_update_fp32_scratch(int nc, int ncel, int nsizes, int nb) {
  const size_t nc1 = (size_t)nc + 1;
  // the arrays of launch_cell_update_fp32, each rounded up to 256 bytes
  auto r = [](size_t b) { return (b + 255) / 256 * 256; };
  return r(nc1 * kX * 4) + 2 * r(nc1 * 4) + r(nc1 * 5 * 4) + r(nc1 * (size_t)ncel * 4) + 4 * r(nc1 * 4) + r(8) +
         (nsizes > 0 ? 2 * r(nc1 * 4) + r(nc1 * (size_t)((nb + 1) & ~1) * 4) : 0);
}

cudaError_t launch_cell_update_fp32(const UpdArgs &a, void *scratch, int num_sms, cudaStream_t stream) {
  const size_t nc1 = (size_t)a.nc + 1;
  WaveArgs w{};
  w.a = a;
  char *p = (char *)scratch;
  auto take = [&](size_t bytes) { char *q = p; p += (bytes + 255) / 256 * 256; return q; };
  w.Xs = (float *)take(nc1 * kX * sizeof(float));
  w.Te = (float *)take(nc1 * sizeof(float));
  w.Ne = (float *)take(nc1 * sizeof(float));
  w.sec = (float *)take(nc1 * 5 * sizeof(float));
  w.cool = (float *)take(nc1 * (size_t)a.ncel * sizeof(float));
  w.nit = (int *)take(nc1 * sizeof(int));
  w.flags = (int *)take(nc1 * sizeof(int));
  w.act[0] = (int *)take(nc1 * sizeof(int));
  w.act[1] = (int *)take(nc1 * sizeof(int));
  w.count = (int *)take(4 * sizeof(int));  // two list lengths, the task counter
  w.cel_ctr = (unsigned int *)(w.count + 2);
  if (a.g.nsizes > 0) {
    w.gheat = (float *)take(nc1 * sizeof(float));
    w.gcool = (float *)take(nc1 * sizeof(float));
    w.gpf = (float *)take(nc1 * (size_t)((a.g.nb + 1) & ~1) * sizeof(float));
  }
  cudaError_t e = cudaMemsetAsync(w.count, 0, 4 * sizeof(int), stream);
  if (e != cudaSuccess) return e;
  const int blocks = num_sms * 8;
  wave_init_kernel<<<blocks, 256, 0, stream>>>(w);
  if (a.g.nsizes > 0) grain_flux_kernel<<<num_sms * 8, 256, 0, stream>>>(w);
  // a warm start may send a cell back to the cold solve after its first step
  const int steps = a.x_prev ? 26 : 25;
  for (int t = 0; t < steps; ++t) {
    const int cur = t & 1;
    wave_reset_kernel<<<1, 1, 0, stream>>>(w.count, cur ^ 1, w.cel_ctr);
    wave_ion_kernel<<<blocks * 2, kIonThreads, 4 * kNB * kIonThreads * sizeof(float), stream>>>(w, cur);
    if (a.g.nsizes > 0) wave_grain_kernel<<<blocks, 128, grain_smem(a.g), stream>>>(w, cur);
    wave_cel_kernel<<<num_sms * kCelBlocksPerSm, 128, cel_smem(), stream>>>(w, cur);
    wave_therm_kernel<<<blocks, 128, 0, stream>>>(w, cur);
  }
  return cudaGetLastError();
}

}  // namespace mcg
