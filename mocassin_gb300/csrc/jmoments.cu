// jmoments.cu -- frequency moments of the mean-intensity estimator on the
// device, for the cell update.
//
// updateCell (source/update_mod.f90:175-269) starts with, for every cell and
// ion, the number of photoionisations
//     nPhotoSte(elem, ion) = 1e-20 + sum_j Jste(cell, j) * phXSec(j) / (hcRyd * nuArray(j))
// over the ion's frequency range, with Jste already normalised
// (iteration_mod.f90:705-724); the heating integrals of the thermal balance
// are sums of the same shape with other weights.  All of them are
//     out(o, cell) = scale * sum_nu Jste(nu, cell) * W(nu, o)
// for a weight table W [nbins][nout] that the caller builds, computed here on
// the resident Jste so that only the moments leave the GPU.
//
// jmoment_tc_kernel: tcgen05.mma kind::f16, both operands split into BF16
// hi + lo (D = hi*hi + hi*lo + lo*hi, FP32 accumulate in tensor memory).  A
// CTA of 4 warps walks 128-cell tiles; for each tile it streams Jste in
// 64-bin chunks (FP64 -> FP32 -> BF16 hi/lo, K-major core matrices in shared
// memory, loads coalesced along cells; the scale is applied in FP64 before
// the FP32 rounding, as the reference stores the normalised Jste in single
// precision), issues 12 MMAs per chunk from one
// thread and waits on an mbarrier (bounded).  Bound by reading Jste (8 B per
// cell and bin).
#include <cuda_runtime.h>

#include <cstdint>

#include "mc_launch.h"
#include "tc_util.cuh"

namespace mcg {

constexpr int kJM = 128;  // cells per tile
constexpr int kJK = 64;   // bins per chunk

struct JMomentArgs {
  int nc1, nb, nout, N;  // N = nout rounded up to 16 (<= 128)
  const double *J;       // [nb][nc1]
  const float *W;        // [nb][nout]
  double scale;
  float *out;            // [nout][nc1]
  int *error;
};

__global__ void __launch_bounds__(128, 4) jmoment_tc_kernel(const __grid_constant__ JMomentArgs a) {
  extern __shared__ __align__(1024) unsigned char sm[];
  const uint32_t abytes = (uint32_t)kJM * kJK * 2, bbytes = (uint32_t)a.N * kJK * 2;
  unsigned char *sAhi = sm, *sAlo = sm + abytes;
  unsigned char *sBhi = sm + 2 * abytes, *sBlo = sm + 2 * abytes + bbytes;
  uint64_t *bar = (uint64_t *)(sm + 2 * abytes + 2 * bbytes);
  uint32_t *tslot = (uint32_t *)(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t ncols = a.N <= 32 ? 32u : (a.N <= 64 ? 64u : 128u);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  const uint32_t idesc = mma_idesc(kJM, a.N);
  const uint32_t lbo = 128, sbo = (kJK / 8) * 128;
  uint32_t phase = 0;
  bool failed = false;
  const int ntiles = (a.nc1 + kJM - 1) / kJM;
  const int nchunks = (a.nb + kJK - 1) / kJK;

  for (int t = blockIdx.x; t < ntiles && !failed; t += gridDim.x) {
    const int c0 = t * kJM;
    for (int ch = 0; ch < nchunks && !failed; ++ch) {
      const int v0 = ch * kJK;
      {  // A: Jste for cells c0.. (row = cell, column = bin), thread = cell
        const int c = c0 + tid;
#pragma unroll 1
        for (int kc = 0; kc < kJK / 8; ++kc) {
          float x[8];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int v = v0 + kc * 8 + j;
            x[j] = (c < a.nc1 && v < a.nb) ? (float)(__ldg(a.J + (long long)v * a.nc1 + c) * a.scale) : 0.f;
          }
          uint32_t hw[4], lw[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) pack_split(x[2 * j], x[2 * j + 1], hw[j], lw[j]);
          const uint32_t off = kmajor_off(tid, kc * 8, kJK);
          *(uint4 *)(sAhi + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
          *(uint4 *)(sAlo + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
        }
      }
      // B: W^T for the chunk (row = output, column = bin)
      for (int i = tid; i < a.N * (kJK / 8); i += blockDim.x) {
        const int n = i % a.N, kc = i / a.N;
        float x[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int v = v0 + kc * 8 + j;
          x[j] = (n < a.nout && v < a.nb) ? __ldg(a.W + (long long)v * a.nout + n) : 0.f;
        }
        uint32_t hw[4], lw[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) pack_split(x[2 * j], x[2 * j + 1], hw[j], lw[j]);
        const uint32_t off = kmajor_off(n, kc * 8, kJK);
        *(uint4 *)(sBhi + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
        *(uint4 *)(sBlo + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      if (tid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t ah = smem_addr(sAhi), al = smem_addr(sAlo), bh = smem_addr(sBhi), bl = smem_addr(sBlo);
        for (int s = 0; s < kJK / 16; ++s) {
          const uint32_t ko = (uint32_t)s * 256;
          const uint64_t dAh = smem_desc(ah + ko, lbo, sbo), dAl = smem_desc(al + ko, lbo, sbo);
          const uint64_t dBh = smem_desc(bh + ko, lbo, sbo), dBl = smem_desc(bl + ko, lbo, sbo);
          const uint32_t acc0 = (ch == 0 && s == 0) ? 0u : 1u;
          umma_bf16(tmem, dAh, dBh, idesc, acc0);
          umma_bf16(tmem, dAh, dBl, idesc, 1u);
          umma_bf16(tmem, dAl, dBh, idesc, 1u);
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_addr(bar))
                     : "memory");
      }
      const bool done = mbar_wait(smem_addr(bar), phase);
      failed = __syncthreads_or(!done);
      if (failed && tid == 0) atomicExch(a.error, (int)MC_ERR_TIMEOUT);
      phase ^= 1u;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!failed) {
      const int c = c0 + warp * 32 + lane;
      for (int j0 = 0; j0 < a.N; j0 += 32) {
        uint32_t r[32];
        tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)j0, r);
        if (c < a.nc1) {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int o = j0 + j;
            if (o < a.nout) a.out[(long long)o * a.nc1 + c] = __uint_as_float(r[j]);
          }
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}

// Grain temperatures of getDustT (update_mod.f90:1899-1925): per cell and
// size bin, the absorbed integral A (a moment of Jste) located in the
// emission table E(T), T = 1..nt K, with locate's rules (interpolation_mod
// locate: nt above the table, 0 below it, else the last entry <= A, and 1
// when no entry exceeds A), then T = i + (A - E(i)) / (E(i+1) - E(i));
// below the table T = 1, above it T = nt.  Row 0 of tdust is the
// weighted mean over sizes; cells no packet reached get 0.  With gas and
// grains (gcd, gpd non-null: [nsizes][nc1] of the last cell update) the
// absorbed integral gains gasDustColl_d - photoelHeat_d (:1886-1889).
__global__ void dust_temperature_kernel(int nc1, int nsizes, int nt, const float *A, const float *E,
                                        const float *gw, const float *hit, float *tdust, const double *gcd,
                                        const double *gpd) {
  for (int c = 1 + blockIdx.x * blockDim.x + threadIdx.x; c < nc1; c += gridDim.x * blockDim.x) {
    const bool reached = hit[c] > 0.f;
    float mean = 0.f;
    for (int k = 0; k < nsizes; ++k) {
      float x = A[(size_t)k * nc1 + c];
      if (gcd) x = (float)(((double)x + gcd[(size_t)k * nc1 + c]) - gpd[(size_t)k * nc1 + c]);
      const float *e = E + (size_t)k * nt;
      float t = 0.f;
      if (reached) {
        int ns;
        if (x > e[nt - 1]) ns = nt;
        else if (x < e[0]) ns = 0;
        else {
          int lo = 0, hi = nt;  // first index with e > x (0-based), nt if none
          while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (e[mid] > x) hi = mid;
            else lo = mid + 1;
          }
          ns = lo == nt ? 1 : (lo > 1 ? lo : 1);  // 1-based: the entry before the first larger one
        }
        if (ns <= 0) t = 1.f;
        else if (ns >= nt) t = (float)nt;
        else t = (float)ns + (x - e[ns - 1]) * ((float)(ns + 1) - (float)ns) / (e[ns] - e[ns - 1]);
      }
      tdust[(size_t)(1 + k) * nc1 + c] = t;
      mean += t * gw[k];
    }
    tdust[c] = mean;
  }
}

cudaError_t launch_dust_temperature(int nc1, int nsizes, int nt, const float *A, const float *E, const float *gw,
                                    const float *hit, float *tdust, const double *gcd, const double *gpd, int num_sms,
                                    cudaStream_t stream) {
  dust_temperature_kernel<<<num_sms * 4, 256, 0, stream>>>(nc1, nsizes, nt, A, E, gw, hit, tdust, gcd, gpd);
  return cudaGetLastError();
}

cudaError_t launch_jmoments(int nc1, int nb, int nout, const double *J, const float *W, double scale, float *out,
                            int *error, int num_sms, cudaStream_t stream) {
  JMomentArgs a{};
  a.nc1 = nc1; a.nb = nb; a.nout = nout;
  a.N = ((nout + 15) / 16) * 16;
  a.J = J; a.W = W; a.scale = scale; a.out = out; a.error = error;
  const size_t sh = (size_t)2 * kJM * kJK * 2 + (size_t)2 * a.N * kJK * 2 + 64;
  cudaError_t e = raise_smem_limit((const void *)jmoment_tc_kernel, (int)sh);
  if (e != cudaSuccess) return e;
  // the whole carveout as shared memory, so several CTAs (each holding at
  // most 128 of the SM's 512 TMEM columns) share an SM and overlap their
  // Jste streams with each other's MMAs
  e = cudaFuncSetAttribute(jmoment_tc_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (e != cudaSuccess) return e;
  // CTAs per SM from the shared-memory (227 KB) and TMEM (512 columns) budgets
  const int ncols = a.N <= 32 ? 32 : (a.N <= 64 ? 64 : 128);
  int per_sm = (int)((227 * 1024) / (sh + 1024));
  if (per_sm > 512 / ncols) per_sm = 512 / ncols;
  if (per_sm > 4) per_sm = 4;
  if (per_sm < 1) per_sm = 1;
  const int ntiles = (nc1 + kJM - 1) / kJM;
  int blocks = num_sms * per_sm;
  if (blocks > ntiles) blocks = ntiles;
  jmoment_tc_kernel<<<blocks, 128, sh, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace mcg
