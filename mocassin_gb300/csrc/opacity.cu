// opacity.cu -- the per-cell opacity build as a dense contraction.
//
// addOpacity (source/ionization_mod.f90:349-484) sums, for every active
// cell, xSecArray(range) * density over each ion's shell ranges, plus the
// free-free term; the dust add of iterateMC (source/iteration_mod.f90:
// 166-227) then adds grainAbun * grainWeight * Ndust * (xs_sca + xs_abs) per
// grain species and size.  Both are one contraction
//
//   opacity(cell, nu) = sum_k den(k, cell) * XS(k, nu)  +  ff(cell) [nu = 1]
//
// over "species" k = ions (shell-summed, zero below threshold) and grain
// (species, size) bins, with den the number densities (times the sublimation
// mask for grains).  Only bin 1 ever carries free-free opacity: FFOpacity(i)
// for i > 1 is never given a value (ionization_mod.f90:369-374), so ff is a
// one-bin epilogue term.
//
// Layouts (Fortran, cell fastest): den [K][Nc+1], XS [K][nbins],
// opacity [nbins][Nc+1].
//
// Two kernels:
//  opacity_fp32_kernel  CUDA cores, FP32 FMA (the exact path).
//  opacity_tc_kernel    5th-generation tensor cores: tcgen05.mma kind::f16
//                       with BF16 operands split in two terms (x = hi + lo),
//                       D = Ahi*Bhi + Ahi*Blo + Alo*Bhi accumulated in FP32 in
//                       tensor memory; ~1e-5 relative.  One CTA of 4 warps
//                       owns a 128-bin tile of XS in shared memory and walks
//                       128-cell tiles: the warps stage den (hi/lo) into shared
//                       memory, one thread issues the MMAs and commits them
//                       to an mbarrier, and the epilogue reads the accumulator
//                       back with tcgen05.ld and writes opacity coalesced along
//                       cells.  The kernel is output-bound (4 B written per
//                       cell and bin).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>

#include "mc_launch.h"
#include "tc_util.cuh"

namespace mcg {

constexpr int kOpM = 128;  // cells per tile (MMA M, TMEM lanes)
constexpr int kOpN = 128;  // bins per tile (MMA N, TMEM columns)
constexpr int kOpKMax = 64;

// ---------------------------------------------------------------- FP32
__global__ void __launch_bounds__(256) opacity_fp32_kernel(int nc1, int K, int nb, const float *__restrict__ den,
                                                           const float *__restrict__ xs,
                                                           const float *__restrict__ ff, float *__restrict__ out) {
  extern __shared__ float sxs[];  // [K][nb]
  for (int i = threadIdx.x; i < K * nb; i += blockDim.x) sxs[i] = xs[i];
  __syncthreads();
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < nc1; c += (long long)gridDim.x * blockDim.x) {
    float d[kOpKMax];
#pragma unroll
    for (int k = 0; k < kOpKMax; ++k) d[k] = k < K ? __ldg(den + (long long)k * nc1 + c) : 0.f;
    const float f = ff ? __ldg(ff + c) : 0.f;
    for (int v = 0; v < nb; ++v) {
      float acc = v == 0 ? f : 0.f;
#pragma unroll
      for (int k = 0; k < kOpKMax; ++k)
        if (k < K) acc = fmaf(d[k], sxs[k * nb + v], acc);
      out[(long long)v * nc1 + c] = acc;
    }
  }
}

// ------------------------------------------------------------- tcgen05
struct OpacityTcArgs {
  int nc1, K, nb;          // K padded to a multiple of 16 (<= 64)
  int nspecies;            // real species (rows of den / xs)
  const float *den, *xs, *ff;
  float *out;
  int *error;              // set to MC_ERR_TIMEOUT when an mbarrier wait gives up
};

__global__ void __launch_bounds__(128, 4) opacity_tc_kernel(const __grid_constant__ OpacityTcArgs a) {
  // shared: B hi/lo [N=128 bins][K], A hi/lo [M=128 cells][K], mbarrier, TMEM slot
  extern __shared__ __align__(1024) unsigned char sm[];
  const int K = a.K;
  const uint32_t tile_bytes = (uint32_t)kOpM * K * 2;  // 128 x K bf16
  unsigned char *sBhi = sm;
  unsigned char *sBlo = sm + tile_bytes;
  unsigned char *sAhi = sm + 2 * tile_bytes;
  unsigned char *sAlo = sm + 3 * tile_bytes;
  uint64_t *bar = (uint64_t *)(sm + 4 * tile_bytes);
  uint32_t *tslot = (uint32_t *)(bar + 1);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int v0 = blockIdx.x * kOpN;  // this CTA's bin tile

  // B = XS^T for bins v0..v0+127 (row = bin, column = species)
  for (int i = tid; i < kOpN * K; i += blockDim.x) {
    const int r = i / K, k = i % K;
    const int v = v0 + r;
    const float x = (k < a.nspecies && v < a.nb) ? __ldg(a.xs + (long long)k * a.nb + v) : 0.f;
    __nv_bfloat16 hi, lo;
    split_bf16(x, hi, lo);
    *(__nv_bfloat16 *)(sBhi + kmajor_off(r, k, K)) = hi;
    *(__nv_bfloat16 *)(sBlo + kmajor_off(r, k, K)) = lo;
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                 "r"(kOpN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  const uint32_t idesc = mma_idesc(kOpM, kOpN);
  const uint32_t lbo = 128, sbo = (uint32_t)(K / 8) * 128;
  uint32_t phase = 0;
  bool failed = false;

  const int ntiles = (a.nc1 + kOpM - 1) / kOpM;
  for (int t = blockIdx.y; t < ntiles && !failed; t += gridDim.y) {
    const int c0 = t * kOpM;
    // A = den^T for cells c0..c0+127 (row = cell, column = species): thread
    // r owns cell c0 + r; all its species loads are issued together
    // (coalesced along cells across the warp), then each group of 8 species
    // becomes one 16-byte row of a core matrix (conflict-free per quarter
    // warp)
    {
      const int r = tid, c = c0 + r;
      float x[kOpKMax];
#pragma unroll
      for (int k = 0; k < kOpKMax; ++k)
        x[k] = (k < a.nspecies && c < a.nc1) ? __ldg(a.den + (long long)k * a.nc1 + c) : 0.f;
#pragma unroll
      for (int kc = 0; kc < kOpKMax / 8; ++kc) {
        if (kc * 8 >= K) break;
        uint32_t hw[4], lw[4];
#pragma unroll
        for (int j = 0; j < 8; j += 2) {
          __nv_bfloat16 h0, l0, h1, l1;
          split_bf16(x[kc * 8 + j], h0, l0);
          split_bf16(x[kc * 8 + j + 1], h1, l1);
          hw[j / 2] = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
          lw[j / 2] = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
        }
        const uint32_t off = kmajor_off(r, kc * 8, K);
        *(uint4 *)(sAhi + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
        *(uint4 *)(sAlo + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t ah = smem_addr(sAhi), al = smem_addr(sAlo), bh = smem_addr(sBhi), bl = smem_addr(sBlo);
      int first = 1;
      for (int s = 0; s < K / 16; ++s) {
        const uint32_t ko = (uint32_t)s * 256;  // two core matrices along K per MMA
        const uint64_t dAh = smem_desc(ah + ko, lbo, sbo), dAl = smem_desc(al + ko, lbo, sbo);
        const uint64_t dBh = smem_desc(bh + ko, lbo, sbo), dBl = smem_desc(bl + ko, lbo, sbo);
        const uint64_t as[3] = {dAh, dAh, dAl}, bs[3] = {dBh, dBl, dBh};
        for (int j = 0; j < 3; ++j) {
          const uint32_t acc = first ? 0u : 1u;
          first = 0;
          asm volatile(
              "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
              "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
              "l"(as[j]), "l"(bs[j]), "r"(idesc), "r"(acc));
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_addr(bar))
                   : "memory");
    }
    // wait for the MMAs (bounded)
    uint32_t done = 0;
    for (long long it = 0; it < (1ll << 24) && !done; ++it) {
      asm volatile(
          "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
          : "=r"(done)
          : "r"(smem_addr(bar)), "r"(phase)
          : "memory");
    }
    failed = __syncthreads_or(!done);  // the whole CTA agrees
    if (failed && tid == 0) atomicExch(a.error, (int)MC_ERR_TIMEOUT);
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!failed) {
      // epilogue: warp w holds cells c0 + 32w + lane, bins v0 .. v0+127
      const int c = c0 + warp * 32 + lane;
      const float f = (a.ff && c < a.nc1 && v0 == 0) ? __ldg(a.ff + c) : 0.f;
      for (int j0 = 0; j0 < kOpN; j0 += 32) {
        uint32_t r[32];
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)j0;
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
              "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
              "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
              "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (c < a.nc1) {
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int v = v0 + j0 + j;
            if (v < a.nb) {
              float x = __uint_as_float(r[j]);
              if (v == 0) x += f;
              a.out[(long long)v * a.nc1 + c] = x;
            }
          }
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();  // the next tile overwrites the staged A and the accumulator
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kOpN));
}

// opacity_pipe_kernel: the same contraction with the epilogue overlapped.
// A persistent CTA of 8 warps holds one 128-bin tile of XS (hi/lo) and walks
// 128-cell tiles: two A buffers and two TMEM accumulators, so the MMAs of
// tile i run while the threads store tile i - 1 (each warp 32 cells x 64
// bins, coalesced along cells) and load the densities of tile i + 1.  The
// MMAs of a tile are those of opacity_tc_kernel in the same order.
constexpr int kOpPThreads = 256;

__global__ void __launch_bounds__(kOpPThreads, 2) opacity_pipe_kernel(const __grid_constant__ OpacityTcArgs a) {
  extern __shared__ __align__(1024) unsigned char sm[];
  const int K = a.K;
  const uint32_t tile_bytes = (uint32_t)kOpM * K * 2;  // 128 x K bf16
  unsigned char *sBhi = sm, *sBlo = sm + tile_bytes;
  auto sA = [&](int b) { return sm + (2u + 2u * (uint32_t)b) * tile_bytes; };  // hi, then lo
  uint64_t *mdone = (uint64_t *)(sm + 6 * tile_bytes);
  uint32_t *tslot = (uint32_t *)(mdone + 2);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nvt = (a.nb + kOpN - 1) / kOpN, ntiles = (a.nc1 + kOpM - 1) / kOpM;
  // block -> (bin tile, first cell tile, stride): the blocks of a bin tile
  // take its cell tiles in turn
  const int per = (int)gridDim.x / nvt;  // blocks per bin tile (the launch makes gridDim a multiple of nvt)
  const int vt = (int)blockIdx.x / per, t0 = (int)blockIdx.x % per;
  const int v0 = vt * kOpN;
  for (int i = tid; i < kOpN * K; i += blockDim.x) {
    const int r = i / K, k = i % K;
    const int v = v0 + r;
    const float x = (k < a.nspecies && v < a.nb) ? __ldg(a.xs + (long long)k * a.nb + v) : 0.f;
    __nv_bfloat16 hi, lo;
    split_bf16(x, hi, lo);
    *(__nv_bfloat16 *)(sBhi + kmajor_off(r, k, K)) = hi;
    *(__nv_bfloat16 *)(sBlo + kmajor_off(r, k, K)) = lo;
  }
  if (tid == 0) {
    for (int i = 0; i < 2; ++i) asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mdone + i)), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tslot)),
                 "r"(2 * kOpN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  const uint32_t idesc = mma_idesc(kOpM, kOpN);
  const uint32_t lbo = 128, sbo = (uint32_t)(K / 8) * 128;
  const int mytiles = t0 < ntiles ? (ntiles - 1 - t0) / per + 1 : 0;
  uint32_t ph = 0u;  // bit b: the next phase of mdone[b]
  bool ok = true, failed = false;
  int last_b = -1;
  uint32_t last_ph = 0u, cph = 0u;  // thread 0: the last commit and the next commit phases (bit b)

  // stores tile i from accumulator i & 1 once its MMAs are done
  auto epilogue = [&](int i) {
    const int b = i & 1;
    ok = mbar_wait(smem_addr(mdone + b), (ph >> b) & 1u) && ok;
    ph ^= 1u << b;
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const int q = warp & 3, h = warp >> 2;
    const int c = (t0 + i * per) * kOpM + q * 32 + lane;
    const float f = (a.ff && c < a.nc1 && v0 == 0 && h == 0) ? __ldg(a.ff + c) : 0.f;
    for (int j0 = 0; j0 < kOpN / 2; j0 += 32) {
      uint32_t r[32];
      tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)b * kOpN + (uint32_t)(h * (kOpN / 2) + j0), r);
      if (c < a.nc1) {
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int v = v0 + h * (kOpN / 2) + j0 + j;
          if (v < a.nb) {
            float x = __uint_as_float(r[j]);
            if (v == 0) x += f;
            a.out[(long long)v * a.nc1 + c] = x;
          }
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  };

  for (int i = 0; i < mytiles; ++i) {
    const int b = i & 1, c0 = (t0 + i * per) * kOpM;
    // A = den^T of this tile into buffer b (free: the epilogue of tile i - 2,
    // which waited for its MMAs, ran in the previous step)
    {
      const int r = tid & (kOpM - 1), kh = tid >> 7;  // cell row, species half
      const int c = c0 + r;
      const int kb = kh * (kOpKMax / 2);
      float x[kOpKMax / 2];
#pragma unroll
      for (int k = 0; k < kOpKMax / 2; ++k)
        x[k] = (kb + k < a.nspecies && c < a.nc1) ? __ldg(a.den + (long long)(kb + k) * a.nc1 + c) : 0.f;
#pragma unroll
      for (int kc = 0; kc < kOpKMax / 16; ++kc) {
        if (kb + kc * 8 >= K) break;
        uint32_t hw[4], lw[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) pack_split(x[kc * 8 + 2 * j], x[kc * 8 + 2 * j + 1], hw[j], lw[j]);
        const uint32_t off = kmajor_off(r, kb + kc * 8, K);
        *(uint4 *)(sA(b) + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
        *(uint4 *)(sA(b) + tile_bytes + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    failed = __syncthreads_or(!ok);
    if (failed) break;
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t d = tmem + (uint32_t)b * kOpN;
      const uint32_t ah = smem_addr(sA(b)), al = ah + tile_bytes, bh = smem_addr(sBhi), bl = smem_addr(sBlo);
      int first = 1;
      for (int s = 0; s < K / 16; ++s) {
        const uint32_t ko = (uint32_t)s * 256;
        const uint64_t dAh = smem_desc(ah + ko, lbo, sbo), dAl = smem_desc(al + ko, lbo, sbo);
        const uint64_t dBh = smem_desc(bh + ko, lbo, sbo), dBl = smem_desc(bl + ko, lbo, sbo);
        umma_bf16(d, dAh, dBh, idesc, first ? 0u : 1u);
        first = 0;
        umma_bf16(d, dAh, dBl, idesc, 1u);
        umma_bf16(d, dAl, dBh, idesc, 1u);
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                       smem_addr(mdone + b))
                   : "memory");
      last_b = b;
      last_ph = (cph >> b) & 1u;
      cph ^= 1u << b;
    }
    // the previous tile's stores overlap this tile's MMAs
    if (i >= 1) epilogue(i - 1);
  }
  if (!failed && mytiles > 0) {
    epilogue(mytiles - 1);
    failed = __syncthreads_or(!ok);
  } else {
    __syncthreads();
  }
  if (failed && tid == 0) atomicExch(a.error, (int)MC_ERR_TIMEOUT);
  if (tid == 0 && last_b >= 0) (void)mbar_wait(smem_addr(mdone + last_b), last_ph);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * kOpN));
}

size_t opacity_pipe_smem(int K) { return (size_t)6 * kOpM * K * 2 + 64; }

size_t opacity_tc_smem(int K) { return (size_t)4 * kOpM * K * 2 + 64; }

cudaError_t launch_opacity(int method, int nc1, int nspecies, int nb, const float *den, const float *xs,
                           const float *ff, float *out, int *error, int num_sms, cudaStream_t stream) {
  if (method == 0) {
    const size_t sh = (size_t)nspecies * nb * sizeof(float);
    cudaError_t e = raise_smem_limit((const void *)opacity_fp32_kernel, (int)sh);
    if (e != cudaSuccess) return e;
    const long long want = (nc1 + 255) / 256;
    const int blocks = (int)(want < num_sms * 4 ? want : num_sms * 4);
    opacity_fp32_kernel<<<blocks > 0 ? blocks : 1, 256, sh, stream>>>(nc1, nspecies, nb, den, xs, ff, out);
    return cudaGetLastError();
  }
  OpacityTcArgs a{};
  a.nc1 = nc1;
  a.nspecies = nspecies;
  a.K = ((nspecies + 15) / 16) * 16;
  a.nb = nb;
  a.den = den; a.xs = xs; a.ff = ff; a.out = out; a.error = error;
  if (a.K <= kOpKMax) {
    // the pipelined kernel: two CTAs per SM (2 x 256 TMEM columns), the
    // blocks split evenly over the bin tiles
    const size_t shp = opacity_pipe_smem(a.K);
    cudaError_t e = raise_smem_limit((const void *)opacity_pipe_kernel, (int)shp);
    if (e != cudaSuccess) return e;
    const int nvt = (nb + kOpN - 1) / kOpN;
    const int ntiles = (nc1 + kOpM - 1) / kOpM;
    int per = (2 * num_sms) / nvt;
    if (per > ntiles) per = ntiles;
    if (per < 1) per = 1;
    opacity_pipe_kernel<<<nvt * per, kOpPThreads, shp, stream>>>(a);
    return cudaGetLastError();
  }
  const size_t sh = opacity_tc_smem(a.K);
  cudaError_t e = raise_smem_limit((const void *)opacity_tc_kernel, (int)sh);
  if (e != cudaSuccess) return e;
  const int nvt = (nb + kOpN - 1) / kOpN;
  const int ntiles = (nc1 + kOpM - 1) / kOpM;
  e = cudaFuncSetAttribute(opacity_tc_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
  if (e != cudaSuccess) return e;
  // CTAs per SM from the shared-memory budget (227 KB), at most 4 (4 x 128
  // TMEM columns = 512)
  int per_sm = (int)((227 * 1024) / (sh + 1024));
  int want_sm = 4;
  if (const char *e2 = getenv("MC_OPAC_CTAS_PER_SM")) want_sm = atoi(e2);
  if (per_sm > want_sm) per_sm = want_sm;
  if (per_sm > 4) per_sm = 4;
  if (per_sm < 1) per_sm = 1;
  int per = (num_sms * per_sm + nvt - 1) / nvt;
  if (per > ntiles) per = ntiles;
  if (per < 1) per = 1;
  opacity_tc_kernel<<<dim3(nvt, per), 128, sh, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace mcg
