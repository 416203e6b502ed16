// tc_util.cuh -- small helpers of the tcgen05 kernels: shared-memory matrix
// descriptors (K-major, no swizzle), the kind::f16 instruction descriptor,
// the core-matrix layout and the BF16 hi/lo split.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace mcg {

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: K-major, no swizzle.  Core matrices are
// 8 rows x 16 bytes; `lbo` is the byte step between core matrices along K,
// `sbo` along the rows.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;
  d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of sm_100 family
  return d;                // base offset 0, swizzle none
}

// Instruction descriptor of kind::f16: D f32, A and B bf16, both K-major.
__host__ __device__ constexpr uint32_t mma_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// byte offset of (row r, k) in a K-major no-swizzle tile of K columns
__device__ __forceinline__ uint32_t kmajor_off(int r, int k, int K) {
  return (uint32_t)((r >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ void split_bf16(float x, __nv_bfloat16 &hi, __nv_bfloat16 &lo) {
  hi = __float2bfloat16_rn(x);
  lo = __float2bfloat16_rn(x - __bfloat162float(hi));
}


// Issues D (+)= A x B for one K = 16 step (single thread).
__device__ __forceinline__ void umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// Bounded wait on an mbarrier phase; returns false when it gave up.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase) {
  uint32_t done = 0;
  for (long long it = 0; it < (1ll << 24) && !done; ++it) {
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(phase)
        : "memory");
  }
  return done != 0;
}

// 32 consecutive TMEM columns of this warp's 32 lanes into registers.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// (float)d, rounded to nearest even, by integer operations on the IEEE-754
// layouts (GB300 runs FP64 arithmetic and FP64 -> FP32 conversions at a
// small fraction of its FP32 rate): for results that are normal floats;
// zeros, subnormal or overflowing results, infinities and NaNs take the
// conversion instruction.
__device__ __forceinline__ float f64_to_f32_rn(double d) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(d);
  const int e = (int)((u >> 52) & 0x7ff) - 1023 + 127;  // the float's biased exponent
  if (e <= 0 || e >= 255) return (float)d;
  const unsigned long long m = u & 0xFFFFFFFFFFFFFull;  // 52 mantissa bits
  const uint32_t keep = (uint32_t)(m >> 29), rest = (uint32_t)(m & 0x1FFFFFFFull);
  const uint32_t up = (rest > 0x10000000u || (rest == 0x10000000u && (keep & 1u))) ? 1u : 0u;
  // a carry out of the mantissa moves into the exponent, as rounding does
  const uint32_t bits = ((uint32_t)(u >> 32) & 0x80000000u) | (((uint32_t)e << 23) + keep + up);
  if (((bits >> 23) & 0xFFu) == 0xFFu) return (float)d;  // rounded up to infinity
  return __uint_as_float(bits);
}

// Two packed BF16 (hi, lo) words of x0, x1.
__device__ __forceinline__ void pack_split(float x0, float x1, uint32_t &hw, uint32_t &lw) {
  __nv_bfloat16 h0, l0, h1, l1;
  split_bf16(x0, h0, l0);
  split_bf16(x1, h1, l1);
  hw = (uint32_t)__bfloat16_as_ushort(h0) | ((uint32_t)__bfloat16_as_ushort(h1) << 16);
  lw = (uint32_t)__bfloat16_as_ushort(l0) | ((uint32_t)__bfloat16_as_ushort(l1) << 16);
}

}  // namespace mcg
