#include <mutex>
#include <unordered_map>
// FP32 instantiation of the plain transport (contraction allowed).
#include "mc_launch.h"
#include "transport_plain.cuh"

namespace mcg {

cudaError_t launch_plain_fp32(const DevGrid &g, const DevSources &s, const DevReplay &rp,
                              DevCounters *cnt, int num_sms, cudaStream_t stream) {
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, transport_plain_kernel<float>, 256, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  long long want = (s.total + 255) / 256;
  long long blocks = (long long)num_sms * per_sm;
  if (want < blocks) blocks = want < 1 ? 1 : want;
  transport_plain_kernel<float><<<(unsigned)blocks, 256, 0, stream>>>(g, s, rp, cnt);
  return cudaGetLastError();
}

}  // namespace mcg

#include "transport_wave.cuh"

namespace mcg {

static const int kGridPerSm = 4;

template <bool Replay> static cudaError_t sample_stellar_impl(const WaveLaunch &L) {
  auto k = wave_sample_stellar_kernel<float, Replay>;
  const size_t sh = (size_t)L.g.nb * (1 + L.S.nsrc) * sizeof(unsigned int);
  cudaError_t e = raise_smem_limit((const void *)k, (int)sh);
  if (e != cudaSuccess) return e;
  k<<<L.num_sms * kGridPerSm, 256, sh, L.stream>>>(L.g, L.S, L.rp, L.w, L.cnt);
  return cudaGetLastError();
}
cudaError_t launch_wave_sample_stellar_fp32(const WaveLaunch &L) {
  return L.rp.draws ? sample_stellar_impl<true>(L) : sample_stellar_impl<false>(L);
}

template <bool Replay> static cudaError_t sample_reemit_impl(const WaveLaunch &L, unsigned int n) {
  auto k = wave_sample_reemit_kernel<float, Replay>;
  const size_t sh = (size_t)L.g.nb * sizeof(unsigned int);
  cudaError_t e = raise_smem_limit((const void *)k, (int)sh);
  if (e != cudaSuccess) return e;
  const unsigned int blocks = (unsigned int)min((long long)L.num_sms * kGridPerSm, (n + 255ll) / 256 + 1);
  k<<<blocks, 256, sh, L.stream>>>(L.g, L.S, L.rp, L.w, n, L.cnt);
  return cudaGetLastError();
}
cudaError_t launch_wave_sample_reemit_fp32(const WaveLaunch &L, unsigned int n) {
  return L.rp.draws ? sample_reemit_impl<true>(L, n) : sample_reemit_impl<false>(L, n);
}

template <bool Replay> static cudaError_t emit_impl(const WaveLaunch &L, int round) {
  wave_emit_kernel<float, Replay><<<L.num_sms * kGridPerSm, 256, 0, L.stream>>>(L.g, L.S, L.rp, L.w, round, L.cnt);
  return cudaGetLastError();
}
cudaError_t launch_wave_res_inject_fp32(const WaveLaunch &L, const uint32_t *cells, const long long *prefix,
                                        int ncell) {
  wave_res_inject_kernel<float><<<L.num_sms * kGridPerSm, 256, 0, L.stream>>>(L.g, L.S, L.w, cells, prefix, ncell);
  return cudaGetLastError();
}

cudaError_t launch_wave_emit_fp32(const WaveLaunch &L, int round) {
  return L.rp.draws ? emit_impl<true>(L, round) : emit_impl<false>(L, round);
}

template <bool Dust, bool Replay> static cudaError_t march_impl(const WaveLaunch &L) {
  auto k = wave_march_kernel<float, true, Dust, Replay>;
  const size_t sh = march_smem_bytes<float>(L.g.nx, L.g.ny, L.g.nz, 256 / 32);
  cudaError_t e = raise_smem_limit((const void *)k, (int)sh);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 256, sh);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) per_sm = 1;
  k<<<L.num_sms * per_sm, 256, sh, L.stream>>>(L.g, L.S, L.rp, L.w, L.cnt);
  return cudaGetLastError();
}
template <bool Dust> static cudaError_t march_batch_blocks(size_t smem, int num_sms, int *blocks) {
  auto k = wave_march_batch_kernel<float, true, Dust>;
  cudaError_t e = raise_smem_limit((const void *)k, (int)smem);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 256, smem);
  if (e != cudaSuccess) return e;
  *blocks = num_sms * (per_sm < 1 ? 1 : per_sm);
  return cudaSuccess;
}
cudaError_t launch_wave_march_batch_blocks_fp32(bool dust, size_t smem, int num_sms, int *blocks) {
  return dust ? march_batch_blocks<true>(smem, num_sms, blocks) : march_batch_blocks<false>(smem, num_sms, blocks);
}
cudaError_t launch_wave_march_batch_fp32(const BatchLaunch &B) {
  if (B.dust)
    wave_march_batch_kernel<float, true, true><<<B.blocks, 256, B.smem, B.stream>>>(B.models, B.nmodels, B.tasks_per_pass,
                                                                                  B.task_ctr);
  else
    wave_march_batch_kernel<float, true, false><<<B.blocks, 256, B.smem, B.stream>>>(B.models, B.nmodels, B.tasks_per_pass,
                                                                                   B.task_ctr);
  return cudaGetLastError();
}
size_t march_batch_smem_fp32(int nx, int ny, int nz) { return march_smem_bytes<float>(nx, ny, nz, 256 / 32); }

cudaError_t launch_wave_march_fp32(const WaveLaunch &L) {
  const bool dust = L.g.flags & MC_FLAG_DUST;
  if (L.rp.draws) return dust ? march_impl<true, true>(L) : march_impl<false, true>(L);
  return dust ? march_impl<true, false>(L) : march_impl<false, false>(L);
}

cudaError_t raise_smem_limit(const void *func, size_t bytes) {
  static std::mutex m;
  static std::unordered_map<const void *, size_t> limits;
  std::lock_guard<std::mutex> lock(m);
  size_t &cur = limits[func];
  if (bytes <= cur) return cudaSuccess;
  const cudaError_t e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) cur = bytes;
  return e;
}

}  // namespace mcg
