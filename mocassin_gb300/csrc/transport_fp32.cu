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
