// cellupdate_fp32.cu -- the FP32 instantiation of the cell-update kernel
// (the reference's own updateCell arithmetic is 4-byte `real`); compiled
// with the default contraction into FMA.
#include "cellupdate.cuh"

namespace mcg {

// the level-population matrices of a block's warps in shared memory
cudaError_t launch_cell_update_fp32(const UpdArgs &a, int blocks, cudaStream_t stream) {
  const size_t smem = (size_t)kW * a.ncel * a.mat_stride * sizeof(float);
  cudaError_t e = cudaFuncSetAttribute(cell_update_kernel<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  cell_update_kernel<float, true><<<blocks, kW * 32, smem, stream>>>(a);
  return cudaGetLastError();
}

}  // namespace mcg
