// Instantiations of the tcgen05 evaluation kernel (umma.cuh): f32 meshes and split precision.
#include "eval_launch.cuh"
#include "umma.cuh"

namespace tlg {

cudaError_t launch_umma(bool split, const UmmaArgs& a, size_t smem, cudaStream_t s) {
  auto kern = split ? umma_eval_kernel<true> : umma_eval_kernel<false>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int64_t tiles = (a.padded + kUmmaCells - 1) / kUmmaCells;
  const int grid = persistent_grid(kern, smem, tiles * kUmmaThreads, kUmmaThreads);
  kern<<<grid, kUmmaThreads, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace tlg
