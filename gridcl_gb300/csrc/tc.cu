// Instantiations of the tensor-core evaluation kernel (tc.cuh): cells of 2 or 3 dimensions, f32
// meshes and split precision.
#include "eval_launch.cuh"
#include "tc.cuh"

namespace tlg {

cudaError_t launch_tc(bool split, int td, int gd, const TcArgs& a, size_t smem, cudaStream_t s, bool* found) {
  *found = true;
  const int64_t warps = a.padded / 16;
#define TLG_TC(SPLIT, TD, GD) \
  if (split == SPLIT && td == TD && gd == GD) { \
    auto kern = tc_eval_kernel<SPLIT, TD, GD>; \
    if (smem > 48 * 1024) { \
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
      if (e != cudaSuccess) return e; \
    } \
    const int grid = persistent_grid(kern, smem, warps * 32, kTcWarps * 32); \
    kern<<<grid, kTcWarps * 32, smem, s>>>(a); \
    return cudaGetLastError(); \
  }
  TLG_TC(true, 3, 3)
  TLG_TC(true, 2, 2)
  TLG_TC(true, 2, 3)
  TLG_TC(false, 3, 3)
  TLG_TC(false, 2, 2)
  TLG_TC(false, 2, 3)
#undef TLG_TC
  *found = false;
  return cudaSuccess;
}

}  // namespace tlg
