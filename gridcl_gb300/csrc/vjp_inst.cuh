// Instantiations of vjp_kernel for one mode (included by vjp_f64.cu and vjp_split.cu with
// TLG_VJP_SPLIT and TLG_VJP_LAUNCH defined).
#include "eval_launch.cuh"
#include "vjp.cuh"

namespace tlg {

cudaError_t TLG_VJP_LAUNCH(int d, int k, const VjpArgs& a, size_t smem, cudaStream_t s, bool* found) {
  *found = true;
#define TLG_VJP(D, K) \
  if (d == D && k == K) { \
    auto kern = vjp_kernel<TLG_VJP_SPLIT, D, K>; \
    if (smem > 48 * 1024) { \
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
      if (e != cudaSuccess) return e; \
    } \
    const int grid = persistent_grid(kern, smem, a.padded * kVjpGroup, kEvalThreads); \
    kern<<<grid, kEvalThreads, smem, s>>>(a); \
    return cudaGetLastError(); \
  }
  TLG_VJP(3, 4)
  TLG_VJP(3, 10)
  TLG_VJP(3, 20)
  TLG_VJP(3, 8)
  TLG_VJP(3, 27)
  TLG_VJP(3, 6)
  TLG_VJP(3, 18)
  TLG_VJP(3, 5)
  TLG_VJP(3, 14)
  TLG_VJP(3, 30)
  TLG_VJP(2, 3)
  TLG_VJP(2, 6)
  TLG_VJP(2, 10)
  TLG_VJP(2, 15)
  TLG_VJP(2, 4)
  TLG_VJP(2, 9)
#undef TLG_VJP
  *found = false;
  return cudaSuccess;
}

}  // namespace tlg
