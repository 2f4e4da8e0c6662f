// Instantiations of the sum-factorised kernels (sumfact.cuh): hexahedra Q1-Q3, quadrilaterals
// Q1-Q5 (planar and embedded in 3D), prisms P1-P3, and the hexahedral adjoint.
#include <algorithm>

#include "eval_launch.cuh"
#include "sumfact.cuh"

namespace tlg {


cudaError_t launch_vjp_sumfact(bool split, int n, const VjpSfArgs& a, size_t smem, int threads, cudaStream_t s,
                               bool* found) {
  *found = true;
#define TLG_VSF(F, SPLIT, NN) \
  if (n == NN) { \
    auto kern = a.m[0] == NN ? vjp_sumfact_kernel<F, SPLIT, NN, NN> : vjp_sumfact_kernel<F, SPLIT, NN, 0>; \
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
    if (e != cudaSuccess) return e; \
    int per_sm = 0, sms = 1, dev = 0; \
    cudaGetDevice(&dev); \
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev); \
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem) != cudaSuccess || per_sm < 1) \
      per_sm = 1; \
    const int64_t need = (a.padded + threads - 1) / threads; \
    const int grid = (int)std::min<int64_t>(need, (int64_t)sms * per_sm); \
    kern<<<grid > 0 ? grid : 1, threads, smem, s>>>(a); \
    return cudaGetLastError(); \
  }
  if (split) {
    TLG_VSF(float, true, 2)
    TLG_VSF(float, true, 3)
  } else {
    TLG_VSF(double, false, 2)
    TLG_VSF(double, false, 3)
  }
#undef TLG_VSF
  *found = false;
  return cudaSuccess;
}

cudaError_t launch_vjp_sumfact_bwd(bool split, int n, const VjpSfArgs& a, size_t smem, int threads, cudaStream_t s,
                                   bool* found) {
  *found = true;
#define TLG_VSB(F, NN) \
  if (n == NN) { \
    auto kern = a.m[0] == NN ? vjp_sumfact_bwd_kernel<F, NN, NN> : vjp_sumfact_bwd_kernel<F, NN, 0>; \
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
    if (e != cudaSuccess) return e; \
    const int grid = persistent_grid(kern, smem, a.padded, threads); \
    kern<<<grid, threads, smem, s>>>(a); \
    return cudaGetLastError(); \
  }
  if (split) {
    TLG_VSB(float, 2)
    TLG_VSB(float, 3)
  } else {
    TLG_VSB(double, 2)
    TLG_VSB(double, 3)
  }
#undef TLG_VSB
  *found = false;
  return cudaSuccess;
}

cudaError_t launch_vjp_sumfact_tile(bool split, int n, const VjpSfArgs& a, size_t smem, cudaStream_t s, bool* found) {
  *found = true;
  const bool cube = a.m[0] == a.m[1] && a.m[1] == a.m[2];
#define TLG_VST(F, NN, MM) \
  if (n == NN && (MM == 0 || (cube && a.m[0] == MM))) { \
    auto kern = vjp_sumfact_tile_kernel<F, NN, MM>; \
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
    if (e != cudaSuccess) return e; \
    const int grid = persistent_grid(kern, smem, a.padded / 16 * kTileBwdThreads, kTileBwdThreads); \
    kern<<<grid, kTileBwdThreads, smem, s>>>(a); \
    return cudaGetLastError(); \
  }
  if (split) {
    TLG_VST(float, 2, 2)
    TLG_VST(float, 3, 3)
    TLG_VST(float, 2, 0)
    TLG_VST(float, 3, 0)
  } else {
    TLG_VST(double, 2, 2)
    TLG_VST(double, 3, 3)
    TLG_VST(double, 2, 0)
    TLG_VST(double, 3, 0)
  }
#undef TLG_VST
  *found = false;
  return cudaSuccess;
}

cudaError_t launch_sumfact(int precision, int td, int gd, int n, const SfArgs& a, size_t smem, cudaStream_t s,
                           bool* found) {
  if (a.mask & kOutFacetNormals) return launch_sumfact_fn(precision, td, gd, n, a, smem, s, found);
  switch (precision) {
    case 4: return launch_sf<float, false, false>(td, gd, n, a, smem, s, found);
    case 8: return launch_sf<double, false, false>(td, gd, n, a, smem, s, found);
    default: return launch_sf<float, true, false>(td, gd, n, a, smem, s, found);
  }
}

}  // namespace tlg
