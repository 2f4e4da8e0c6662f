// Instantiations of the sum-factorised kernels (sumfact.cuh): hexahedra Q1-Q3, quadrilaterals
// Q1-Q5 (planar and embedded in 3D), prisms P1-P3, and the hexahedral adjoint.
#include <algorithm>

#include "eval_launch.cuh"
#include "sumfact.cuh"

namespace tlg {

namespace {

template <typename F, bool SPLIT>
cudaError_t launch_sf(int td, int gd, int n, const SfArgs& a, size_t smem, cudaStream_t s, bool* found) {
  *found = true;
  if (a.prism) {
    if (n == 2) return launch_persistent(sumfact_prism_kernel<F, SPLIT, 2>, a, a.padded, smem, s);
    if (n == 3) return launch_persistent(sumfact_prism_kernel<F, SPLIT, 3>, a, a.padded, smem, s);
    if (n == 4) return launch_persistent(sumfact_prism_kernel<F, SPLIT, 4>, a, a.padded, smem, s);
    *found = false;
    return cudaSuccess;
  }
#define TLG_SF(TD, GD, NN) \
  if (td == TD && gd == GD && n == NN) \
    return launch_persistent(sumfact_kernel<F, SPLIT, TD, GD, NN>, a, a.padded, smem, s);
  TLG_SF(3, 3, 2)
  TLG_SF(3, 3, 3)
  TLG_SF(3, 3, 4)
  TLG_SF(2, 2, 2)
  TLG_SF(2, 2, 3)
  TLG_SF(2, 2, 4)
  TLG_SF(2, 2, 5)
  TLG_SF(2, 2, 6)
  TLG_SF(2, 3, 2)
  TLG_SF(2, 3, 3)
  TLG_SF(2, 3, 4)
  TLG_SF(2, 3, 5)
  TLG_SF(2, 3, 6)
#undef TLG_SF
  *found = false;
  return cudaSuccess;
}

}  // namespace

cudaError_t launch_vjp_sumfact(bool split, int n, const VjpSfArgs& a, size_t smem, int threads, cudaStream_t s,
                               bool* found) {
  *found = true;
#define TLG_VSF(F, SPLIT, NN) \
  if (n == NN) { \
    auto kern = vjp_sumfact_kernel<F, SPLIT, NN>; \
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

cudaError_t launch_sumfact(int precision, int td, int gd, int n, const SfArgs& a, size_t smem, cudaStream_t s,
                           bool* found) {
  switch (precision) {
    case 4: return launch_sf<float, false>(td, gd, n, a, smem, s, found);
    case 8: return launch_sf<double, false>(td, gd, n, a, smem, s, found);
    default: return launch_sf<float, true>(td, gd, n, a, smem, s, found);
  }
}

}  // namespace tlg
