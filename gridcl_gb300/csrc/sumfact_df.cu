// Instantiations of the double-float sum-factorised kernels (sumfact_df.cuh): hexahedra Q1-Q3,
// quadrilaterals Q1-Q5 (planar and embedded in 3D), prisms P1-P3, with and without facet normals,
// and the three-lanes-per-cell hexahedra.
#include "eval_launch.cuh"
#include "sumfact_df.cuh"

namespace tlg {

template <bool FN>
static cudaError_t launch_sf_df(int td, int gd, int n, const SfArgs& a, size_t smem, cudaStream_t s, bool* found) {
  *found = true;
  if (a.prism) {
    if (n == 2) return launch_persistent(sumfact_prism_df_kernel<2, FN>, a, a.padded, smem, s);
    if (n == 3) return launch_persistent(sumfact_prism_df_kernel<3, FN>, a, a.padded, smem, s);
    if (n == 4) return launch_persistent(sumfact_prism_df_kernel<4, FN>, a, a.padded, smem, s);
    *found = false;
    return cudaSuccess;
  }
#define TLG_SFD(TD, GD, NN) \
  if (td == TD && gd == GD && n == NN) return launch_persistent(sumfact_df_kernel<TD, GD, NN, FN>, a, a.padded, smem, s);
  TLG_SFD(3, 3, 2)
  TLG_SFD(3, 3, 3)
  TLG_SFD(3, 3, 4)
  TLG_SFD(2, 2, 2)
  TLG_SFD(2, 2, 3)
  TLG_SFD(2, 2, 4)
  TLG_SFD(2, 2, 5)
  TLG_SFD(2, 2, 6)
  if constexpr (!FN) {
    TLG_SFD(2, 3, 2)
    TLG_SFD(2, 3, 3)
    TLG_SFD(2, 3, 4)
    TLG_SFD(2, 3, 5)
    TLG_SFD(2, 3, 6)
  }
#undef TLG_SFD
  *found = false;
  return cudaSuccess;
}

cudaError_t launch_sumfact_df(int td, int gd, int n, const SfArgs& a, size_t smem, cudaStream_t s, bool* found) {
  return (a.mask & kOutFacetNormals) ? launch_sf_df<true>(td, gd, n, a, smem, s, found)
                                     : launch_sf_df<false>(td, gd, n, a, smem, s, found);
}

cudaError_t launch_sumfact_df3(int n, const SfArgs& a, size_t smem, cudaStream_t s, bool* found) {
  *found = true;
  // Ten cells per warp: the persistent grid covers padded / 10 warps.
  const int64_t work = (a.padded + 9) / 10 * 32;
  // Register caps: three CTAs per SM at Q2 (168 registers; 220 without a cap ran 8.26 ms against
  // 7.34 ms on 128^3 Q2 hexahedra, 128 registers 7.27 ms with 276 bytes of spills).
  if (n == 2) return launch_persistent(sumfact_df3_kernel<2, 3>, a, work, smem, s);
  if (n == 3) return launch_persistent(sumfact_df3_kernel<3, 3>, a, work, smem, s);
  if (n == 4) return launch_persistent(sumfact_df3_kernel<4, 2>, a, work, smem, s);
  *found = false;
  return cudaSuccess;
}

}  // namespace tlg
