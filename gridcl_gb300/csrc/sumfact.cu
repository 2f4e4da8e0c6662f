// Instantiations of the sum-factorised kernel (sumfact.cuh): hexahedra Q1-Q3 and quadrilaterals
// Q1-Q5, planar and embedded in 3D.
#include "eval_launch.cuh"
#include "sumfact.cuh"

namespace tlg {

namespace {

template <typename F, bool SPLIT>
cudaError_t launch_sf(int td, int gd, int n, const SfArgs& a, size_t smem, cudaStream_t s, bool* found) {
  *found = true;
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

cudaError_t launch_sumfact(int precision, int td, int gd, int n, const SfArgs& a, size_t smem, cudaStream_t s,
                           bool* found) {
  switch (precision) {
    case 4: return launch_sf<float, false>(td, gd, n, a, smem, s, found);
    case 8: return launch_sf<double, false>(td, gd, n, a, smem, s, found);
    default: return launch_sf<float, true>(td, gd, n, a, smem, s, found);
  }
}

}  // namespace tlg
