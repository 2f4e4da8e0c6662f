// Instantiations of the cooperative kernel (coop.cuh): cells of 2 or 3 dimensions in f32, f64 and
// split precision, up to 16, 32, 64 or 128 nodes per cell (4, 8, 16 or 32 per lane; f64 up to 64).
#include "coop.cuh"
#include "eval_launch.cuh"

namespace tlg {

namespace {

template <typename F, bool SPLIT, int TD, int GD>
cudaError_t launch_coop_k(int k, const CoopArgs& a, size_t smem, cudaStream_t s, bool* found) {
  *found = true;
  const int64_t work = a.padded * kCoopLanes;
  const size_t dyn = a.tab_global ? 0 : smem;
  if (k <= 4 * 4) return launch_persistent(coop_kernel<F, SPLIT, TD, GD, 4>, a, work, dyn, s);
  if (k <= 4 * 8) return launch_persistent(coop_kernel<F, SPLIT, TD, GD, 8>, a, work, dyn, s);
  if (k <= 4 * 16) return launch_persistent(coop_kernel<F, SPLIT, TD, GD, 16>, a, work, dyn, s);
  if constexpr (sizeof(F) == 4) {  // f64 coordinates of 32 nodes per lane do not fit the registers
    if (k <= 4 * 32) return launch_persistent(coop_kernel<F, SPLIT, TD, GD, 32>, a, work, dyn, s);
  }
  *found = false;
  return cudaSuccess;
}

template <typename F, bool SPLIT>
cudaError_t launch_coop_t(int td, int gd, int k, const CoopArgs& a, size_t smem, cudaStream_t s, bool* found) {
  if (td == 3 && gd == 3) return launch_coop_k<F, SPLIT, 3, 3>(k, a, smem, s, found);
  if (td == 2 && gd == 2) return launch_coop_k<F, SPLIT, 2, 2>(k, a, smem, s, found);
  if (td == 2 && gd == 3) return launch_coop_k<F, SPLIT, 2, 3>(k, a, smem, s, found);
  *found = false;
  return cudaSuccess;
}

}  // namespace

cudaError_t launch_coop(int precision, int td, int gd, int k, const CoopArgs& a, size_t smem, cudaStream_t s,
                        bool* found) {
  switch (precision) {
    case 4: return launch_coop_t<float, false>(td, gd, k, a, smem, s, found);
    case 8: return launch_coop_t<double, false>(td, gd, k, a, smem, s, found);
    default: return launch_coop_t<float, true>(td, gd, k, a, smem, s, found);
  }
}

}  // namespace tlg
