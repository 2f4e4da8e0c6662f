// The sum-factorised kernels with facet normals among their outputs (sumfact.cuh), for facet
// rules on quadrilaterals, hexahedra and prisms: a separate translation unit so that the two sets
// of instantiations compile in parallel.
#include "eval_launch.cuh"
#include "sumfact.cuh"

namespace tlg {

cudaError_t launch_sumfact_fn(int precision, int td, int gd, int n, const SfArgs& a, size_t smem, cudaStream_t s,
                              bool* found) {
  switch (precision) {
    case 4: return launch_sf<float, false, true>(td, gd, n, a, smem, s, found);
    case 8: return launch_sf<double, false, true>(td, gd, n, a, smem, s, found);
    default: return launch_sf<float, true, true>(td, gd, n, a, smem, s, found);
  }
}

}  // namespace tlg
