// Paired-FP32 instantiations that also sum each cell's det J * w as they evaluate
// (PairArgs::cell_measure); a translation unit of their own so that the build compiles them in
// parallel with the plain ones.
#include "pair_list.cuh"

namespace tlg {

cudaError_t launch_eval_pair_meas(bool split, int td, int gd, int k, const PairArgs& a, size_t smem,
                                  cudaStream_t s, bool* found) {
  return split ? launch_pair<true, true>(td, gd, k, a, smem, s, found)
               : launch_pair<false, true>(td, gd, k, a, smem, s, found);
}

}  // namespace tlg
