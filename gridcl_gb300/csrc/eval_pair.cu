// Paired-FP32 instantiations (eval.cuh): f32 meshes and split precision, tile 16.
#include "pair_list.cuh"

namespace tlg {

cudaError_t launch_eval_pair(bool split, int td, int gd, int k, const PairArgs& a, size_t smem,
                             cudaStream_t s, bool* found) {
  return split ? launch_pair<true, false>(td, gd, k, a, smem, s, found)
               : launch_pair<false, false>(td, gd, k, a, smem, s, found);
}

cudaError_t launch_split_loops(int td, int gd, bool tab_global, const PairArgs& a, size_t smem, cudaStream_t s) {
#define TLG_SPLIT_LOOPS(TD, GD) \
  if (td == TD && gd == GD) \
    return tab_global ? launch_persistent(split_loops_kernel<TD, GD, true>, a, a.padded, 0, s) \
                      : launch_persistent(split_loops_kernel<TD, GD, false>, a, a.padded, smem, s);
  TLG_SPLIT_LOOPS(1, 1)
  TLG_SPLIT_LOOPS(1, 2)
  TLG_SPLIT_LOOPS(1, 3)
  TLG_SPLIT_LOOPS(2, 2)
  TLG_SPLIT_LOOPS(2, 3)
  TLG_SPLIT_LOOPS(3, 3)
#undef TLG_SPLIT_LOOPS
  return cudaErrorInvalidValue;
}

}  // namespace tlg
