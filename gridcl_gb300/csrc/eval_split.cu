// Split-precision instantiations: f64 meshes, FP32 arithmetic, f32 fields (eval.cuh).
#include "eval_launch.cuh"

namespace tlg {

cudaError_t launch_eval_split(int td, int gd, int k, const SplitArgs& a, size_t smem, cudaStream_t s,
                              bool* found) {
  *found = true;
#define TLG_SPLIT(TD, GD, K) \
  if (td == TD && gd == GD && k == K) return launch_persistent(eval_split_kernel<TD, GD, K>, a, a.padded, smem, s);
  TLG_SPLIT(3, 3, 4)
  TLG_SPLIT(3, 3, 10)
  TLG_SPLIT(3, 3, 20)
  TLG_SPLIT(3, 3, 8)
  TLG_SPLIT(3, 3, 27)
  TLG_SPLIT(3, 3, 6)
  TLG_SPLIT(3, 3, 18)
  TLG_SPLIT(2, 2, 3)
  TLG_SPLIT(2, 2, 6)
  TLG_SPLIT(2, 2, 10)
  TLG_SPLIT(2, 2, 15)
  TLG_SPLIT(2, 2, 4)
  TLG_SPLIT(2, 2, 9)
  TLG_SPLIT(2, 3, 3)
  TLG_SPLIT(2, 3, 6)
  TLG_SPLIT(2, 3, 10)
  TLG_SPLIT(2, 3, 15)
  TLG_SPLIT(2, 3, 4)
  TLG_SPLIT(2, 3, 9)
#undef TLG_SPLIT
  *found = false;
  return cudaSuccess;
}

}  // namespace tlg
