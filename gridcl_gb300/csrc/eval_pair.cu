// Paired-FP32 instantiations (eval.cuh): f32 meshes and split precision, tile 16.
#include "eval_launch.cuh"

namespace tlg {

template <bool SPLIT>
static cudaError_t launch_pair(int td, int gd, int k, const PairArgs& a, size_t smem, cudaStream_t s,
                               bool* found) {
  *found = true;
#define TLG_PAIR(TD, GD, K) \
  if (td == TD && gd == GD && k == K) return launch_persistent(eval_pair_kernel<SPLIT, TD, GD, K>, a, a.padded, smem, s);
  // Tetrahedra P1-P3, hexahedra Q1-Q2, prisms P1-P2.
  TLG_PAIR(3, 3, 4)
  TLG_PAIR(3, 3, 10)
  TLG_PAIR(3, 3, 20)
  TLG_PAIR(3, 3, 8)
  TLG_PAIR(3, 3, 27)
  TLG_PAIR(3, 3, 6)
  TLG_PAIR(3, 3, 18)
  // Triangles P1-P4 and quadrilaterals Q1-Q2, planar and embedded in 3D.
  TLG_PAIR(2, 2, 3)
  TLG_PAIR(2, 2, 6)
  TLG_PAIR(2, 2, 10)
  TLG_PAIR(2, 2, 15)
  TLG_PAIR(2, 2, 4)
  TLG_PAIR(2, 2, 9)
  TLG_PAIR(2, 3, 3)
  TLG_PAIR(2, 3, 6)
  TLG_PAIR(2, 3, 10)
  TLG_PAIR(2, 3, 15)
  TLG_PAIR(2, 3, 4)
  TLG_PAIR(2, 3, 9)
#undef TLG_PAIR
  *found = false;
  return cudaSuccess;
}

cudaError_t launch_eval_pair(bool split, int td, int gd, int k, const PairArgs& a, size_t smem,
                             cudaStream_t s, bool* found) {
  return split ? launch_pair<true>(td, gd, k, a, smem, s, found)
               : launch_pair<false>(td, gd, k, a, smem, s, found);
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
