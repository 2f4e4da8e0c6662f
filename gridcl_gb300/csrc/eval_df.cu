// Double-float instantiations (eval_df.cuh): f64 meshes and fields, tile 16, for the elements of
// the paired kernels' list.
#include "eval_df.cuh"
#include "eval_launch.cuh"

namespace tlg {

cudaError_t launch_eval_df(int td, int gd, int k, const DfArgs& a, size_t smem, cudaStream_t s, bool* found) {
  *found = true;
  if (a.mono) {
    // The monomial form (its rows are not the nodes'): tetrahedra P1-P3 only.
#define TLG_DFM(TD, GD, K) \
  if (td == TD && gd == GD && k == K) return launch_persistent(eval_df_kernel<TD, GD, K, true>, a, a.padded, smem, s);
    TLG_DFM(3, 3, 4)
    TLG_DFM(3, 3, 10)
    TLG_DFM(3, 3, 20)
#undef TLG_DFM
    *found = false;
    return cudaSuccess;
  }
#define TLG_DFK(TD, GD, K) \
  if (td == TD && gd == GD && k == K) return launch_persistent(eval_df_kernel<TD, GD, K>, a, a.padded, smem, s);
  // Tetrahedra P1-P3, hexahedra Q1-Q2, prisms P1-P2.
  TLG_DFK(3, 3, 4)
  TLG_DFK(3, 3, 10)
  TLG_DFK(3, 3, 20)
  TLG_DFK(3, 3, 8)
  TLG_DFK(3, 3, 27)
  TLG_DFK(3, 3, 6)
  TLG_DFK(3, 3, 18)
  // Pyramids P1-P3.
  TLG_DFK(3, 3, 5)
  TLG_DFK(3, 3, 14)
  TLG_DFK(3, 3, 30)
  // Triangles P1-P4 and quadrilaterals Q1-Q2, planar and embedded in 3D.
  TLG_DFK(2, 2, 3)
  TLG_DFK(2, 2, 6)
  TLG_DFK(2, 2, 10)
  TLG_DFK(2, 2, 15)
  TLG_DFK(2, 2, 4)
  TLG_DFK(2, 2, 9)
  TLG_DFK(2, 3, 3)
  TLG_DFK(2, 3, 6)
  TLG_DFK(2, 3, 10)
  TLG_DFK(2, 3, 15)
  TLG_DFK(2, 3, 4)
  TLG_DFK(2, 3, 9)
  // Intervals P1-P2.
  TLG_DFK(1, 1, 2)
  TLG_DFK(1, 2, 2)
  TLG_DFK(1, 3, 2)
  TLG_DFK(1, 1, 3)
  TLG_DFK(1, 2, 3)
  TLG_DFK(1, 3, 3)
#undef TLG_DFK
  *found = false;
  return cudaSuccess;
}

}  // namespace tlg
