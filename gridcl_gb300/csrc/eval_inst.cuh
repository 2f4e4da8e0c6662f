// Instantiation list of the scalar evaluation kernels for one scalar type (included by
// eval_f32.cu and eval_f64.cu with TLG_F and TLG_LAUNCH defined). Unrolled direct kernels exist
// for f64 at the elements of the benchmark meshes and the low degrees (f32 at tile 16 runs the
// paired kernel of eval_pair.cu); every other (TD, GD, K, tile) runs the loops kernel.
#include "eval_launch.cuh"

namespace tlg {

cudaError_t TLG_LAUNCH(int td, int gd, int k, const EvalArgs<TLG_F>& a, size_t smem,
                       cudaStream_t s, bool* direct) {
#ifdef TLG_WITH_DIRECT
  // Unrolled kernels are compiled for f64 and the GPU tile of 16 cells; they read staged tables
  // (the host clears loops_only only when the tables are staged).
  *direct = a.tile_shift == 4 && !a.loops_only;
#define TLG_DIRECT(TD, GD, K) \
  if (*direct && td == TD && gd == GD && k == K) \
    return launch_persistent(eval_direct_kernel<TLG_F, TD, GD, K, 16>, a, a.padded, smem, s);
  // Tetrahedra P1-P3, hexahedra Q1-Q2, prisms P1-P2.
  TLG_DIRECT(3, 3, 4)
  TLG_DIRECT(3, 3, 10)
  TLG_DIRECT(3, 3, 20)
  TLG_DIRECT(3, 3, 8)
  TLG_DIRECT(3, 3, 27)
  TLG_DIRECT(3, 3, 6)
  TLG_DIRECT(3, 3, 18)
  // Pyramids P1-P3.
  TLG_DIRECT(3, 3, 5)
  TLG_DIRECT(3, 3, 14)
  TLG_DIRECT(3, 3, 30)
  // Triangles P1-P4 and quadrilaterals Q1-Q2, planar and embedded in 3D.
  TLG_DIRECT(2, 2, 3)
  TLG_DIRECT(2, 2, 6)
  TLG_DIRECT(2, 2, 10)
  TLG_DIRECT(2, 2, 15)
  TLG_DIRECT(2, 2, 4)
  TLG_DIRECT(2, 2, 9)
  TLG_DIRECT(2, 3, 3)
  TLG_DIRECT(2, 3, 6)
  TLG_DIRECT(2, 3, 10)
  TLG_DIRECT(2, 3, 15)
  TLG_DIRECT(2, 3, 4)
  TLG_DIRECT(2, 3, 9)
  // Intervals P1-P2.
  TLG_DIRECT(1, 1, 2)
  TLG_DIRECT(1, 2, 2)
  TLG_DIRECT(1, 3, 2)
  TLG_DIRECT(1, 1, 3)
  TLG_DIRECT(1, 2, 3)
  TLG_DIRECT(1, 3, 3)
#undef TLG_DIRECT
#endif
  *direct = false;
#define TLG_LOOPS(TD, GD) \
  if (td == TD && gd == GD) \
    return a.tab_global ? launch_persistent(eval_loops_kernel<TLG_F, TD, GD, true>, a, a.padded, 0, s) \
                        : launch_persistent(eval_loops_kernel<TLG_F, TD, GD, false>, a, a.padded, smem, s);
  TLG_LOOPS(1, 1)
  TLG_LOOPS(1, 2)
  TLG_LOOPS(1, 3)
  TLG_LOOPS(2, 2)
  TLG_LOOPS(2, 3)
  TLG_LOOPS(3, 3)
#undef TLG_LOOPS
  return cudaErrorInvalidValue;
}

}  // namespace tlg
