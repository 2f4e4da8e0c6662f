// The paired-FP32 kernels' (element, precision) list, shared by the translation units that
// instantiate them (eval_pair.cu: plain; eval_pair_meas.cu: with the per-cell measure).
#pragma once
#include "eval_launch.cuh"

namespace tlg {

template <bool SPLIT, bool MEAS>
static cudaError_t launch_pair(int td, int gd, int k, const PairArgs& a, size_t smem, cudaStream_t s,
                               bool* found) {
  *found = true;
#define TLG_PAIR(TD, GD, K) \
  if (td == TD && gd == GD && k == K) return launch_persistent(eval_pair_kernel<SPLIT, TD, GD, K, MEAS>, a, a.padded, smem, s);
  // Tetrahedra P1-P3, hexahedra Q1-Q2, prisms P1-P2.
  TLG_PAIR(3, 3, 4)
  TLG_PAIR(3, 3, 10)
  TLG_PAIR(3, 3, 20)
  TLG_PAIR(3, 3, 8)
  TLG_PAIR(3, 3, 27)
  TLG_PAIR(3, 3, 6)
  TLG_PAIR(3, 3, 18)
  // Pyramids P1-P3.
  TLG_PAIR(3, 3, 5)
  TLG_PAIR(3, 3, 14)
  TLG_PAIR(3, 3, 30)
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

}  // namespace tlg
