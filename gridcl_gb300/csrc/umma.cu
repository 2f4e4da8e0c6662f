// Instantiations of the tcgen05 evaluation kernel (umma.cuh): f32 meshes and split precision.
#include <algorithm>

#include "eval_launch.cuh"
#include "umma.cuh"

namespace tlg {

constexpr int kMaxItemsPerTile = kUmmaMaxGroups;

// Work items: with T tiles on a grid of C resident CTAs, each tile's n chunks go in G groups
// (G <= 8) minimising ceil(T G / C) (ceil(n / G) + 10): the rounds of items times an item's
// chunks plus its start (the gather and the first chunk's copy and MMAs, not overlapped with an
// epilogue: about ten chunks in GB300 timings of P4-P6 tetrahedra), so that a few tiles more than
// CTAs do not leave most SMs idle for a second round of whole tiles.
cudaError_t launch_umma(bool split, const UmmaArgs& args, size_t smem, cudaStream_t s) {
  auto kern = split ? umma_eval_kernel<true> : umma_eval_kernel<false>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  UmmaArgs a = args;
  const int64_t tiles = (a.padded + kUmmaCells - 1) / kUmmaCells;
  const int64_t ctas = persistent_grid(kern, smem, tiles * kMaxItemsPerTile * kUmmaThreads, kUmmaThreads);
  int64_t best = -1;
  for (int g = 1; g <= kUmmaMaxGroups && g <= a.chunks; ++g) {
    const int64_t per = (a.chunks + g - 1) / g;
    const int64_t cost = ((tiles * g + ctas - 1) / ctas) * (per + 10);
    if (best < 0 || cost < best) {
      best = cost;
      a.groups = g;
      a.per_group = (int)per;
    }
  }
  const int64_t grid = std::min<int64_t>(ctas, tiles * a.groups);
  kern<<<(unsigned)std::max<int64_t>(grid, 1), kUmmaThreads, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace tlg
