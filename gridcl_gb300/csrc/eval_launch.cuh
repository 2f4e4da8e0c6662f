// Launch helpers of the evaluation kernels: persistent grid sizing and the dispatch from run-time
// (TD, GD, K) to the compiled instantiations.
#pragma once

#include <cuda_runtime.h>

#include "eval.cuh"

namespace tlg {

// A grid size chosen by the batch autotuner for the next launches on this thread (0: none).
inline thread_local int g_grid_override = 0;

// Grid of persistent CTAs: enough to cover the range, at most the resident CTAs of the device
// (or the autotuner's choice).
template <typename Kernel>
inline int persistent_grid(Kernel kern, size_t smem, int64_t work_items, int threads) {
  if (g_grid_override > 0) return g_grid_override;
  static thread_local int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  // Resident CTAs per SM, queried once per (kernel, shared memory, threads) on this thread.
  struct Entry {
    const void* kern;
    size_t smem;
    int threads, per_sm;
  };
  static thread_local Entry cache[64];
  static thread_local int cached = 0;
  int per_sm = 0;
  for (int i = 0; i < cached; ++i)
    if (cache[i].kern == (const void*)kern && cache[i].smem == smem && cache[i].threads == threads) {
      per_sm = cache[i].per_sm;
      break;
    }
  if (per_sm == 0) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem) != cudaSuccess ||
        per_sm < 1)
      per_sm = 1;
    cache[cached % 64] = {(const void*)kern, smem, threads, per_sm};
    if (cached < 64) ++cached;
  }
  const int64_t need = (work_items + threads - 1) / threads;
  const int64_t cap = (int64_t)sms * per_sm;
  return (int)(need < cap ? (need > 0 ? need : 1) : cap);
}

template <typename Kernel, typename Args>
inline cudaError_t launch_persistent(Kernel kern, const Args& a, int64_t work, size_t smem,
                                     cudaStream_t s) {
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  const int grid = persistent_grid(kern, smem, work, kEvalThreads);
  kern<<<grid, kEvalThreads, smem, s>>>(a);
  return cudaGetLastError();
}

// Defined in eval_f32.cu / eval_f64.cu. `direct` receives whether an unrolled kernel ran.
cudaError_t launch_eval_f32(int td, int gd, int k, const EvalArgs<float>& a, size_t smem,
                            cudaStream_t s, bool* direct);
cudaError_t launch_eval_f64(int td, int gd, int k, const EvalArgs<double>& a, size_t smem,
                            cudaStream_t s, bool* direct);
// Defined in eval_pair.cu: the paired-FP32 kernel for an f32 mesh (split = false) or split
// precision (split = true), tile 16; `found` is false when none exists for (td, gd, k).
cudaError_t launch_eval_pair(bool split, int td, int gd, int k, const PairArgs& a, size_t smem,
                             cudaStream_t s, bool* found);
// Defined in eval_pair_meas.cu: the same kernels summing each cell's det J * w into
// a.cell_measure (a.weights [Q]) as they evaluate.
cudaError_t launch_eval_pair_meas(bool split, int td, int gd, int k, const PairArgs& a, size_t smem,
                                  cudaStream_t s, bool* found);
// Defined in eval_pair.cu: split precision with K at run time (tile 16), tables staged in
// shared memory or (tab_global) read from global memory.
cudaError_t launch_split_loops(int td, int gd, bool tab_global, const PairArgs& a, size_t smem, cudaStream_t s);

struct DfArgs;
// Defined in eval_df.cu: the double-float kernel (f64 mesh and fields) for (td, gd, k), tile 16;
// `found` is false when none is compiled.
cudaError_t launch_eval_df(int td, int gd, int k, const DfArgs& a, size_t smem, cudaStream_t s, bool* found);

struct SfArgs;
struct VjpSfArgs;
// Defined in sumfact.cu: the sum-factorised adjoint of hexahedra (split: f32 arithmetic, else f64),
// N nodes per direction, `threads` per CTA; `found` is false when none is compiled for n.
cudaError_t launch_vjp_sumfact(bool split, int n, const VjpSfArgs& a, size_t smem, int threads, cudaStream_t s,
                               bool* found);
// Defined in sumfact.cu: the same adjoint from forward fields already written (det J and K read
// back, vjp_sumfact_bwd_kernel).
cudaError_t launch_vjp_sumfact_bwd(bool split, int n, const VjpSfArgs& a, size_t smem, int threads, cudaStream_t s,
                                   bool* found);
// Defined in sumfact.cu: the same with a 16-cell tile spread over the CTA (vjp_sumfact_tile_kernel;
// kTileBwdThreads threads; work over a.padded / 16 tiles).
cudaError_t launch_vjp_sumfact_tile(bool split, int n, const VjpSfArgs& a, size_t smem, cudaStream_t s, bool* found);
// Defined in sumfact.cu: the sum-factorised kernel for precision 4 (f32), 8 (f64) or 12 (split),
// N nodes per direction; `found` is false when none is compiled for (td, gd, n).
cudaError_t launch_sumfact(int precision, int td, int gd, int n, const SfArgs& a, size_t smem, cudaStream_t s,
                           bool* found);
// Defined in sumfact_df.cu: the double-float sum-factorised kernels (f64 mesh and fields, tile 16;
// a.tab the tables' double-float section), and those of hexahedra with three lanes per cell (no
// facet normals; smem: the section and sumfact_df3_slot_bytes).
cudaError_t launch_sumfact_df(int td, int gd, int n, const SfArgs& a, size_t smem, cudaStream_t s, bool* found);
cudaError_t launch_sumfact_df3(int n, const SfArgs& a, size_t smem, cudaStream_t s, bool* found);
// Defined in sumfact_fn.cu: the same with facet normals among the outputs (codimension 0).
cudaError_t launch_sumfact_fn(int precision, int td, int gd, int n, const SfArgs& a, size_t smem, cudaStream_t s,
                              bool* found);

struct TcArgs;
// Defined in tc.cu: the tensor-core kernel (split: f64 mesh, else f32 mesh), TD >= 2, tile 16.
cudaError_t launch_tc(bool split, int td, int gd, const TcArgs& a, size_t smem, cudaStream_t s, bool* found);

struct CoopArgs;
// Defined in coop.cu: the cooperative kernel (four lanes per cell) for precision 4, 8 or 12, cells of
// 2 or 3 dimensions and at most 128 nodes; `found` is false otherwise.
cudaError_t launch_coop(int precision, int td, int gd, int k, const CoopArgs& a, size_t smem, cudaStream_t s,
                        bool* found);

struct VjpArgs;
struct VjpSurfArgs;
// Defined in vjp_surface.cu: the adjoint below codimension 0 (TD < GD), `threads` per CTA.
cudaError_t launch_vjp_surface(bool split, int td, int gd, const VjpSurfArgs& a, size_t smem, int threads,
                               cudaStream_t s, bool* found);
// Defined in vjp_f64.cu / vjp_split.cu; `found` is false when no kernel exists for (d, k). `smem`
// is the dynamic shared memory: the staged tables (rounded up to 16 bytes) and the staging slots.
cudaError_t launch_vjp_f64(int d, int k, const VjpArgs& a, size_t smem, cudaStream_t s, bool* found);
cudaError_t launch_vjp_split(int d, int k, const VjpArgs& a, size_t smem, cudaStream_t s, bool* found);
cudaError_t launch_vjp_gather(const uint32_t* offsets, const uint32_t* entries, int64_t num_nodes, int d,
                              const void* local, int local_dtype, double* grad, cudaStream_t s, bool add = false);
// Defined in vjp_split.cu: the adjoint from det J and K fields for volume cells of any kind
// (vjp_tile_kernel; a.k_runtime = K, the group and CTA sizes from vjp_tile_shape; smem: the node rows, then 12 * 16 values per point).
cudaError_t launch_vjp_tile(bool split, const VjpArgs& a, size_t smem, cudaStream_t s);
struct GatherBlocks;
// Defined in vjp_split.cu: the node sums of up to kGatherMaxBlocks blocks in one pass
// (vjp_gather_blocks_kernel), rows of one dtype.
cudaError_t launch_vjp_gather_blocks(const GatherBlocks& gb, int64_t num_nodes, int d, int local_dtype, double* grad,
                                     cudaStream_t s, bool add);

}  // namespace tlg
