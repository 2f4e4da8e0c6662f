// Measure of a block: per-cell sums of det J * w over the points, then sums of 64 consecutive
// values, level by level, down to one value (tetraloma-geometry/src/measure.rs:15-102). Each
// value is summed in F in a fixed order, so the result is the same on every run and for every
// grid shape.
#include <cstdint>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "../../include/tlgeom.h"
#include "convert.cuh"
#include "status.h"

namespace tlg {

constexpr int kSumBlock = 64;  // measure.rs:44

// det J * w summed over the points of one cell, in point order: d0*w0, then fma(d_q, w_q, acc).
// The loads are issued eight at a time ahead of the fma chain, so that each thread keeps several
// reads in flight; the order of the arithmetic does not depend on that.
template <typename F>
__device__ __forceinline__ F cell_sum(const F* __restrict__ detj, const F* __restrict__ weights,
                                      int64_t base, int num_points, int tile_shift) {
  constexpr int U = 8;
  F acc = F(0);
  for (int q0 = 0; q0 < num_points; q0 += U) {
    F v[U];
#pragma unroll
    for (int u = 0; u < U; ++u)
      v[u] = q0 + u < num_points ? __ldg(detj + base + ((int64_t)(q0 + u) << tile_shift)) : F(0);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int q = q0 + u;
      if (q < num_points) acc = q == 0 ? v[u] * __ldg(weights) : fma(v[u], __ldg(weights + q), acc);
    }
  }
  return acc;
}

template <typename F>
__global__ void __launch_bounds__(256) cell_sums_kernel(const F* detj, const F* weights, F* out,
                                                        int64_t num_cells, int num_points,
                                                        int tile_shift) {
  const int64_t mask = (1 << tile_shift) - 1;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < num_cells;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t base = (((c >> tile_shift) * num_points) << tile_shift) + (c & mask);
    out[c] = cell_sum(detj, weights, base, num_points, tile_shift);
  }
}

// Left fold ((v0 + v1) + v2) + ... of the `count` <= 64 values a warp holds two per lane (lane l:
// v[l] in lo, v[32 + l] in hi); every lane gets the result. The shuffles do not depend on the
// running sum, so they issue ahead of the chain of adds.
template <typename F>
__device__ __forceinline__ F warp_fold(F lo, F hi, int count) {
  F acc = __shfl_sync(0xffffffffu, lo, 0);
#pragma unroll
  for (int j = 1; j < 32; ++j) {
    const F v = __shfl_sync(0xffffffffu, lo, j);
    if (j < count) acc += v;
  }
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    const F v = __shfl_sync(0xffffffffu, hi, j);
    if (32 + j < count) acc += v;
  }
  return acc;
}

// One level of the tree: out[i] = x[64 i] + ... + x[64 i + 63] (fewer at the end), summed in that
// order. One warp per output: two coalesced loads, then the fold.
template <typename F>
__global__ void __launch_bounds__(256) block_sum_kernel(const F* x, F* out, int64_t len, int64_t num_out) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < num_out; i += warps) {
    const int64_t start = i * kSumBlock;
    const int count = (int)(len - start < kSumBlock ? len - start : kSumBlock);
    const F lo = lane < count ? x[start + lane] : F(0);
    const F hi = 32 + lane < count ? x[start + 32 + lane] : F(0);
    const F acc = warp_fold(lo, hi, count);
    if (lane == 0) out[i] = acc;
  }
}

inline unsigned grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > 152 * 64) b = 152 * 64;
  return (unsigned)b;
}

// Elements of the level buffers of a tree over n values: ceil(n/64) + ceil(n/64^2) + ... down
// to one value.
inline int64_t tree_elems(int64_t n) {
  int64_t total = 0;
  while (n > 1) {
    n = (n + kSumBlock - 1) / kSumBlock;
    total += n;
  }
  return total;
}

template <typename F>
cudaError_t sum_tree(const F* x, int64_t n, F* work, F* result, cudaStream_t s) {
  if (n == 1) return cudaMemcpyAsync(result, x, sizeof(F), cudaMemcpyDeviceToDevice, s);
  const F* cur = x;
  F* next = work;
  while (n > 1) {
    const int64_t m = (n + kSumBlock - 1) / kSumBlock;
    F* dst = m == 1 ? result : next;
    block_sum_kernel<F><<<grid_for(m * 32, 256), 256, 0, s>>>(cur, dst, n, m);
    cur = dst;
    next = dst + m;
    n = m;
  }
  return cudaGetLastError();
}

// ----------------------------------------------------------------------------------------
// Measure without any allocation: the sum-tree levels live in a fixed device array of this
// library. Level 1 (sums of 64 consecutive cell sums) is produced directly from the det J
// field, in the order cell_sums_kernel followed by block_sum_kernel would use, so the result is
// the same bits as the allocating path.

constexpr int64_t kStaticMaxCells = int64_t(1) << 24;  // 16,777,216 cells
// tree_elems(kStaticMaxCells) = 262144 + 4096 + 64 + 1 values, rounded up to a multiple of 64.
constexpr int64_t kStaticScratchElems = 266368;
static __device__ __align__(256) double g_measure_scratch[kStaticScratchElems];  // 2,130,944 bytes

// Level 1 straight from det J: one warp per 64 consecutive cells, lane l summing cells l and
// 32 + l over the points (sixteen loads in flight), then the fold of the 64 cell sums.
template <typename F>
__global__ void __launch_bounds__(256) cell_block_sums_kernel(const F* detj, const F* weights, F* out,
                                                              int64_t num_cells, int num_points,
                                                              int tile_shift) {
  const int lane = threadIdx.x & 31;
  const int64_t mask = (1 << tile_shift) - 1;
  const int64_t nblocks = (num_cells + kSumBlock - 1) / kSumBlock;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nblocks; i += warps) {
    const int64_t start = i * kSumBlock;
    const int count = (int)(num_cells - start < kSumBlock ? num_cells - start : kSumBlock);
    const int64_t c0 = start + lane, c1 = start + 32 + lane;
    const bool v0 = lane < count, v1 = 32 + lane < count;
    const int64_t b0 = (((c0 >> tile_shift) * num_points) << tile_shift) + (c0 & mask);
    const int64_t b1 = (((c1 >> tile_shift) * num_points) << tile_shift) + (c1 & mask);
    F a0 = F(0), a1 = F(0);
    constexpr int U = 8;
    for (int q0 = 0; q0 < num_points; q0 += U) {
      F d0[U], d1[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int64_t off = (int64_t)(q0 + u) << tile_shift;
        const bool in = q0 + u < num_points;
        d0[u] = in && v0 ? __ldg(detj + b0 + off) : F(0);
        d1[u] = in && v1 ? __ldg(detj + b1 + off) : F(0);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int q = q0 + u;
        if (q < num_points) {
          const F w = __ldg(weights + q);
          a0 = q == 0 ? d0[u] * w : fma(d0[u], w, a0);
          a1 = q == 0 ? d1[u] * w : fma(d1[u], w, a1);
        }
      }
    }
    const F acc = warp_fold(a0, a1, count);
    if (lane == 0) out[i] = acc;
  }
}

}  // namespace tlg

namespace {

tlg_status measure_into(const void* detj, int dtype, int64_t num_cells, int64_t num_points, int shift,
                        const void* weights, void* scratch, void* result, cudaStream_t s);

// Device address of g_measure_scratch for each device, found once per device (with that device
// current) by the first call made on it, and again after a device reset.
std::mutex g_scratch_mutex;
void* g_scratch_ptr[64] = {};

tlg_status static_scratch(void** ptr) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return tlg::cuda_fail(e, "tlg_measure_static: cudaGetDevice");
  if (dev < 0 || dev >= 64) return tlg::fail(TLG_ERR_INVALID_ARGUMENT, "tlg_measure_static: device ordinal above 63");
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (g_scratch_ptr[dev]) {
    // The address found before belongs to the context of that time: after a device reset the
    // library's module is loaded anew and the array lives elsewhere, so look it up again when the
    // cached address is no longer this device's memory.
    cudaPointerAttributes at;
    const cudaError_t pe = cudaPointerGetAttributes(&at, g_scratch_ptr[dev]);
    if (pe != cudaSuccess) cudaGetLastError();  // (not sticky: clear it)
    if (pe != cudaSuccess || at.type != cudaMemoryTypeDevice || at.device != dev) g_scratch_ptr[dev] = nullptr;
  }
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, tlg::g_measure_scratch);
    if (e != cudaSuccess) return tlg::cuda_fail(e, "tlg_measure_static: cudaGetSymbolAddress");
    g_scratch_ptr[dev] = p;
  }
  *ptr = g_scratch_ptr[dev];
  return TLG_OK;
}

}  // namespace

extern "C" {

int64_t tlg_sum_workspace_bytes(int dtype, int64_t n) {
  if ((dtype != TLG_F32 && dtype != TLG_F64) || n < 0) return -1;
  return tlg::tree_elems(n) * dtype;
}

tlg_status tlg_measure_cell_sums(const void* detj, int dtype, int64_t num_cells, int64_t num_points,
                                 int tile, const void* weights, void* sums, void* stream) {
  int shift = -1;
  for (int s = 0; s <= 4; ++s)
    if (tile == (1 << s)) shift = s;
  if (shift < 0 || (dtype != TLG_F32 && dtype != TLG_F64) || num_cells < 0 || num_points < 0 ||
      num_points > (1 << 30))
    return tlg::fail(TLG_ERR_INVALID_ARGUMENT, "tlg_measure_cell_sums: bad tile, dtype or sizes");
  if (num_cells == 0) return tlg::ok();
  if (!detj || !sums || (num_points > 0 && !weights))
    return tlg::fail(TLG_ERR_INVALID_ARGUMENT, "tlg_measure_cell_sums: NULL pointer");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (num_points == 0) {
    cudaError_t e = cudaMemsetAsync(sums, 0, (size_t)num_cells * dtype, s);
    return e == cudaSuccess ? tlg::ok() : tlg::cuda_fail(e, "tlg_measure_cell_sums");
  }
  if (dtype == TLG_F32)
    tlg::cell_sums_kernel<float><<<tlg::grid_for(num_cells, 256), 256, 0, s>>>(
        static_cast<const float*>(detj), static_cast<const float*>(weights), static_cast<float*>(sums),
        num_cells, (int)num_points, shift);
  else
    tlg::cell_sums_kernel<double><<<tlg::grid_for(num_cells, 256), 256, 0, s>>>(
        static_cast<const double*>(detj), static_cast<const double*>(weights),
        static_cast<double*>(sums), num_cells, (int)num_points, shift);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? tlg::ok() : tlg::cuda_fail(e, "tlg_measure_cell_sums launch");
}

tlg_status tlg_sum(const void* x, int dtype, int64_t n, void* workspace, int64_t workspace_bytes,
                   void* result, void* stream) {
  if ((dtype != TLG_F32 && dtype != TLG_F64) || n < 0 || !result)
    return tlg::fail(TLG_ERR_INVALID_ARGUMENT, "tlg_sum: bad dtype, length or result");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (n == 0) {
    cudaError_t e = cudaMemsetAsync(result, 0, dtype, s);
    return e == cudaSuccess ? tlg::ok() : tlg::cuda_fail(e, "tlg_sum");
  }
  if (!x) return tlg::fail(TLG_ERR_INVALID_ARGUMENT, "tlg_sum: NULL input");
  if (workspace_bytes < tlg::tree_elems(n) * dtype || (tlg::tree_elems(n) > 0 && !workspace))
    return tlg::fail(TLG_ERR_LENGTH_MISMATCH,
                     "tlg_sum: workspace of " + std::to_string(workspace_bytes) + " bytes, " +
                         std::to_string(tlg::tree_elems(n) * dtype) + " needed");
  cudaError_t e =
      dtype == TLG_F32
          ? tlg::sum_tree<float>(static_cast<const float*>(x), n, static_cast<float*>(workspace),
                                 static_cast<float*>(result), s)
          : tlg::sum_tree<double>(static_cast<const double*>(x), n, static_cast<double*>(workspace),
                                  static_cast<double*>(result), s);
  return e == cudaSuccess ? tlg::ok() : tlg::cuda_fail(e, "tlg_sum launch");
}

int64_t tlg_measure_static_max_cells(void) { return tlg::kStaticMaxCells; }

tlg_status tlg_measure_static(const void* detj, int dtype, int64_t num_cells, int64_t num_points,
                              int tile, const void* weights, void* result, void* stream) {
  int shift = -1;
  for (int s = 0; s <= 4; ++s)
    if (tile == (1 << s)) shift = s;
  if (shift < 0 || (dtype != TLG_F32 && dtype != TLG_F64) || num_cells < 0 || num_points < 0 ||
      num_points > (1 << 30) || !result)
    return tlg::fail(TLG_ERR_INVALID_ARGUMENT, "tlg_measure_static: bad tile, dtype, sizes or result");
  if (num_cells > tlg::kStaticMaxCells)
    return tlg::fail(TLG_ERR_ALLOCATION_TOO_LARGE,
                     "tlg_measure_static: " + std::to_string(num_cells) +
                         " cells exceed the fixed scratch's maximum of " +
                         std::to_string(tlg::kStaticMaxCells));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (num_cells == 0 || num_points == 0) {
    cudaError_t e = cudaMemsetAsync(result, 0, dtype, s);
    return e == cudaSuccess ? tlg::ok() : tlg::cuda_fail(e, "tlg_measure_static");
  }
  if (!detj || !weights) return tlg::fail(TLG_ERR_INVALID_ARGUMENT, "tlg_measure_static: NULL input");
  void* scratch = nullptr;
  tlg_status st = static_scratch(&scratch);
  if (st != TLG_OK) return st;
  return measure_into(detj, dtype, num_cells, num_points, shift, weights, scratch, result, s);
}

int64_t tlg_measure_workspace_bytes(int dtype, int64_t num_cells) {
  if ((dtype != TLG_F32 && dtype != TLG_F64) || num_cells < 0) return -1;
  const int64_t level1 = (num_cells + tlg::kSumBlock - 1) / tlg::kSumBlock;
  return level1 > 1 ? (level1 + tlg::tree_elems(level1)) * dtype : 0;
}

tlg_status tlg_measure(const void* detj, int dtype, int64_t num_cells, int64_t num_points, int tile,
                       const void* weights, void* workspace, int64_t workspace_bytes, void* result, void* stream) {
  int shift = -1;
  for (int s = 0; s <= 4; ++s)
    if (tile == (1 << s)) shift = s;
  if (shift < 0 || (dtype != TLG_F32 && dtype != TLG_F64) || num_cells < 0 || num_points < 0 ||
      num_points > (1 << 30) || !result)
    return tlg::fail(TLG_ERR_INVALID_ARGUMENT, "tlg_measure: bad tile, dtype, sizes or result");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (num_cells == 0 || num_points == 0) {
    cudaError_t e = cudaMemsetAsync(result, 0, dtype, s);
    return e == cudaSuccess ? tlg::ok() : tlg::cuda_fail(e, "tlg_measure");
  }
  if (!detj || !weights) return tlg::fail(TLG_ERR_INVALID_ARGUMENT, "tlg_measure: NULL input");
  const int64_t need = tlg_measure_workspace_bytes(dtype, num_cells);
  if (workspace_bytes < need || (need > 0 && !workspace))
    return tlg::fail(TLG_ERR_LENGTH_MISMATCH, "tlg_measure: workspace of " + std::to_string(workspace_bytes) +
                                                  " bytes, " + std::to_string(need) + " needed");
  return measure_into(detj, dtype, num_cells, num_points, shift, weights, workspace, result, s);
}

}  // extern "C"

namespace {

// Level 1 (sums of 64 consecutive cell sums) straight from the det J field into `scratch` (or the
// result when there is one value), then the tree.
tlg_status measure_into(const void* detj, int dtype, int64_t num_cells, int64_t num_points, int shift,
                        const void* weights, void* scratch, void* result, cudaStream_t s) {
  const int64_t level1 = (num_cells + tlg::kSumBlock - 1) / tlg::kSumBlock;
  const unsigned grid = tlg::grid_for(level1 * 32, 256);
  cudaError_t e = cudaSuccess;
  if (dtype == TLG_F32) {
    float* l1 = level1 == 1 ? static_cast<float*>(result) : static_cast<float*>(scratch);
    tlg::cell_block_sums_kernel<float><<<grid, 256, 0, s>>>(
        static_cast<const float*>(detj), static_cast<const float*>(weights), l1, num_cells,
        (int)num_points, shift);
    e = cudaGetLastError();
    if (e == cudaSuccess && level1 > 1) e = tlg::sum_tree<float>(l1, level1, l1 + level1, static_cast<float*>(result), s);
  } else {
    double* l1 = level1 == 1 ? static_cast<double*>(result) : static_cast<double*>(scratch);
    tlg::cell_block_sums_kernel<double><<<grid, 256, 0, s>>>(
        static_cast<const double*>(detj), static_cast<const double*>(weights), l1, num_cells,
        (int)num_points, shift);
    e = cudaGetLastError();
    if (e == cudaSuccess && level1 > 1) e = tlg::sum_tree<double>(l1, level1, l1 + level1, static_cast<double*>(result), s);
  }
  return e == cudaSuccess ? tlg::ok() : tlg::cuda_fail(e, "measure launch");
}

}  // namespace

// ----------------------------------------------------------------------------------------
// Self-test of the integer conversions used by the split kernels.

namespace {

__global__ void conversions_kernel(const double* x, int64_t n, unsigned long long* mismatches) {
  unsigned long long bad_round = 0, bad_widen = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = x[i];
    const float want = __double2float_rn(v);
    const float got = tlg::d2f_rn(v);
    const bool nan = want != want;
    if (nan ? got == got : __float_as_uint(got) != __float_as_uint(want)) ++bad_round;
    const double w = (double)want;
    const double wg = tlg::f2d_exact(want);
    if (nan ? wg == wg : __double_as_longlong(wg) != __double_as_longlong(w)) ++bad_widen;
  }
  if (bad_round) atomicAdd(mismatches, bad_round);
  if (bad_widen) atomicAdd(mismatches + 1, bad_widen);
}

}  // namespace

tlg_status tlg_selftest_conversions(const double* x, int64_t n, unsigned long long* mismatches, void* stream) {
  if (n < 0 || !mismatches || (n > 0 && !x))
    return tlg::fail(TLG_ERR_INVALID_ARGUMENT, "tlg_selftest_conversions: bad arguments");
  if (n == 0) return tlg::ok();
  int64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 16) blocks = 152 * 16;
  conversions_kernel<<<(unsigned)blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(x, n, mismatches);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return tlg::cuda_fail(e, "tlg_selftest_conversions launch");
  return tlg::ok();
}
