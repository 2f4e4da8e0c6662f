// Node-to-(cell, local node) CSR of a block's dofmap, by a stable LSD radix sort on the device.
//
// The entries of the dofmap, e = c * K + k, are sorted by node index with their entry index as
// the value. The sort is stable, so each node's entries stay in ascending e, that is in cell
// order and then local-node order: the CSR, and every sum taken through it, is the same on every
// run. This is the reference's deterministic recipe for incidence lists (sort, then scan;
// tetraloma-topology/src/connectivity.rs:1-3, tetraloma-device/src/primitives/radix_sort.rs).
//
// One pass per 8-bit digit (as many as the largest node index needs):
//  1. tile_histograms: each CTA counts the digits of its tile of 4096 entries;
//  2. an exclusive scan of the counts laid out [digit][tile] gives every (digit, tile) its first
//     output position;
//  3. tile_scatter: each CTA walks its tile in rounds of 256 entries in entry order; in a round,
//     a thread's rank among equal digits comes from its warp (__match_any_sync) and the earlier
//     warps' counts, so entries of one digit keep their order.
// Then csr_offsets (and csr_fill_gaps, for long runs of nodes without entries) mark where each
// node's run starts in the sorted keys.
#include <algorithm>
#include <cstdint>
#include <string>
#include <utility>

#include <cuda_runtime.h>

#include "../../include/tlgeom.h"
#include "status.h"

namespace tlg {
namespace {

constexpr int kSortThreads = 256;
constexpr int kRounds = 16;
constexpr int kTileItems = kSortThreads * kRounds;  // 4096 entries per CTA
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;  // per thread in the block scans: 4096 values per CTA
constexpr uint32_t kNoDigit = 0xFFFFFFFFu;

__global__ void __launch_bounds__(kSortThreads) tile_histograms(const uint32_t* keys, int64_t n, int shift,
                                                                uint32_t* counts, int64_t ntiles) {
  __shared__ uint32_t hist[256];
  hist[threadIdx.x] = 0;
  __syncthreads();
  const int64_t start = (int64_t)blockIdx.x * kTileItems;
  for (int r = 0; r < kRounds; ++r) {
    const int64_t i = start + (int64_t)r * kSortThreads + threadIdx.x;
    if (i < n) atomicAdd(&hist[(keys[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  counts[(int64_t)threadIdx.x * ntiles + blockIdx.x] = hist[threadIdx.x];
}

__global__ void __launch_bounds__(kSortThreads) tile_scatter(const uint32_t* keys_in, const uint32_t* vals_in,
                                                             uint32_t* keys_out, uint32_t* vals_out,
                                                             int64_t n, int shift,
                                                             const uint32_t* offsets, int64_t ntiles) {
  __shared__ uint32_t base[256];
  __shared__ uint32_t wcount[kSortThreads / 32][256];
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  base[threadIdx.x] = offsets[(int64_t)threadIdx.x * ntiles + blockIdx.x];
  const int64_t start = (int64_t)blockIdx.x * kTileItems;
  const uint32_t lt = (1u << lane) - 1u;
  for (int r = 0; r < kRounds; ++r) {
    for (int w = 0; w < kSortThreads / 32; ++w) wcount[w][threadIdx.x] = 0;
    __syncthreads();
    const int64_t i = start + (int64_t)r * kSortThreads + threadIdx.x;
    uint32_t key = 0, val = 0, digit = kNoDigit;
    if (i < n) {
      key = keys_in[i];
      val = vals_in[i];
      digit = (key >> shift) & 255u;
    }
    const uint32_t peers = __match_any_sync(0xFFFFFFFFu, digit);
    const uint32_t rank = __popc(peers & lt);
    if (digit != kNoDigit && rank == 0) wcount[warp][digit] = __popc(peers);
    __syncthreads();
    if (digit != kNoDigit) {
      uint32_t pos = base[digit] + rank;
      for (int w = 0; w < warp; ++w) pos += wcount[w][digit];
      keys_out[pos] = key;
      vals_out[pos] = val;
    }
    __syncthreads();
    uint32_t total = 0;
    for (int w = 0; w < kSortThreads / 32; ++w) total += wcount[w][threadIdx.x];
    base[threadIdx.x] += total;
    __syncthreads();
  }
}

// Block-level exclusive scan of kScanThreads * kScanItems values; returns the block total.
__device__ uint32_t block_exclusive_scan(uint32_t* v) {
  __shared__ uint32_t warp_sums[kScanThreads / 32];
  uint32_t local = 0;
  for (int j = 0; j < kScanItems; ++j) {
    const uint32_t x = v[j];
    v[j] = local;
    local += x;
  }
  const int lane = threadIdx.x % 32, warp = threadIdx.x / 32;
  uint32_t incl = local;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_sums[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t s = lane < kScanThreads / 32 ? warp_sums[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < kScanThreads / 32) warp_sums[lane] = s;  // inclusive
  }
  __syncthreads();
  const uint32_t before = (warp > 0 ? warp_sums[warp - 1] : 0) + incl - local;
  const uint32_t total = warp_sums[kScanThreads / 32 - 1];
  for (int j = 0; j < kScanItems; ++j) v[j] += before;
  __syncthreads();
  return total;
}

// Per-CTA totals of consecutive chunks of kScanThreads * kScanItems values.
__global__ void __launch_bounds__(kScanThreads) scan_partials(const uint32_t* x, int64_t n, uint32_t* partial) {
  __shared__ uint32_t s[32];
  const int64_t start = (int64_t)blockIdx.x * kScanThreads * kScanItems;
  uint32_t sum = 0;
  for (int j = 0; j < kScanItems; ++j) {
    const int64_t i = start + (int64_t)threadIdx.x * kScanItems + j;
    if (i < n) sum += x[i];
  }
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_down_sync(0xFFFFFFFFu, sum, o);
  if (threadIdx.x % 32 == 0) s[threadIdx.x / 32] = sum;
  __syncthreads();
  if (threadIdx.x < 32) {
    uint32_t t = s[threadIdx.x];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xFFFFFFFFu, t, o);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
  }
}

// Exclusive scan of `n` partials in one CTA, in chunks (sequential over chunks).
__global__ void __launch_bounds__(kScanThreads) scan_single(uint32_t* x, int64_t n) {
  uint32_t carry = 0;
  for (int64_t start = 0; start < n; start += kScanThreads * kScanItems) {
    uint32_t v[kScanItems];
    for (int j = 0; j < kScanItems; ++j) {
      const int64_t i = start + (int64_t)threadIdx.x * kScanItems + j;
      v[j] = i < n ? x[i] : 0;
    }
    const uint32_t total = block_exclusive_scan(v);
    for (int j = 0; j < kScanItems; ++j) {
      const int64_t i = start + (int64_t)threadIdx.x * kScanItems + j;
      if (i < n) x[i] = v[j] + carry;
    }
    carry += total;
    __syncthreads();
  }
}

// Exclusive scan of each chunk, offset by its scanned partial.
__global__ void __launch_bounds__(kScanThreads) scan_chunks(const uint32_t* x, uint32_t* y, int64_t n,
                                                            const uint32_t* partial) {
  const int64_t start = (int64_t)blockIdx.x * kScanThreads * kScanItems;
  uint32_t v[kScanItems];
  for (int j = 0; j < kScanItems; ++j) {
    const int64_t i = start + (int64_t)threadIdx.x * kScanItems + j;
    v[j] = i < n ? x[i] : 0;
  }
  block_exclusive_scan(v);
  const uint32_t off = partial[blockIdx.x];
  for (int j = 0; j < kScanItems; ++j) {
    const int64_t i = start + (int64_t)threadIdx.x * kScanItems + j;
    if (i < n) y[i] = v[j] + off;
  }
}

__global__ void init_entries(const uint32_t* dofmap, int64_t n, uint32_t last_node, uint32_t* keys,
                             uint32_t* vals) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    keys[i] = min(dofmap[i], last_node);  // the gather's clamp: such entries belong to the last node
    vals[i] = (uint32_t)i;
  }
}

// offsets[m] = first position of a key >= m, for m = 0..num_nodes. Position i (0 <= i <= n)
// starts the nodes keys[i - 1] + 1 .. keys[i] (from 0 at i = 0; up to num_nodes at i = n). Runs of
// at most kShortRun nodes are written by the position's thread; longer ones (the nodes before a
// block's first key or after its last, in a mesh of several blocks) are left to csr_fill_gaps.
constexpr int64_t kShortRun = 256;

__global__ void csr_offsets(const uint32_t* keys, int64_t n, int64_t num_nodes, uint32_t* offsets) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t lo = i == 0 ? -1 : (int64_t)keys[i - 1];
    const int64_t last = i == n ? num_nodes : (int64_t)keys[i];
    if (last - lo > kShortRun) continue;
    for (int64_t m = lo + 1; m <= last; ++m) offsets[m] = (uint32_t)i;
  }
}

// The nodes left unset (0xFFFFFFFF) by csr_offsets: a binary search over the sorted keys.
__global__ void csr_fill_gaps(const uint32_t* keys, int64_t n, int64_t num_nodes, uint32_t* offsets) {
  for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m <= num_nodes; m += (int64_t)gridDim.x * blockDim.x) {
    if (offsets[m] != 0xFFFFFFFFu) continue;
    int64_t lo = 0, hi = n;  // first position with keys[pos] >= m
    while (lo < hi) {
      const int64_t mid = (lo + hi) / 2;
      if ((int64_t)keys[mid] < m) lo = mid + 1;
      else hi = mid;
    }
    offsets[m] = (uint32_t)lo;
  }
}

inline unsigned grid_of(int64_t n, int threads, int64_t cap = 152 * 32) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > cap) b = cap;
  return (unsigned)b;
}

struct Workspace {
  uint32_t *keys_a, *vals_a, *keys_b, *vals_b, *counts, *partial;
  int64_t ntiles, ncounts, npartial;
};

int64_t align256(int64_t x) { return (x + 255) / 256 * 256; }

int64_t layout(int64_t n, Workspace* w, unsigned char* base) {
  const int64_t ntiles = (n + kTileItems - 1) / kTileItems;
  const int64_t ncounts = 256 * std::max<int64_t>(ntiles, 1);
  const int64_t npartial = (ncounts + kScanThreads * kScanItems - 1) / (kScanThreads * kScanItems);
  int64_t off = 0;
  auto take = [&](int64_t elems) {
    uint32_t* p = base ? reinterpret_cast<uint32_t*>(base + off) : nullptr;
    off += align256(std::max<int64_t>(elems, 1) * 4);
    return p;
  };
  if (w) {
    w->ntiles = ntiles;
    w->ncounts = ncounts;
    w->npartial = npartial;
  }
  uint32_t* p[6];
  p[0] = take(n);
  p[1] = take(n);
  p[2] = take(n);
  p[3] = take(n);
  p[4] = take(ncounts);
  p[5] = take(npartial);
  if (w) {
    w->keys_a = p[0];
    w->vals_a = p[1];
    w->keys_b = p[2];
    w->vals_b = p[3];
    w->counts = p[4];
    w->partial = p[5];
  }
  return off;
}

cudaError_t exclusive_scan(uint32_t* x, int64_t n, uint32_t* partial, int64_t npartial, cudaStream_t s) {
  const unsigned blocks = (unsigned)npartial;
  scan_partials<<<blocks, kScanThreads, 0, s>>>(x, n, partial);
  scan_single<<<1, kScanThreads, 0, s>>>(partial, npartial);
  scan_chunks<<<blocks, kScanThreads, 0, s>>>(x, x, n, partial);
  return cudaGetLastError();
}

}  // namespace
}  // namespace tlg

extern "C" {

int64_t tlg_csr_workspace_bytes(int64_t num_cells, int nodes_per_cell) {
  if (num_cells < 0 || nodes_per_cell < 1) return -1;
  return tlg::layout(num_cells * nodes_per_cell, nullptr, nullptr);
}

tlg_status tlg_csr_build(const uint32_t* dofmap, int64_t num_cells, int nodes_per_cell, int64_t num_nodes,
                         void* workspace, int64_t workspace_bytes, uint32_t* offsets, uint32_t* entries,
                         void* stream) {
  if (num_cells < 0 || nodes_per_cell < 1 || num_nodes < 1 || !offsets || (num_cells > 0 && (!dofmap || !entries)))
    return tlg::fail(TLG_ERR_INVALID_ARGUMENT, "tlg_csr_build: bad sizes or NULL pointer");
  const int64_t n = num_cells * nodes_per_cell;
  if (n > (int64_t)UINT32_MAX || num_nodes > (int64_t)UINT32_MAX)
    return tlg::fail(TLG_ERR_TOO_LARGE, "tlg_csr_build: entry or node count does not fit u32");
  const int64_t need = tlg::layout(n, nullptr, nullptr);
  if (workspace_bytes < need || !workspace)
    return tlg::fail(TLG_ERR_LENGTH_MISMATCH, "tlg_csr_build: workspace of " + std::to_string(workspace_bytes) +
                                                  " bytes, " + std::to_string(need) + " needed");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  tlg::Workspace w;
  tlg::layout(n, &w, static_cast<unsigned char*>(workspace));
  const uint32_t last_node = (uint32_t)(num_nodes - 1);
  if (n > 0) {
    tlg::init_entries<<<tlg::grid_of(n, 256), 256, 0, s>>>(dofmap, n, last_node, w.keys_a, w.vals_a);
    int bits = 0;
    while (bits < 32 && (last_node >> bits) != 0) ++bits;
    const int passes = bits == 0 ? 0 : (bits + 7) / 8;
    for (int p = 0; p < passes; ++p) {
      tlg::tile_histograms<<<(unsigned)w.ntiles, tlg::kSortThreads, 0, s>>>(w.keys_a, n, 8 * p, w.counts, w.ntiles);
      cudaError_t e = tlg::exclusive_scan(w.counts, w.ncounts, w.partial, w.npartial, s);
      if (e != cudaSuccess) return tlg::cuda_fail(e, "tlg_csr_build scan");
      tlg::tile_scatter<<<(unsigned)w.ntiles, tlg::kSortThreads, 0, s>>>(w.keys_a, w.vals_a, w.keys_b, w.vals_b, n,
                                                                      8 * p, w.counts, w.ntiles);
      std::swap(w.keys_a, w.keys_b);
      std::swap(w.vals_a, w.vals_b);
    }
    cudaError_t e = cudaMemcpyAsync(entries, w.vals_a, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return tlg::cuda_fail(e, "tlg_csr_build copy");
  }
  cudaError_t e = cudaMemsetAsync(offsets, 0xFF, (size_t)(num_nodes + 1) * sizeof(uint32_t), s);
  if (e != cudaSuccess) return tlg::cuda_fail(e, "tlg_csr_build offsets");
  tlg::csr_offsets<<<tlg::grid_of(n + 1, 256), 256, 0, s>>>(w.keys_a, n, num_nodes, offsets);
  tlg::csr_fill_gaps<<<tlg::grid_of(num_nodes + 1, 256), 256, 0, s>>>(w.keys_a, n, num_nodes, offsets);
  e = cudaGetLastError();
  if (e != cudaSuccess) return tlg::cuda_fail(e, "tlg_csr_build");
  return tlg::ok();
}

}  // extern "C"
