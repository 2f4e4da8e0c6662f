// Blackwell tensor-core evaluation (tcgen05) for volume cells of many nodes: the node-by-basis
// contraction X^T Phi as a UMMA with FP32 accumulators in tensor memory.
//
// Per tile of 64 cells, for each coordinate g the A operand (M = 128 rows, K = nodes) holds the
// TF32 heads of the cells' coordinates relative to their first node in rows 0-63 and the TF32
// tails (the rounding remainders) in rows 64-127; the B operand (N = 32 columns: 8 points x phi,
// dphi_0..2) holds the tables' TF32 heads, a second B their tails. Two MMAs per k-step (A B_head,
// A B_tail) give rows c and 64 + c the products head x (B_head + B_tail) and tail x (B_head +
// B_tail): every partial product of the operands' heads and tails, so that the error stays at
// FP32 level (the tails' rounding at 2^-22). x and J of (cell c, point) are the sums of the two
// rows; the warps reading lane c and lane 64 + c (eight warps, two per lane quarter) exchange
// their rows' values through shared memory and each finishes two of the chunk's points: the
// epilogue of the other kernels (det J, K, facet normals; in split precision the condition
// estimate, and the FP64 recompute of ill-conditioned points by the whole warp, lanes splitting
// the nodes, so that one point does not stall its CTA).
//
// Operands: A is written by the threads (gather, subtraction, head/tail split) into shared memory
// in the canonical K-major layout without swizzle (8-row x 16-byte core matrices; core matrices
// along K 128 bytes apart, 8-row blocks kpad * 32 bytes apart); the tables are laid out on the host
// in the same form per chunk of 8 points and copied in by cp.async.bulk (double-buffered, an
// mbarrier per buffer). A ninth warp issues the copies, and the MMAs of the next chunk into the
// second accumulator buffer while the other eight run the epilogue of the current one;
// tcgen05.commit arrives on the chunk's mbarrier. Tensor memory: 2 buffers x 3 coordinates x 32 columns, allocated as 256
// columns; the launch's shared memory keeps at most two CTAs on an SM, so that the allocations
// never wait. Every wait is bounded: on expiry the CTA records an error, waits (bounded) for what
// it has in flight, frees its tensor memory and returns.
#pragma once

#include <cstdint>
#include <type_traits>

#include "convert.cuh"
#include "eval.cuh"

namespace tlg {

constexpr int kUmmaCells = 64;      // cells per tile
constexpr int kUmmaPoints = 8;      // points per chunk
constexpr int kUmmaN = 32;          // columns per chunk: 8 points x (phi, dphi_0, dphi_1, dphi_2)
constexpr int kUmmaEpi = 256;       // eight epilogue warps
constexpr int kUmmaThreads = 288;   // and one warp that issues the copies and the MMAs
constexpr int kUmmaIssuer = 256;    // its first thread
constexpr int kUmmaTmemCols = 256;  // 2 buffers x 3 coordinates x 32 columns, rounded to a power of 2
constexpr int kUmmaMaxKpad = 88;
constexpr int kUmmaFix = 1024;      // split: ill-conditioned points queued per tile

struct UmmaArgs {
  const void* nodes;
  const uint32_t* dofmap;
  const uint32_t* flags;
  const unsigned char* btab;  // [chunk][head, tail][32 x kpad, canonical layout] TF32 values
  const float* refn;          // reference normals [Q][3] (facet rules)
  const double* dphi64;       // split: the f64 derivative table [Q][K][3] of the recompute
  void* out[6];               // points, jacobian, detj, pinv, normals, facet normals (f32)
  int* err;                   // err[0] error word, err[1] poll override, err[2] = 1: no copies
  unsigned long long* recomputed;
  int64_t first_cell, padded, range_cells, out_first_cell, last_cell;
  double origin[3];
  float cond_limit;
  uint32_t last_node, mask;
  int k, kpad, num_points, chunks;
  // Work items: each tile's chunks in `groups` groups of `per_group` (the last ones padded with
  // zero tables; the table section holds chunks + kUmmaMaxGroups - 1 chunks).
  int groups, per_group;
};

constexpr int kUmmaMaxGroups = 8;

// Shared memory: A (3 x 128 x kpad), B (2 buffers x head and tail x 32 x kpad), the exchange
// (2 directions x 2 warp pairs x 24 values x 64 cells), 4 mbarriers, the tensor-memory address
// and the queue's count, the queue of ill-conditioned points, 1 KiB of alignment slack.
inline size_t umma_smem_bytes(int kpad) {
  return 1024 + (size_t)3 * 128 * kpad * 4 + (size_t)4 * kUmmaN * kpad * 4 + 2 * 48 * 64 * 4 + 64 + kUmmaFix * 4;
}

__device__ __forceinline__ uint32_t umma_tf32_head(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// Shared-memory matrix descriptor: start address, the byte distances of core matrices adjacent
// in K (leading) and in M/N (stride), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t umma_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor of kind::tf32: F32 accumulator, TF32 A and B, both K-major, N and M.
__host__ __device__ constexpr uint32_t umma_idesc(uint32_t m, uint32_t n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((n >> 3) << 17) | ((m >> 4) << 24);
}

__device__ __forceinline__ void umma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tmem_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive 32-bit columns of this thread's lane, waited for in the same statement.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15}, [%16];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// 8 consecutive 32-bit columns of this thread's lane, waited for in the same statement.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// J of one cell at one point in FP64 from the f64 nodes (relative to the cell's first node) and
// the f64 derivative table of the point ([K][TD]), by a whole warp: lane l takes nodes
// 1 + l, 33 + l, ...; a butterfly sums the lanes' partial J, which every lane receives.
template <int TD, int GD>
__device__ __noinline__ void recompute_j_f64_warp(const double* __restrict__ nodes, const uint32_t* row, int K,
                                                  uint32_t last_node, const double* d64, double* jd, int lane) {
  constexpr int LJ = TD * GD;
  double x0[GD], acc[LJ];
  const uint32_t n0 = min(__ldg(row), last_node);
#pragma unroll
  for (int g = 0; g < GD; ++g) x0[g] = __ldg(nodes + (int64_t)n0 * GD + g);
#pragma unroll
  for (int i = 0; i < LJ; ++i) acc[i] = 0.0;
  for (int k = 1 + lane; k < K; k += 32) {
    const uint32_t nk = min(__ldg(row + k), last_node);
#pragma unroll
    for (int g = 0; g < GD; ++g) {
      const double y = __ldg(nodes + (int64_t)nk * GD + g) - x0[g];
#pragma unroll
      for (int d = 0; d < TD; ++d) acc[d * GD + g] = __fma_rn(y, __ldg(d64 + k * TD + d), acc[d * GD + g]);
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
#pragma unroll
    for (int i = 0; i < LJ; ++i) acc[i] += __shfl_xor_sync(0xFFFFFFFFu, acc[i], off);
#pragma unroll
  for (int i = 0; i < LJ; ++i) jd[i] = acc[i];
}

// One thread: the copy of table chunk `chunk` into B buffer `buf` (head and tail, one bulk copy).
__device__ __forceinline__ void umma_load_b(const UmmaArgs& a, uint32_t bs, uint32_t bar, int chunk, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(bs),
               "l"(a.btab + (size_t)chunk * bytes), "r"(bytes), "r"(bar)
               : "memory");
}

__device__ __forceinline__ bool umma_wait(uint32_t bar, uint32_t parity, int polls) {
  bool done = false;
  for (int i = 0; i < polls && !done; ++i) done = mbar_try_wait(bar, parity);
  return done;
}

// Defined in umma.cu: the kernel of the precision, on a persistent grid.
cudaError_t launch_umma(bool split, const UmmaArgs& a, size_t smem, cudaStream_t s);

template <bool SPLIT>
__global__ void __launch_bounds__(kUmmaThreads, 1) umma_eval_kernel(const __grid_constant__ UmmaArgs a) {
  constexpr int TD = 3, GD = 3, LJ = 9;
  using A = Ar<float>;
  using M = Factors<float, TD, GD>;
  using NT = typename std::conditional<SPLIT, double, float>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // 1 KiB-aligned base (the operands' descriptors address 16-byte units).
  const uint32_t raw_s = (uint32_t)__cvta_generic_to_shared(smem_raw);
  unsigned char* smem = smem_raw + (((raw_s + 1023u) & ~1023u) - raw_s);
  const int kpad = a.kpad, K = a.k, nq = a.num_points;
  const uint32_t a_bytes = 128u * kpad * 4u;      // one coordinate's A
  const uint32_t b_half = (uint32_t)kUmmaN * kpad * 4u;  // head or tail of one B chunk
  const uint32_t sbo = (uint32_t)kpad * 32u;        // 8-row blocks
  float* xch = reinterpret_cast<float*>(smem + 3 * a_bytes + 4 * b_half);  // [2][48][64]
  uint64_t* bars = reinterpret_cast<uint64_t*>(xch + 2 * 48 * 64);         // B[2], MMA[2]
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 4);
  uint32_t* fix_n = tslot + 1;                                   // queued points of this tile
  uint32_t* fix = reinterpret_cast<uint32_t*>(bars + 8);         // [kUmmaFix]: (cell << 16) | point
  const uint32_t a_s = (uint32_t)__cvta_generic_to_shared(smem);
  const uint32_t b_s = a_s + 3 * a_bytes;
  const uint32_t bar_s = (uint32_t)__cvta_generic_to_shared(bars);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int polls = (a.err && a.err[1] > 0) ? a.err[1] : (1 << 22);
  const bool issue_copies = !(a.err && a.err[2] == 1);
  const NT* nodes = static_cast<const NT*>(a.nodes);
  const uint32_t mask = a.mask;
  const int64_t tiles = (a.padded + kUmmaCells - 1) / kUmmaCells;
  const int cpg = a.per_group;
  const int64_t items = tiles * a.groups;
  constexpr uint32_t kIdesc = umma_idesc(128, kUmmaN);

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     (uint32_t)__cvta_generic_to_shared(tslot)),
                 "r"((uint32_t)kUmmaTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    for (int i = 0; i < 4; ++i) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_s + 8 * i) : "memory");
    *fix_n = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tmem_fence_before();
  __syncthreads();
  tmem_fence_after();
  const uint32_t tmem = *tslot;

  // Chunk sequence of this CTA: chunk j of its i-th work item is number i * cpg + j; it uses B and
  // accumulator buffer (number & 1). Item t covers tile t / groups, chunks (t % groups) * cpg + j.
  auto item_of = [&](int64_t seq) { return (int64_t)blockIdx.x + (seq / cpg) * (int64_t)gridDim.x; };
  auto exists = [&](int64_t seq) { return item_of(seq) < items; };
  auto chunk_of = [&](int64_t seq) { return (int)(item_of(seq) % a.groups) * cpg + (int)(seq % cpg); };
  uint32_t ph_b[2] = {0u, 0u}, ph_m[2] = {0u, 0u};
  bool pend_b[2] = {false, false}, pend_m[2] = {false, false};  // thread 0: in flight
  const uint32_t bbytes = 2 * b_half;
  if (tid == kUmmaIssuer && issue_copies) {
    for (int s = 0; s < 2; ++s)
      if (exists(s)) {
        umma_load_b(a, b_s + s * bbytes, bar_s + 8 * s, chunk_of(s), bbytes);
        pend_b[s] = true;
      }
  }
  // Thread 0: the MMAs of chunk `seq` into accumulator buffer seq & 1, after its tables landed.
  auto issue = [&](int64_t seq) -> bool {
    const int buf = (int)(seq & 1);
    if (!umma_wait(bar_s + 8 * buf, ph_b[buf], polls)) return false;
    ph_b[buf] ^= 1u;
    pend_b[buf] = false;
    const uint32_t bh = b_s + buf * bbytes, bl = bh + b_half;
    for (int g = 0; g < GD; ++g) {
      const uint32_t d = tmem + (uint32_t)(buf * 96 + g * 32);
      const uint32_t ag = a_s + g * a_bytes;
      for (int s = 0; s < kpad / 8; ++s) {
        const uint64_t ad = umma_desc(ag + s * 256u, 128u, sbo);
        umma_tf32(d, ad, umma_desc(bh + s * 256u, 128u, sbo), kIdesc, s > 0);
        umma_tf32(d, ad, umma_desc(bl + s * 256u, 128u, sbo), kIdesc, 1u);
      }
    }
    umma_commit(bar_s + 16 + 8 * buf);
    pend_m[buf] = true;
    return true;
  };

  // Warp w reads tensor-memory lane quarter w % 4: quarters 0-1 the head rows of cells 0-63,
  // quarters 2-3 their tail rows. Of a chunk's 8 points, head-row warps finish points 0-3 and
  // tail-row warps 4-7, two per warp (w / 4 picks which two); each sends its rows' values of the
  // two points its partner (the warp with the other rows of the same cells and the same w / 4)
  // finishes.
  const bool mma_warp = warp == kUmmaEpi / 32;
  const int qd = warp & 3, sub = (warp >> 2) & 1;
  const bool top = qd < 2;
  const int c = (qd & 1) * 32 + lane;              // this thread's cell in the tile
  const int own0 = (top ? 0 : 4) + 2 * sub;        // first of the two points this warp finishes
  const int send0 = (top ? 4 : 0) + 2 * sub;       // first of the two points it sends
  float* xs_out = xch + (top ? 0 : 3072) + sub * 1536;
  const float* xs_in = xch + (top ? 3072 : 0) + sub * 1536;
  bool good = true;
  int64_t seq = 0;
  for (int64_t item = blockIdx.x; item < items && good; item += gridDim.x) {
    const int64_t tile = item / a.groups;
    const int chunk0 = (int)(item % a.groups) * cpg;
    // Gather: epilogue thread (cell tid % 64, nodes k = tid / 64 (mod 4)) writes heads to row c,
    // tails to row 64 + c of each coordinate's A.
    if (tid < kUmmaEpi) {
      const int gc = tid & 63;
      const int64_t cell = min(a.first_cell + tile * kUmmaCells + gc, a.last_cell);
      const uint32_t* row = a.dofmap + cell * K;
      NT x0[GD];
      const uint32_t n0 = min(__ldg(row), a.last_node);
#pragma unroll
      for (int g = 0; g < GD; ++g) x0[g] = __ldg(nodes + (int64_t)n0 * GD + g);
      for (int k = tid >> 6; k < kpad; k += kUmmaEpi / 64) {
        float y[GD];
        if (k < K) {
          const uint32_t n = min(__ldg(row + k), a.last_node);
#pragma unroll
          for (int g = 0; g < GD; ++g) {
            const NT v = __ldg(nodes + (int64_t)n * GD + g);
            if constexpr (SPLIT) y[g] = d2f_rn(v - x0[g]);
            else y[g] = v - x0[g];
          }
        } else {
#pragma unroll
          for (int g = 0; g < GD; ++g) y[g] = 0.0f;
        }
        const uint32_t o_hi = (uint32_t)(gc >> 3) * sbo + (uint32_t)(k >> 2) * 128u + (gc & 7) * 16u + (k & 3) * 4u;
        const uint32_t o_lo = o_hi + 8u * sbo;  // row 64 + gc
#pragma unroll
        for (int g = 0; g < GD; ++g) {
          const uint32_t h = umma_tf32_head(y[g]);
          const uint32_t t = umma_tf32_head(y[g] - __uint_as_float(h));
          *reinterpret_cast<uint32_t*>(smem + g * a_bytes + o_hi) = h;
          *reinterpret_cast<uint32_t*>(smem + g * a_bytes + o_lo) = t;
        }
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    tmem_fence_before();
    __syncthreads();
    tmem_fence_after();
    int ok = 1;
    if (tid == kUmmaIssuer) ok = issue(seq);

    // This thread's cell: its first node plus the origin (split: as an f32 pair), its output slot.
    const int64_t cr = tile * kUmmaCells + c;  // cell index in the range
    const int64_t cell = min(a.first_cell + cr, a.last_cell);
    const bool store = cr < a.padded;
    float xh[GD], xl[GD];
    {
      const uint32_t n0 = min(__ldg(a.dofmap + cell * K), a.last_node);
#pragma unroll
      for (int g = 0; g < GD; ++g) {
        if constexpr (SPLIT) {
          const double v = __ldg(static_cast<const double*>(a.nodes) + (int64_t)n0 * GD + g) + a.origin[g];
          xh[g] = d2f_rn(v);
          xl[g] = d2f_rn(v - f2d_exact(xh[g]));
        } else {
          xh[g] = __ldg(static_cast<const float*>(a.nodes) + (int64_t)n0 * GD + g);
          xl[g] = (float)a.origin[g];
        }
      }
    }
    const int64_t o = a.out_first_cell + cr;
    const int64_t tile_idx = o >> 4;
    const int tl = (int)(o & 15);

    for (int j = 0; j < cpg; ++j, ++seq) {
      const int buf = (int)(seq & 1);
      // Chunk j's accumulators (and its B buffer free again). The tensor-memory loads are
      // warp-collective: a warp loads only when all its lanes saw the chunk complete.
      bool done = ok && umma_wait(bar_s + 16 + 8 * buf, ph_m[buf], polls);
      if (done) {
        ph_m[buf] ^= 1u;
        if (tid == kUmmaIssuer) pend_m[buf] = false;
      }
      tmem_fence_after();
      if (tid == kUmmaIssuer && done && issue_copies && exists(seq + 2)) {
        umma_load_b(a, b_s + buf * bbytes, bar_s + 8 * buf, chunk_of(seq + 2), bbytes);
        pend_b[buf] = true;
      }
      const uint32_t trow = tmem + ((uint32_t)(qd * 32) << 16) + (uint32_t)(buf * 96);
      if (!mma_warp && __all_sync(0xFFFFFFFFu, done)) {
#pragma unroll
        for (int g = 0; g < GD; ++g) {
          float v[8];
          tmem_ld8(trow + g * 32 + 4 * send0, v);
#pragma unroll
          for (int i = 0; i < 8; ++i) xs_out[(g * 8 + i) * 64 + c] = v[i];
        }
      }
      if (__syncthreads_or(!done)) {
        good = false;
        break;
      }
      if (mma_warp) {
        // The next chunk's MMAs while the epilogue warps finish this one (its accumulator buffer
        // was freed by the previous chunk's closing barrier, its tables copied a chunk ago).
        if (tid == kUmmaIssuer && ok && j + 1 < cpg) ok = issue(seq + 1);
        tmem_fence_before();
        __syncthreads();
        tmem_fence_after();
        continue;
      }
      float u[GD][8];  // column 4 p + r of this warp's two points: r = 0 phi, 1 + d dphi_d
#pragma unroll
      for (int g = 0; g < GD; ++g) {
        tmem_ld8(trow + g * 32 + 4 * own0, u[g]);
#pragma unroll
        for (int i = 0; i < 8; ++i) u[g][i] = A::add(u[g][i], xs_in[(g * 8 + i) * 64 + c]);
      }
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        const int q = (chunk0 + j) * kUmmaPoints + own0 + p;
        if (q >= nq) continue;  // the same for the whole warp
        float x[GD], jm[LJ];
#pragma unroll
        for (int g = 0; g < GD; ++g) {
          x[g] = u[g][4 * p];
#pragma unroll
          for (int d = 0; d < TD; ++d) jm[d * GD + g] = u[g][4 * p + 1 + d];
        }
        if ((mask & kOutPoints) && store) {
          float xp[GD];
#pragma unroll
          for (int g = 0; g < GD; ++g)
            xp[g] = SPLIT ? A::add(xh[g], A::add(xl[g], x[g])) : A::add(A::add(x[g], xh[g]), xl[g]);
          store_point(static_cast<float*>(a.out[0]), tile_idx, q, nq, GD, tl, 4, xp, GD);
        }
        if ((mask & ~kOutPoints) == 0) continue;
        float kk[LJ];
        M::pinv(jm, kk);
        float dj = M::detj(jm);
        bool deferred = false;
        if constexpr (SPLIT) {
          // Ill-conditioned points go to the tile's queue (J, det J, K and facet normals from
          // FP64 at the end of the tile); beyond its capacity J comes from the f64 nodes and
          // table here, the warp's lanes splitting the nodes, one flagged lane at a time.
          const float kap = M::condition(jm, kk);
          const bool need = store && !(kap <= a.cond_limit) && (mask & (kOutJacobian | kOutDetJ | kOutPinv));
          bool here = false;
          if (need) {
            const uint32_t slot = atomicAdd(fix_n, 1u);
            if (slot < (uint32_t)kUmmaFix) {
              fix[slot] = ((uint32_t)c << 16) | (uint32_t)q;
              deferred = true;
            } else {
              here = true;
            }
          }
          uint32_t flagged = __ballot_sync(0xFFFFFFFFu, here);
          while (flagged) {
            const int src = __ffs(flagged) - 1;
            flagged &= flagged - 1;
            const int64_t cs = __shfl_sync(0xFFFFFFFFu, cell, src);
            double jd[LJ];
            recompute_j_f64_warp<TD, GD>(static_cast<const double*>(a.nodes), a.dofmap + cs * K, K, a.last_node,
                                         a.dphi64 + (int64_t)q * K * TD, jd, lane);
            if (lane == src) {
              using M64 = Factors<double, TD, GD>;
              double kd[LJ];
              M64::pinv(jd, kd);
              dj = (float)M64::detj(jd);
#pragma unroll
              for (int i = 0; i < LJ; ++i) {
                jm[i] = (float)jd[i];
                kk[i] = (float)kd[i];
              }
              if (a.recomputed && cr < a.range_cells) atomicAdd(a.recomputed, 1ull);
            }
          }
        }
        if (!store || deferred) continue;
        if (mask & kOutJacobian) store_point(static_cast<float*>(a.out[1]), tile_idx, q, nq, LJ, tl, 4, jm, LJ);
        if (mask & kOutDetJ) store_point(static_cast<float*>(a.out[2]), tile_idx, q, nq, 1, tl, 4, &dj, 1);
        if (mask & kOutPinv) store_point(static_cast<float*>(a.out[3]), tile_idx, q, nq, LJ, tl, 4, kk, LJ);
        if (mask & kOutFacetNormals) {
          float n[GD];
          M::facet_normal(kk, a.refn + q * TD, n);
          store_point(static_cast<float*>(a.out[5]), tile_idx, q, nq, GD, tl, 4, n, GD);
        }
      }
      // The accumulator buffer and the exchange are free for the chunk after next.
      tmem_fence_before();
      __syncthreads();
      tmem_fence_after();
    }
    if constexpr (SPLIT) {
      // The tile's queued points, one per thread: J, det J, K (and facet normals) from FP64.
      if (good) {
        const int nfix = min((int)*fix_n, kUmmaFix);
        __syncthreads();
        if (tid == 0) *fix_n = 0;  // the next tile's gather ends with a barrier
        for (int e = tid; e < nfix; e += kUmmaThreads) {  // the issuing warp too
          const int fc = (int)(fix[e] >> 16), fq = (int)(fix[e] & 0xFFFFu);
          const int64_t fcr = tile * kUmmaCells + fc;
          const int64_t fcell = min(a.first_cell + fcr, a.last_cell);
          float jr[LJ], kr[LJ], dr;
          recompute_f64_rt<TD, GD>(static_cast<const double*>(a.nodes), a.dofmap + fcell * K, K, a.last_node,
                                   a.dphi64 + (int64_t)fq * K * TD, jr, &dr, kr, 1);
          const int64_t fo = a.out_first_cell + fcr;
          const int64_t ft = fo >> 4;
          const int fl = (int)(fo & 15);
          if (mask & kOutJacobian) store_point(static_cast<float*>(a.out[1]), ft, fq, nq, LJ, fl, 4, jr, LJ);
          if (mask & kOutDetJ) store_point(static_cast<float*>(a.out[2]), ft, fq, nq, 1, fl, 4, &dr, 1);
          if (mask & kOutPinv) store_point(static_cast<float*>(a.out[3]), ft, fq, nq, LJ, fl, 4, kr, LJ);
          if (mask & kOutFacetNormals) {
            float n[GD];
            M::facet_normal(kr, a.refn + fq * TD, n);
            store_point(static_cast<float*>(a.out[5]), ft, fq, nq, GD, fl, 4, n, GD);
          }
          if (a.recomputed && fcr < a.range_cells) atomicAdd(a.recomputed, 1ull);
        }
      }
    }
  }
  if (!good) {
    // A wait expired: record it, let what is in flight land (bounded), then free the tensor
    // memory.
    if (tid == kUmmaIssuer) {
      if (a.err) atomicExch(a.err, 1);
      for (int b = 0; b < 2; ++b) {
        if (pend_m[b]) umma_wait(bar_s + 16 + 8 * b, ph_m[b], polls);
        if (pend_b[b]) umma_wait(bar_s + 8 * b, ph_b[b], polls);
      }
    }
  }
  tmem_fence_before();
  __syncthreads();
  tmem_fence_after();
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)kUmmaTmemCols)
                 : "memory");
}

}  // namespace tlg
