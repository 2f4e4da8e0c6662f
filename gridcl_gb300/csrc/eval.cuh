// Fused geometry-evaluation kernels for sm_103a.
//
// One thread per cell of a block range; persistent CTAs (a grid-stride loop). Each CTA stages
// the element's tabulation from global memory into its own shared memory with one bulk
// asynchronous copy (cp.async.bulk completing on an mbarrier); threads then read table entries
// at warp-uniform addresses, which shared memory broadcasts. A thread gathers its cell's K nodes
// through the dofmap (index clamped to the last node, the cell clamped to the block's last cell,
// tetraloma-geometry/src/evector.rs:221-222) into registers and walks the Q points: J, then
// every requested factor from J, each stored straight into its QuadField chunk at
// ((cell / tile) * Q * LEN + q * LEN + k) * tile + cell % tile
// (tetraloma-geometry/src/field.rs:121-162). Consecutive threads are consecutive cells, so each
// warp store covers whole tile rows.
//
// Arithmetic follows tetraloma-geometry/src/layout.rs:133-369: J(g, d) is the sum over the
// nodes in ascending k starting with the k = 0 product; det J and K by the same cofactor
// formulas; normals as s (J0 x J1) / |J0 x J1|. Every operation is an explicitly rounded
// intrinsic (no compiler contraction), written once for scalars and for f32 pairs, so the
// kernels below give the same bits for the same point whichever of them runs.
//
// Kernels:
//  - eval_pair_kernel<SPLIT, TD, GD, K>: f32 arithmetic on two quadrature points at once with
//    Blackwell's paired FP32 instructions (FFMA2 / FMUL2 / FADD2). SPLIT = false: an f32 mesh.
//    SPLIT = true: an f64 mesh, each cell shifted by its node 0 in f64 before rounding to f32,
//    f32 fields, and an FP64 recompute of J, det J and K at points whose condition estimate
//    exceeds a limit (counted in a device counter).
//  - eval_direct_kernel<F, TD, GD, K, TILE>: scalar, everything unrolled (the f64 path).
//  - eval_loops_kernel<F, TD, GD>: K and the tile at run time (every other element and tile).
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

#include "convert.cuh"

namespace tlg {

constexpr int kEvalThreads = 128;

// Output selection bits.
enum : uint32_t {
  kOutPoints = 1u,
  kOutJacobian = 2u,
  kOutDetJ = 4u,
  kOutPinv = 8u,
  kOutNormals = 16u,
  kOutFacetNormals = 32u,
  kOutCellMeasure = 64u,  // per-cell sums of det J * w (PairArgs::cell_measure; the MEAS kernels)
};

template <typename F>
struct EvalArgs {
  const F* nodes;            // [node][GD]
  const uint32_t* dofmap;    // [cell][K]
  const uint32_t* flags;     // [cell] or nullptr
  const unsigned char* tab;  // staged table bytes (16-byte aligned, size multiple of 16)
  F* out[6];                 // points, jacobian, detj, pinv, normals, facet normals
  F origin[3];
  int* err;                  // device error word (bounded waits)
  int64_t first_cell;        // first cell of the range in the block
  int64_t padded;            // range cells rounded up to the tile
  int64_t out_first_cell;    // the range's first cell in the output chunks
  int64_t last_cell;         // block cells - 1
  int64_t last_flag;         // last readable flag index, or -1
  uint32_t last_node;        // node count - 1
  uint32_t tab_bytes;
  uint32_t off_dphi;         // byte offset of the derivative table [Q][K][TD]
  uint32_t off_refn;         // byte offset of the reference normals [Q][TD]
  uint32_t mask;             // kOut* bits
  int num_points;            // Q
  int tile_shift;            // log2(tile)
  int k_runtime;             // K for the loops kernel
  int tab_global;            // loops kernel: tables read from global memory, not staged
  int loops_only;            // the loops kernel even where an unrolled kernel is compiled
};

// Arguments of the paired kernels (f32 arithmetic; nodes f32, or f64 with SPLIT).
struct PairArgs {
  const void* nodes;
  const uint32_t* dofmap;
  const uint32_t* flags;
  const unsigned char* tab;  // phi | dphi | refn | rows2 [QP][K][RW] | dphi64
  float* out[6];
  int* err;
  unsigned long long* recomputed;  // may be null
  int64_t first_cell, padded, range_cells, out_first_cell, last_cell, last_flag;
  double origin[3];
  float cond_limit;
  uint32_t last_node, tab_bytes, off_refn, off_rows2, off_dphi64, mask;
  int num_points;
  uint32_t off_dphi;  // the f32 derivative table [Q][K][TD] (split loops kernel; phi [Q][K] at 0)
  int k_runtime;      // K (split loops kernel)
  const float* weights;  // [Q], with kOutCellMeasure
  float* cell_measure;   // [range_cells], with kOutCellMeasure
};

// ----------------------------------------------------------------------------------------
// Table staging: one elected thread issues a bulk copy into shared memory; all threads wait on
// the mbarrier with a bounded number of polls. On expiry the CTA records an error and does a
// second bounded wait for its copy; a CTA whose tables never arrived returns without computing.

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

// err[0] is the error word; err[1] overrides the number of polls of each bounded wait (0: the
// default 2^22) and err[2] = 1 leaves the copy unissued, so that the wait runs out with nothing in
// flight (the tables' test hook, tlg_tables_set_wait). Returns whether the tables arrived, the
// same for every thread of the CTA; a CTA whose tables did not arrive computes nothing.
__device__ __forceinline__ bool stage_table(const unsigned char* src, unsigned char* dst,
                                            uint32_t bytes, uint64_t* bar, int* err) {
  const uint32_t bar_s = (uint32_t)__cvta_generic_to_shared(bar);
  const uint32_t dst_s = (uint32_t)__cvta_generic_to_shared(dst);
  const int limit = err ? err[1] : 0;
  const bool issue = !err || err[2] != 1;
  const int polls = limit > 0 ? limit : (1 << 22);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_s) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0 && issue) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_s), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(dst_s),
        "l"(src), "r"(bytes), "r"(bar_s)
        : "memory");
  }
  // Bounded poll: try_wait itself suspends for a hardware-defined interval per call. On expiry
  // the error word is set and a second bounded wait gives the copy time to land (the CTA must
  // not exit with its copy in flight).
  bool done = false;
  for (int i = 0; i < polls && !done; ++i) done = mbar_try_wait(bar_s, 0);
  if (!done) {
    if (err) atomicExch(err, 1);
    for (int i = 0; i < polls && !done; ++i) done = mbar_try_wait(bar_s, 0);
  }
  return __syncthreads_and(done) != 0;
}

// ----------------------------------------------------------------------------------------
// Explicitly rounded arithmetic on scalars and f32 pairs.

template <typename V>
struct Ar;

template <>
struct Ar<float> {
  using S = float;
  __device__ static float splat(float s) { return s; }
  __device__ static float mul(float a, float b) { return __fmul_rn(a, b); }
  __device__ static float add(float a, float b) { return __fadd_rn(a, b); }
  __device__ static float sub(float a, float b) { return __fsub_rn(a, b); }
  __device__ static float fma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
  __device__ static float neg(float a) { return -a; }
  __device__ static float rcp(float a) { return __frcp_rn(a); }
  __device__ static float div(float a, float b) { return __fdiv_rn(a, b); }
  __device__ static float sqrt(float a) { return __fsqrt_rn(a); }
};

template <>
struct Ar<double> {
  using S = double;
  __device__ static double splat(double s) { return s; }
  __device__ static double mul(double a, double b) { return __dmul_rn(a, b); }
  __device__ static double add(double a, double b) { return __dadd_rn(a, b); }
  __device__ static double sub(double a, double b) { return __dsub_rn(a, b); }
  __device__ static double fma(double a, double b, double c) { return __fma_rn(a, b, c); }
  __device__ static double neg(double a) { return -a; }
  __device__ static double rcp(double a) { return __drcp_rn(a); }
  __device__ static double div(double a, double b) { return __ddiv_rn(a, b); }
  __device__ static double sqrt(double a) { return __dsqrt_rn(a); }
};

// Two quadrature points at once: .x is point q, .y point q + 1.
template <>
struct Ar<float2> {
  using S = float;
  __device__ static float2 splat(float s) { return make_float2(s, s); }
  __device__ static float2 mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
  __device__ static float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
  __device__ static float2 neg(float2 a) { return make_float2(-a.x, -a.y); }
  __device__ static float2 sub(float2 a, float2 b) { return __fadd2_rn(a, neg(b)); }
  __device__ static float2 fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
  __device__ static float2 rcp(float2 a) { return make_float2(__frcp_rn(a.x), __frcp_rn(a.y)); }
  __device__ static float2 div(float2 a, float2 b) {
    return make_float2(__fdiv_rn(a.x, b.x), __fdiv_rn(a.y, b.y));
  }
  __device__ static float2 sqrt(float2 a) { return make_float2(__fsqrt_rn(a.x), __fsqrt_rn(a.y)); }
};

// Four values of F at a 16-byte-aligned address in one 16-byte access (f32) or two (f64).
template <typename F>
struct Vec4;
template <>
struct Vec4<float> {
  __device__ __forceinline__ static void put(float* p, float a, float b, float c, float d) {
    *reinterpret_cast<float4*>(p) = make_float4(a, b, c, d);
  }
  __device__ __forceinline__ static void get(const float* p, float* v) {
    const float4 u = *reinterpret_cast<const float4*>(p);
    v[0] = u.x;
    v[1] = u.y;
    v[2] = u.z;
    v[3] = u.w;
  }
};
template <>
struct Vec4<double> {
  __device__ __forceinline__ static void put(double* p, double a, double b, double c, double d) {
    reinterpret_cast<double2*>(p)[0] = make_double2(a, b);
    reinterpret_cast<double2*>(p)[1] = make_double2(c, d);
  }
  __device__ __forceinline__ static void get(const double* p, double* v) {
    const double2 u = reinterpret_cast<const double2*>(p)[0], w = reinterpret_cast<const double2*>(p)[1];
    v[0] = u.x;
    v[1] = u.y;
    v[2] = w.x;
    v[3] = w.y;
  }
};

// ----------------------------------------------------------------------------------------
// Factor math on J (column-major GD x TD), tetraloma-geometry/src/layout.rs:166-369, in the
// value type V. a*b - c*d is fma(a, b, -(c*d)) throughout.

template <typename V, int TD, int GD>
struct Factors {
  using A = Ar<V>;
  __device__ __forceinline__ static V cross(V a, V b, V c, V d) { return A::fma(a, b, A::neg(A::mul(c, d))); }

  __device__ __forceinline__ static V column_dot(const V* j, int a, int b) {
    V acc = A::mul(j[a * GD], j[b * GD]);
#pragma unroll
    for (int g = 1; g < GD; ++g) acc = A::fma(j[a * GD + g], j[b * GD + g], acc);
    return acc;
  }

  __device__ __forceinline__ static V square_det(const V* j) {
    if constexpr (TD == 1) {
      return j[0];
    } else if constexpr (TD == 2) {
      return cross(j[0], j[3], j[2], j[1]);
    } else {
      // j0 (j4 j8 - j7 j5) - j3 (j1 j8 - j7 j2) + j6 (j1 j5 - j4 j2)
      const V c0 = cross(j[4], j[8], j[7], j[5]);
      const V c1 = cross(j[1], j[8], j[7], j[2]);
      const V c2 = cross(j[1], j[5], j[4], j[2]);
      return A::fma(j[6], c2, A::fma(j[0], c0, A::neg(A::mul(j[3], c1))));
    }
  }

  // The normal n = J0 x J1 of a surface in 3D (TD = 2, GD = 3).
  __device__ __forceinline__ static void surface_normal(const V* j, V* n) {
    n[0] = cross(j[1], j[5], j[2], j[4]);
    n[1] = cross(j[2], j[3], j[0], j[5]);
    n[2] = cross(j[0], j[4], j[1], j[3]);
  }

  __device__ __forceinline__ static V dot3(const V* u, const V* v) {
    return A::fma(u[2], v[2], A::fma(u[1], v[1], A::mul(u[0], v[0])));
  }

  // det J, or the area element when TD < GD. For TD = 2, GD = 3 it is |J0 x J1|, which equals the
  // reference's sqrt(det(J^T J)) = sqrt(ac - b^2) (Lagrange's identity) with a rounding error
  // that grows with the condition number of J, not with its square.
  __device__ __forceinline__ static V detj(const V* j) {
    if constexpr (TD == GD) {
      return square_det(j);
    } else if constexpr (TD == 1) {
      return A::sqrt(column_dot(j, 0, 0));
    } else {
      V n[3];
      surface_normal(j, n);
      return A::sqrt(dot3(n, n));
    }
  }

  // K(t, g) at g * TD + t.
  __device__ __forceinline__ static void pinv(const V* j, V* k) {
    if constexpr (TD == GD) {
      const V inv = A::rcp(square_det(j));
      if constexpr (TD == 1) {
        k[0] = inv;
      } else if constexpr (TD == 2) {
        k[0] = A::mul(j[3], inv);
        k[2] = A::mul(A::neg(j[2]), inv);
        k[1] = A::mul(A::neg(j[1]), inv);
        k[3] = A::mul(j[0], inv);
      } else {
        k[0] = A::mul(cross(j[4], j[8], j[7], j[5]), inv);
        k[3] = A::mul(cross(j[6], j[5], j[3], j[8]), inv);
        k[6] = A::mul(cross(j[3], j[7], j[6], j[4]), inv);
        k[1] = A::mul(cross(j[7], j[2], j[1], j[8]), inv);
        k[4] = A::mul(cross(j[0], j[8], j[6], j[2]), inv);
        k[7] = A::mul(cross(j[6], j[1], j[0], j[7]), inv);
        k[2] = A::mul(cross(j[1], j[5], j[4], j[2]), inv);
        k[5] = A::mul(cross(j[3], j[2], j[0], j[5]), inv);
        k[8] = A::mul(cross(j[0], j[4], j[3], j[1]), inv);
      }
    } else if constexpr (TD == 1) {
      const V inv = A::rcp(column_dot(j, 0, 0));
#pragma unroll
      for (int g = 0; g < GD; ++g) k[g] = A::mul(j[g], inv);
    } else {
      // (J^T J)^-1 J^T with the identities c J0 - b J1 = J1 x n and a J1 - b J0 = n x J0, over
      // |n|^2 = ac - b^2, n = J0 x J1: the reference's G^-1 J^T (layout.rs:253-266) without
      // forming J^T J.
      V n[3];
      surface_normal(j, n);
      const V inv = A::rcp(dot3(n, n));
      const V* j0 = j;
      const V* j1 = j + 3;
      const V r0[3] = {cross(j1[1], n[2], j1[2], n[1]), cross(j1[2], n[0], j1[0], n[2]),
                       cross(j1[0], n[1], j1[1], n[0])};
      const V r1[3] = {cross(n[1], j0[2], n[2], j0[1]), cross(n[2], j0[0], n[0], j0[2]),
                       cross(n[0], j0[1], n[1], j0[0])};
#pragma unroll
      for (int g = 0; g < 3; ++g) {
        k[g * 2] = A::mul(r0[g], inv);
        k[g * 2 + 1] = A::mul(r1[g], inv);
      }
    }
  }

  // Codimension 1: s (J0_y, -J0_x) / |J0| or s (J0 x J1) / |J0 x J1|.
  __device__ __forceinline__ static void normal(const V* j, V s, V* n) {
    V v[GD];
    if constexpr (GD == 2) {
      v[0] = j[1];
      v[1] = A::neg(j[0]);
    } else {
      v[0] = cross(j[1], j[5], j[2], j[4]);
      v[1] = cross(j[2], j[3], j[0], j[5]);
      v[2] = cross(j[0], j[4], j[1], j[3]);
    }
    V s2 = A::mul(v[0], v[0]);
#pragma unroll
    for (int g = 1; g < GD; ++g) s2 = A::fma(v[g], v[g], s2);
    const V norm = A::sqrt(s2);
#pragma unroll
    for (int g = 0; g < GD; ++g) n[g] = A::div(A::mul(s, v[g]), norm);
  }

  // Codimension 0: m = K^T n_ref, m / |m| (nref: the reference normal of each point).
  __device__ __forceinline__ static void facet_normal(const V* k, const V* nref, V* n) {
    V m[GD];
#pragma unroll
    for (int g = 0; g < GD; ++g) {
      V acc = A::mul(k[g * TD], nref[0]);
#pragma unroll
      for (int t = 1; t < TD; ++t) acc = A::fma(k[g * TD + t], nref[t], acc);
      m[g] = acc;
    }
    V s2 = A::mul(m[0], m[0]);
#pragma unroll
    for (int g = 1; g < GD; ++g) s2 = A::fma(m[g], m[g], s2);
    const V norm = A::sqrt(s2);
#pragma unroll
    for (int g = 0; g < GD; ++g) n[g] = A::div(m[g], norm);
  }

  // |J|_F |K|_F / TD, the Frobenius condition estimate (tetraloma-testing/src/reference.rs:237).
  __device__ __forceinline__ static V condition(const V* j, const V* k) {
    V a = A::mul(j[0], j[0]), b = A::mul(k[0], k[0]);
#pragma unroll
    for (int i = 1; i < TD * GD; ++i) {
      a = A::fma(j[i], j[i], a);
      b = A::fma(k[i], k[i], b);
    }
    return A::mul(A::sqrt(A::mul(a, b)), A::splat((typename A::S)(1.0 / TD)));
  }
};

// ----------------------------------------------------------------------------------------
// Stores.

// Stores `len` components of one point of one cell: element (tile, q, comp, lane).
template <typename F>
__device__ __forceinline__ void store_point(F* out, int64_t tile_idx, int q, int nq, int len,
                                            int lane, int tile_shift, const F* v, int n) {
  F* base = out + ((((tile_idx * nq + q) * len) << tile_shift) + lane);
  for (int c = 0; c < n; ++c) base[(int64_t)c << tile_shift] = v[c];
}

// Output cursor of one field for one cell of a kernel with a compile-time tile: points at
// (tile, q, 0, lane); `put` stores one point's LEN components (immediate offsets c * TILE) and
// advances; `put2` stores two consecutive points (the second only when `both`).
template <typename F, int LEN, int TILE>
struct Cursor {
  F* p;
  __device__ __forceinline__ void init(F* out, int64_t tile_idx, int nq, int lane) {
    p = out + tile_idx * (int64_t)nq * (LEN * TILE) + lane;
  }
  __device__ __forceinline__ void put(const F* v) {
#pragma unroll
    for (int c = 0; c < LEN; ++c) p[c * TILE] = v[c];
    p += LEN * TILE;
  }
  __device__ __forceinline__ void put2(const float2* v, bool both) {
#pragma unroll
    for (int c = 0; c < LEN; ++c) p[c * TILE] = v[c].x;
    if (both) {
#pragma unroll
      for (int c = 0; c < LEN; ++c) p[(LEN + c) * TILE] = v[c].y;
    }
    p += 2 * LEN * TILE;
  }
};

// Loads the K node indices of one cell with the widest aligned vector loads.
template <int K>
__device__ __forceinline__ void load_row(const uint32_t* row, uint32_t* idx) {
  if constexpr (K % 4 == 0) {
#pragma unroll
    for (int k = 0; k < K; k += 4) {
      const uint4 v = __ldg(reinterpret_cast<const uint4*>(row + k));
      idx[k] = v.x;
      idx[k + 1] = v.y;
      idx[k + 2] = v.z;
      idx[k + 3] = v.w;
    }
  } else if constexpr (K % 2 == 0) {
#pragma unroll
    for (int k = 0; k < K; k += 2) {
      const uint2 v = __ldg(reinterpret_cast<const uint2*>(row + k));
      idx[k] = v.x;
      idx[k + 1] = v.y;
    }
  } else {
#pragma unroll
    for (int k = 0; k < K; ++k) idx[k] = __ldg(row + k);
  }
}

// ----------------------------------------------------------------------------------------
// FP64 recompute of one point of the split kernel: J from the f64 nodes shifted by node 0 and
// the f64 derivative row of the point, then det J and K, rounded to f32 and stored over the
// f32 values at the given addresses (component stride `stride`). Not inlined: it runs only at
// flagged points, and its FP64 registers stay out of the kernel body.
template <int TD, int GD, int K>
__device__ __noinline__ void recompute_f64(const double* __restrict__ nodes, const uint32_t* row,
                                           uint32_t last_node, const double* d64, float* pj,
                                           float* pd, float* pk, int stride) {
  constexpr int LJ = TD * GD;
  using M64 = Factors<double, TD, GD>;
  double jd[LJ], kd[LJ], x0[GD];
  const uint32_t n0 = min(__ldg(row), last_node);
#pragma unroll
  for (int g = 0; g < GD; ++g) x0[g] = __ldg(nodes + (int64_t)n0 * GD + g);
#pragma unroll
  for (int i = 0; i < LJ; ++i) jd[i] = 0.0;
  for (int k = 1; k < K; ++k) {
    const uint32_t nk = min(__ldg(row + k), last_node);
#pragma unroll
    for (int g = 0; g < GD; ++g) {
      const double yk = __ldg(nodes + (int64_t)nk * GD + g) - x0[g];
#pragma unroll
      for (int d = 0; d < TD; ++d) jd[d * GD + g] = __fma_rn(yk, d64[k * TD + d], jd[d * GD + g]);
    }
  }
  M64::pinv(jd, kd);
  if (pd) *pd = (float)M64::detj(jd);
#pragma unroll
  for (int i = 0; i < LJ; ++i) {
    if (pj) pj[i * stride] = (float)jd[i];
    if (pk) pk[i * stride] = (float)kd[i];
  }
}

// ----------------------------------------------------------------------------------------
// The paired f32 kernel (tile 16).

// Cells c0, c0 + step, ... below c_end of one block range, tables at `tabs` (shared memory).
template <bool SPLIT, int TD, int GD, int K, bool MEAS = false>
__device__ __forceinline__ void pair_cells(const PairArgs& a, const unsigned char* tabs, int64_t c0,
                                           int64_t c_end, int64_t step) {
  constexpr int TILE = 16;
  constexpr int LJ = TD * GD;
  using A = Ar<float2>;
  using M = Factors<float2, TD, GD>;
  // Per node of a point pair: (phi, dphi_0) in one 16-byte row, (dphi_1, dphi_2) in the next.
  constexpr int RW4 = TD == 1 ? 1 : 2;  // 16-byte rows per node
  const float4* rows2 = reinterpret_cast<const float4*>(tabs + a.off_rows2);
  const float* refn = reinterpret_cast<const float*>(tabs + a.off_refn);
  const double* dphi64 = reinterpret_cast<const double*>(tabs + a.off_dphi64);
  const int nq = a.num_points;
  const int nqp = (nq + 1) / 2;
  const uint32_t mask = a.mask;
  const bool want_j = (mask & ~kOutPoints) != 0;
  constexpr int K0 = SPLIT ? 1 : 0;  // the split kernel's node-0 term vanishes

  for (int64_t c = c0; c < c_end; c += step) {
    const int64_t cell = min(a.first_cell + c, a.last_cell);
    uint32_t idx[K];
    load_row<K>(a.dofmap + cell * K, idx);
    float x[K][GD];  // f32 nodes, or (SPLIT) x_k - x_0 rounded to f32 for k >= 1
    float xh[GD], xl[GD];  // the origin (f32 mesh) or x_0 + origin as an f32 pair (SPLIT)
    if constexpr (SPLIT) {
      const double* nodes = static_cast<const double*>(a.nodes);
      double x0[GD];
      const uint32_t n0 = min(idx[0], a.last_node);
#pragma unroll
      for (int g = 0; g < GD; ++g) x0[g] = __ldg(nodes + (int64_t)n0 * GD + g);
#pragma unroll
      for (int k = 1; k < K; ++k) {
        const uint32_t n = min(idx[k], a.last_node);
#pragma unroll
        for (int g = 0; g < GD; ++g) x[k][g] = d2f_rn(__ldg(nodes + (int64_t)n * GD + g) - x0[g]);
      }
#pragma unroll
      for (int g = 0; g < GD; ++g) {
        const double v = x0[g] + a.origin[g];
        xh[g] = d2f_rn(v);
        xl[g] = d2f_rn(v - f2d_exact(xh[g]));
      }
    } else {
      const float* nodes = static_cast<const float*>(a.nodes);
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const uint32_t n = min(idx[k], a.last_node);
#pragma unroll
        for (int g = 0; g < GD; ++g) x[k][g] = __ldg(nodes + (int64_t)n * GD + g);
      }
#pragma unroll
      for (int g = 0; g < GD; ++g) {
        xh[g] = (float)a.origin[g];
        xl[g] = 0.0f;
      }
    }
    float2 sign = A::splat(1.0f);
    if ((mask & kOutNormals) && a.flags != nullptr && a.last_flag >= 0) {
      const uint32_t f = __ldg(a.flags + min(a.first_cell + c, a.last_flag));
      sign = A::splat((f & 1u) ? -1.0f : 1.0f);
    }
    const int64_t o = a.out_first_cell + c;
    const int64_t tile_idx = o / TILE;
    const int lane = (int)(o % TILE);
    Cursor<float, GD, TILE> cx, cn, cf;
    Cursor<float, LJ, TILE> cj, ck;
    Cursor<float, 1, TILE> cd;
    if (mask & kOutPoints) cx.init(a.out[0], tile_idx, nq, lane);
    if (mask & kOutJacobian) cj.init(a.out[1], tile_idx, nq, lane);
    if (mask & kOutDetJ) cd.init(a.out[2], tile_idx, nq, lane);
    if (mask & kOutPinv) ck.init(a.out[3], tile_idx, nq, lane);
    if (mask & kOutNormals) cn.init(a.out[4], tile_idx, nq, lane);
    if (mask & kOutFacetNormals) cf.init(a.out[5], tile_idx, nq, lane);

    float meas = 0.0f;  // MEAS: the sum of det J * w over the points so far, in point order
    for (int qp = 0; qp < nqp; ++qp) {
      const bool both = 2 * qp + 1 < nq;
      const float4* rq = rows2 + (int64_t)qp * K * RW4;
      // One pass over the nodes: X and J of the pair from each node's one or two 16-byte rows
      // (X accumulated only when asked for; J only when anything beyond X is).
      const bool want_x = (mask & kOutPoints) != 0;
      float2 s[GD], j[LJ];
      {
        float2 w[4];
        const float4 r0 = rq[K0 * RW4];
        w[0] = make_float2(r0.x, r0.y);
        w[1] = make_float2(r0.z, r0.w);
        if constexpr (TD > 1) {
          const float4 r1 = rq[K0 * RW4 + 1];
          w[2] = make_float2(r1.x, r1.y);
          w[3] = make_float2(r1.z, r1.w);
        }
#pragma unroll
        for (int g = 0; g < GD; ++g) s[g] = A::mul(A::splat(x[K0][g]), w[0]);
#pragma unroll
        for (int d = 0; d < TD; ++d)
#pragma unroll
          for (int g = 0; g < GD; ++g) j[d * GD + g] = A::mul(A::splat(x[K0][g]), w[1 + d]);
      }
      // Below 27 nodes X and J share one pass over the rows; at 27 the shared pass holds too many
      // rows in flight (238 registers against 168 for two passes), so X and J take a pass each.
      constexpr bool kOnePass = K < 27;
      if (want_x && want_j && kOnePass) {
#pragma unroll
        for (int k = K0 + 1; k < K; ++k) {
          float2 w[4];
          const float4 r0 = rq[k * RW4];
          w[0] = make_float2(r0.x, r0.y);
          w[1] = make_float2(r0.z, r0.w);
          if constexpr (TD > 1) {
            const float4 r1 = rq[k * RW4 + 1];
            w[2] = make_float2(r1.x, r1.y);
            w[3] = make_float2(r1.z, r1.w);
          }
#pragma unroll
          for (int g = 0; g < GD; ++g) s[g] = A::fma(A::splat(x[k][g]), w[0], s[g]);
#pragma unroll
          for (int d = 0; d < TD; ++d)
#pragma unroll
            for (int g = 0; g < GD; ++g) j[d * GD + g] = A::fma(A::splat(x[k][g]), w[1 + d], j[d * GD + g]);
        }
      } else {
        if (want_x) {
#pragma unroll
          for (int k = K0 + 1; k < K; ++k) {
            const float4 r0 = rq[k * RW4];
            const float2 w0 = make_float2(r0.x, r0.y);
#pragma unroll
            for (int g = 0; g < GD; ++g) s[g] = A::fma(A::splat(x[k][g]), w0, s[g]);
          }
        }
        if (want_j) {
#pragma unroll
          for (int k = K0 + 1; k < K; ++k) {
            float2 w[4];
            const float4 r0 = rq[k * RW4];
            w[1] = make_float2(r0.z, r0.w);
            if constexpr (TD > 1) {
              const float4 r1 = rq[k * RW4 + 1];
              w[2] = make_float2(r1.x, r1.y);
              w[3] = make_float2(r1.z, r1.w);
            }
#pragma unroll
            for (int d = 0; d < TD; ++d)
#pragma unroll
              for (int g = 0; g < GD; ++g) j[d * GD + g] = A::fma(A::splat(x[k][g]), w[1 + d], j[d * GD + g]);
          }
        }
      }
      if (want_x) {
#pragma unroll
        for (int g = 0; g < GD; ++g) {
          if constexpr (SPLIT) s[g] = A::add(A::splat(xh[g]), A::add(A::splat(xl[g]), s[g]));
          else s[g] = A::add(s[g], A::splat(xh[g]));
        }
        cx.put2(s, both);
      }
      if (!want_j) continue;
      float2 kk[LJ];
      const bool want_k = (mask & (kOutPinv | kOutFacetNormals)) != 0 || SPLIT;
      if (want_k) M::pinv(j, kk);
      float* pj = (mask & kOutJacobian) ? cj.p : nullptr;
      float* pd = (mask & kOutDetJ) ? cd.p : nullptr;
      float* pk = (mask & kOutPinv) ? ck.p : nullptr;
      if (mask & kOutJacobian) cj.put2(j, both);
      float2 dj = A::splat(0.0f);
      if (mask & kOutDetJ) {
        dj = M::detj(j);
        cd.put2(&dj, both);
      }
      if (mask & kOutPinv) ck.put2(kk, both);
      if constexpr (TD == GD) {
        if (mask & kOutFacetNormals) {
          float2 nr[TD], n[GD];
#pragma unroll
          for (int t = 0; t < TD; ++t)
            nr[t] = make_float2(refn[(2 * qp) * TD + t], refn[min(2 * qp + 1, nq - 1) * TD + t]);
          M::facet_normal(kk, nr, n);
          cf.put2(n, both);
        }
      }
      if constexpr (TD + 1 == GD) {
        if (mask & kOutNormals) {
          float2 n[GD];
          M::normal(j, sign, n);
          cn.put2(n, both);
        }
      }
      bool redone = false;
      if constexpr (SPLIT) {
        // Near-degenerate points (or non-finite estimates) again in FP64.
        const float2 kap = M::condition(j, kk);
        if ((pj || pd || pk) && (!(kap.x <= a.cond_limit) || (both && !(kap.y <= a.cond_limit)))) {
          redone = true;
          const double* nodes = static_cast<const double*>(a.nodes);
          const uint32_t* row = a.dofmap + cell * K;
          for (int h = 0; h < (both ? 2 : 1); ++h) {
            const float kp = h == 0 ? kap.x : kap.y;
            if (kp <= a.cond_limit) continue;
            const int shift = h * LJ * TILE;
            recompute_f64<TD, GD, K>(nodes, row, a.last_node, dphi64 + (2 * qp + h) * K * TD,
                                     pj ? pj + shift : nullptr, pd ? pd + h * TILE : nullptr,
                                     pk ? pk + shift : nullptr, TILE);
            if (a.recomputed && c < a.range_cells) atomicAdd(a.recomputed, 1ull);
          }
        }
      }
      if constexpr (MEAS) {
        if (redone) {  // the det J values as stored (this thread's own writes)
          dj.x = pd[0];
          if (both) dj.y = pd[TILE];
        }
        const int q0 = 2 * qp;
        meas = q0 == 0 ? dj.x * __ldg(a.weights) : fmaf(dj.x, __ldg(a.weights + q0), meas);
        if (both) meas = fmaf(dj.y, __ldg(a.weights + q0 + 1), meas);
      }
    }
    if constexpr (MEAS) {
      if (c < a.range_cells) a.cell_measure[c] = meas;
    }
  }
}

template <bool SPLIT, int TD, int GD, int K, bool MEAS = false>
__global__ void __launch_bounds__(kEvalThreads) eval_pair_kernel(const __grid_constant__ PairArgs a) {
  __shared__ uint64_t bar;
  extern __shared__ __align__(16) unsigned char smem[];
  if (!stage_table(a.tab, smem, a.tab_bytes, &bar, a.err)) return;
  pair_cells<SPLIT, TD, GD, K, MEAS>(a, smem, (int64_t)blockIdx.x * blockDim.x + threadIdx.x, a.padded,
                               (int64_t)gridDim.x * blockDim.x);
}

// ----------------------------------------------------------------------------------------
// The direct kernel: scalar, K, TD, GD and the tile at compile time.

template <typename F, int TD, int GD, int K, int TILE>
__device__ __forceinline__ void direct_cells(const EvalArgs<F>& a, const unsigned char* tabs, int64_t c0,
                                             int64_t c_end, int64_t step) {
  const F* phi = reinterpret_cast<const F*>(tabs);
  const F* dphi = reinterpret_cast<const F*>(tabs + a.off_dphi);
  const F* refn = reinterpret_cast<const F*>(tabs + a.off_refn);
  const int nq = a.num_points;
  const uint32_t mask = a.mask;
  const bool want_j = (mask & ~kOutPoints) != 0;
  constexpr int LJ = TD * GD;
  using A = Ar<F>;
  using M = Factors<F, TD, GD>;

  for (int64_t c = c0; c < c_end; c += step) {
    const int64_t cell = min(a.first_cell + c, a.last_cell);
    uint32_t idx[K];
    load_row<K>(a.dofmap + cell * K, idx);
    F x[K][GD];
#pragma unroll
    for (int k = 0; k < K; ++k) {
      const uint32_t n = min(idx[k], a.last_node);
#pragma unroll
      for (int g = 0; g < GD; ++g) x[k][g] = __ldg(a.nodes + (int64_t)n * GD + g);
    }
    F sign = F(1);
    if ((mask & kOutNormals) && a.flags != nullptr && a.last_flag >= 0) {
      const uint32_t f = __ldg(a.flags + min(a.first_cell + c, a.last_flag));
      sign = (f & 1u) ? F(-1) : F(1);
    }
    const int64_t o = a.out_first_cell + c;
    const int64_t tile_idx = o / TILE;
    const int lane = (int)(o % TILE);
    Cursor<F, GD, TILE> cx, cn, cf;
    Cursor<F, LJ, TILE> cj, ck;
    Cursor<F, 1, TILE> cd;
    if (mask & kOutPoints) cx.init(a.out[0], tile_idx, nq, lane);
    if (mask & kOutJacobian) cj.init(a.out[1], tile_idx, nq, lane);
    if (mask & kOutDetJ) cd.init(a.out[2], tile_idx, nq, lane);
    if (mask & kOutPinv) ck.init(a.out[3], tile_idx, nq, lane);
    if (mask & kOutNormals) cn.init(a.out[4], tile_idx, nq, lane);
    if (mask & kOutFacetNormals) cf.init(a.out[5], tile_idx, nq, lane);

    for (int q = 0; q < nq; ++q) {
      if (mask & kOutPoints) {
        F xp[GD];
        const F* w = phi + q * K;
#pragma unroll
        for (int g = 0; g < GD; ++g) xp[g] = A::mul(x[0][g], w[0]);
#pragma unroll
        for (int k = 1; k < K; ++k) {
          const F wk = w[k];
#pragma unroll
          for (int g = 0; g < GD; ++g) xp[g] = A::fma(x[k][g], wk, xp[g]);
        }
#pragma unroll
        for (int g = 0; g < GD; ++g) xp[g] = A::add(xp[g], a.origin[g]);
        cx.put(xp);
      }
      if (!want_j) continue;
      F j[LJ];
      const F* dq = dphi + q * K * TD;
#pragma unroll
      for (int d = 0; d < TD; ++d) {
        const F w0 = dq[d];
#pragma unroll
        for (int g = 0; g < GD; ++g) j[d * GD + g] = A::mul(x[0][g], w0);
      }
#pragma unroll
      for (int k = 1; k < K; ++k) {
#pragma unroll
        for (int d = 0; d < TD; ++d) {
          const F w = dq[k * TD + d];
#pragma unroll
          for (int g = 0; g < GD; ++g) j[d * GD + g] = A::fma(x[k][g], w, j[d * GD + g]);
        }
      }
      if (mask & kOutJacobian) cj.put(j);
      if (mask & kOutDetJ) {
        const F dj = M::detj(j);
        cd.put(&dj);
      }
      if (mask & (kOutPinv | kOutFacetNormals)) {
        F k[LJ];
        M::pinv(j, k);
        if (mask & kOutPinv) ck.put(k);
        if constexpr (TD == GD) {
          if (mask & kOutFacetNormals) {
            F n[GD];
            M::facet_normal(k, refn + q * TD, n);
            cf.put(n);
          }
        }
      }
      if constexpr (TD + 1 == GD) {
        if (mask & kOutNormals) {
          F n[GD];
          M::normal(j, sign, n);
          cn.put(n);
        }
      }
    }
  }
}

template <typename F, int TD, int GD, int K, int TILE>
__global__ void __launch_bounds__(kEvalThreads) eval_direct_kernel(const __grid_constant__ EvalArgs<F> a) {
  __shared__ uint64_t bar;
  extern __shared__ __align__(16) unsigned char smem[];
  if (!stage_table(a.tab, smem, a.tab_bytes, &bar, a.err)) return;
  direct_cells<F, TD, GD, K, TILE>(a, smem, (int64_t)blockIdx.x * blockDim.x + threadIdx.x, a.padded,
                                   (int64_t)gridDim.x * blockDim.x);
}

// ----------------------------------------------------------------------------------------
// The loops kernel: any K and tile (run time), TD and GD at compile time; node coordinates
// re-read through L1 at each point. The same operations as the kernels above.

// The loops kernel's cells, tables at `tabs` (shared memory, or global memory when they exceed
// the shared-memory budget).
template <typename F, int TD, int GD>
__device__ __forceinline__ void loops_cells(const EvalArgs<F>& a, const unsigned char* tabs) {
  const F* phi = reinterpret_cast<const F*>(tabs);
  const F* dphi = reinterpret_cast<const F*>(tabs + a.off_dphi);
  const F* refn = reinterpret_cast<const F*>(tabs + a.off_refn);
  const int nq = a.num_points;
  const int K = a.k_runtime;
  const uint32_t mask = a.mask;
  const bool want_j = (mask & ~kOutPoints) != 0;
  constexpr int LJ = TD * GD;
  const int tile_mask = (1 << a.tile_shift) - 1;
  using A = Ar<F>;
  using M = Factors<F, TD, GD>;

  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < a.padded;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cell = min(a.first_cell + c, a.last_cell);
    const uint32_t* row = a.dofmap + cell * K;
    F sign = F(1);
    if ((mask & kOutNormals) && a.flags != nullptr && a.last_flag >= 0) {
      const uint32_t f = __ldg(a.flags + min(a.first_cell + c, a.last_flag));
      sign = (f & 1u) ? F(-1) : F(1);
    }
    const int64_t o = a.out_first_cell + c;
    const int64_t tile_idx = o >> a.tile_shift;
    const int lane = (int)(o & tile_mask);
    for (int q = 0; q < nq; ++q) {
      F xp[GD], j[LJ];
#pragma unroll
      for (int i = 0; i < GD; ++i) xp[i] = F(0);
#pragma unroll
      for (int i = 0; i < LJ; ++i) j[i] = F(0);
      for (int k = 0; k < K; ++k) {
        const uint32_t n = min(__ldg(row + k), a.last_node);
        F xk[GD];
#pragma unroll
        for (int g = 0; g < GD; ++g) xk[g] = __ldg(a.nodes + (int64_t)n * GD + g);
        if (mask & kOutPoints) {
          const F w = phi[q * K + k];
#pragma unroll
          for (int g = 0; g < GD; ++g) xp[g] = k == 0 ? A::mul(xk[g], w) : A::fma(xk[g], w, xp[g]);
        }
        if (want_j) {
#pragma unroll
          for (int d = 0; d < TD; ++d) {
            const F w = dphi[(q * K + k) * TD + d];
#pragma unroll
            for (int g = 0; g < GD; ++g)
              j[d * GD + g] = k == 0 ? A::mul(xk[g], w) : A::fma(xk[g], w, j[d * GD + g]);
          }
        }
      }
      if (mask & kOutPoints) {
#pragma unroll
        for (int g = 0; g < GD; ++g) xp[g] = A::add(xp[g], a.origin[g]);
        store_point(a.out[0], tile_idx, q, nq, GD, lane, a.tile_shift, xp, GD);
      }
      if (!want_j) continue;
      if (mask & kOutJacobian) store_point(a.out[1], tile_idx, q, nq, LJ, lane, a.tile_shift, j, LJ);
      if (mask & kOutDetJ) {
        const F dj = M::detj(j);
        store_point(a.out[2], tile_idx, q, nq, 1, lane, a.tile_shift, &dj, 1);
      }
      if (mask & (kOutPinv | kOutFacetNormals)) {
        F k[LJ];
        M::pinv(j, k);
        if (mask & kOutPinv) store_point(a.out[3], tile_idx, q, nq, LJ, lane, a.tile_shift, k, LJ);
        if constexpr (TD == GD) {
          if (mask & kOutFacetNormals) {
            F n[GD];
            M::facet_normal(k, refn + q * TD, n);
            store_point(a.out[5], tile_idx, q, nq, GD, lane, a.tile_shift, n, GD);
          }
        }
      }
      if constexpr (TD + 1 == GD) {
        if (mask & kOutNormals) {
          F n[GD];
          M::normal(j, sign, n);
          store_point(a.out[4], tile_idx, q, nq, GD, lane, a.tile_shift, n, GD);
        }
      }
    }
  }
}

// GTAB: the tables are read from global memory (L1/L2-cached) instead of being staged.
template <typename F, int TD, int GD, bool GTAB>
__global__ void __launch_bounds__(kEvalThreads) eval_loops_kernel(const __grid_constant__ EvalArgs<F> a) {
  if constexpr (GTAB) {
    loops_cells<F, TD, GD>(a, a.tab);
  } else {
    __shared__ uint64_t bar;
    extern __shared__ __align__(16) unsigned char smem[];
    if (!stage_table(a.tab, smem, a.tab_bytes, &bar, a.err)) return;
    loops_cells<F, TD, GD>(a, smem);
  }
}

// J, det J and K of one point in FP64 from the f64 nodes, K at run time (the split loops
// kernel's recompute of near-degenerate points); outputs as recompute_f64.
template <int TD, int GD>
__device__ __noinline__ void recompute_f64_rt(const double* __restrict__ nodes, const uint32_t* row, int K,
                                              uint32_t last_node, const double* d64, float* pj, float* pd,
                                              float* pk, int stride) {
  constexpr int LJ = TD * GD;
  using M64 = Factors<double, TD, GD>;
  double jd[LJ], kd[LJ], x0[GD];
  const uint32_t n0 = min(__ldg(row), last_node);
#pragma unroll
  for (int g = 0; g < GD; ++g) x0[g] = __ldg(nodes + (int64_t)n0 * GD + g);
#pragma unroll
  for (int i = 0; i < LJ; ++i) jd[i] = 0.0;
  for (int k = 1; k < K; ++k) {
    const uint32_t nk = min(__ldg(row + k), last_node);
#pragma unroll
    for (int g = 0; g < GD; ++g) {
      const double y = __ldg(nodes + (int64_t)nk * GD + g) - x0[g];
#pragma unroll
      for (int d = 0; d < TD; ++d) jd[d * GD + g] = __fma_rn(y, d64[k * TD + d], jd[d * GD + g]);
    }
  }
  M64::pinv(jd, kd);
#pragma unroll
  for (int i = 0; i < LJ; ++i) {
    if (pj) pj[i * stride] = (float)jd[i];
    if (pk) pk[i * stride] = (float)kd[i];
  }
  if (pd) *pd = (float)M64::detj(jd);
}

// Split precision with K at run time (elements without a paired kernel, or tables beyond the
// shared-memory budget with GTAB): one cell per thread, one point at a time, the same arithmetic
// as the paired kernel (f64 shift by node 0, FP32 J and X, FP64 recompute above the condition
// limit), tile 16.
template <int TD, int GD>
__device__ __forceinline__ void split_loops_cells(const PairArgs& a, const unsigned char* tabs) {
  constexpr int TILE = 16;
  constexpr int LJ = TD * GD;
  using A = Ar<float>;
  using M = Factors<float, TD, GD>;
  const float* phi = reinterpret_cast<const float*>(tabs);
  const float* dphi = reinterpret_cast<const float*>(tabs + a.off_dphi);
  const float* refn = reinterpret_cast<const float*>(tabs + a.off_refn);
  const double* dphi64 = reinterpret_cast<const double*>(tabs + a.off_dphi64);
  const double* nodes = static_cast<const double*>(a.nodes);
  const int nq = a.num_points;
  const int K = a.k_runtime;
  const uint32_t mask = a.mask;
  const bool want_j = (mask & ~kOutPoints) != 0;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < a.padded;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cell = min(a.first_cell + c, a.last_cell);
    const uint32_t* row = a.dofmap + cell * K;
    double x0[GD];
    const uint32_t n0 = min(__ldg(row), a.last_node);
    float xh[GD], xl[GD];
#pragma unroll
    for (int g = 0; g < GD; ++g) {
      x0[g] = __ldg(nodes + (int64_t)n0 * GD + g);
      const double v = x0[g] + a.origin[g];
      xh[g] = d2f_rn(v);
      xl[g] = d2f_rn(v - f2d_exact(xh[g]));
    }
    float sign = 1.0f;
    if ((mask & kOutNormals) && a.flags != nullptr && a.last_flag >= 0) {
      const uint32_t f = __ldg(a.flags + min(a.first_cell + c, a.last_flag));
      sign = (f & 1u) ? -1.0f : 1.0f;
    }
    const int64_t o = a.out_first_cell + c;
    const int64_t tile_idx = o / TILE;
    const int lane = (int)(o % TILE);
    for (int q = 0; q < nq; ++q) {
      float xp[GD], j[LJ];
#pragma unroll
      for (int i = 0; i < GD; ++i) xp[i] = 0.0f;
#pragma unroll
      for (int i = 0; i < LJ; ++i) j[i] = 0.0f;
      for (int k = 1; k < K; ++k) {
        const uint32_t n = min(__ldg(row + k), a.last_node);
        float y[GD];
#pragma unroll
        for (int g = 0; g < GD; ++g) y[g] = d2f_rn(__ldg(nodes + (int64_t)n * GD + g) - x0[g]);
        if (mask & kOutPoints) {
          const float w = phi[q * K + k];
#pragma unroll
          for (int g = 0; g < GD; ++g) xp[g] = A::fma(y[g], w, xp[g]);
        }
        if (want_j) {
#pragma unroll
          for (int d = 0; d < TD; ++d) {
            const float w = dphi[(q * K + k) * TD + d];
#pragma unroll
            for (int g = 0; g < GD; ++g) j[d * GD + g] = A::fma(y[g], w, j[d * GD + g]);
          }
        }
      }
      if (mask & kOutPoints) {
#pragma unroll
        for (int g = 0; g < GD; ++g) xp[g] = A::add(xh[g], A::add(xl[g], xp[g]));
        store_point(a.out[0], tile_idx, q, nq, GD, lane, 4, xp, GD);
      }
      if (!want_j) continue;
      float kk[LJ];
      M::pinv(j, kk);
      float dj = M::detj(j);
      const float kap = M::condition(j, kk);
      if (!(kap <= a.cond_limit) && (mask & (kOutJacobian | kOutDetJ | kOutPinv))) {
        // Through separate arrays, so that j and kk keep living in registers.
        float jr[LJ], kr[LJ], dr;
        recompute_f64_rt<TD, GD>(nodes, row, K, a.last_node, dphi64 + (int64_t)q * K * TD, jr, &dr, kr, 1);
#pragma unroll
        for (int i = 0; i < LJ; ++i) {
          j[i] = jr[i];
          kk[i] = kr[i];
        }
        dj = dr;
        if (a.recomputed && c < a.range_cells) atomicAdd(a.recomputed, 1ull);
      }
      if (mask & kOutJacobian) store_point(a.out[1], tile_idx, q, nq, LJ, lane, 4, j, LJ);
      if (mask & kOutDetJ) store_point(a.out[2], tile_idx, q, nq, 1, lane, 4, &dj, 1);
      if (mask & kOutPinv) store_point(a.out[3], tile_idx, q, nq, LJ, lane, 4, kk, LJ);
      if constexpr (TD == GD) {
        if (mask & kOutFacetNormals) {
          float n[GD];
          M::facet_normal(kk, refn + q * TD, n);
          store_point(a.out[5], tile_idx, q, nq, GD, lane, 4, n, GD);
        }
      }
      if constexpr (TD + 1 == GD) {
        if (mask & kOutNormals) {
          float n[GD];
          M::normal(j, sign, n);
          store_point(a.out[4], tile_idx, q, nq, GD, lane, 4, n, GD);
        }
      }
    }
  }
}

template <int TD, int GD, bool GTAB>
__global__ void __launch_bounds__(kEvalThreads) split_loops_kernel(const __grid_constant__ PairArgs a) {
  if constexpr (GTAB) {
    split_loops_cells<TD, GD>(a, a.tab);
  } else {
    __shared__ uint64_t bar;
    extern __shared__ __align__(16) unsigned char smem[];
    if (!stage_table(a.tab, smem, a.tab_bytes, &bar, a.err)) return;
    split_loops_cells<TD, GD>(a, smem);
  }
}

// ----------------------------------------------------------------------------------------
// E-vector gather, bit-exact: U is the unsigned integer type of F's width.

template <typename U>
__global__ void __launch_bounds__(256) evector_kernel(const U* nodes, const uint32_t* dofmap, U* out,
                                                      int64_t first_cell, int64_t last_cell,
                                                      uint32_t last_node, int K, int GD,
                                                      int64_t padded, int64_t stride) {
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < padded;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cell = min(first_cell + c, last_cell);
    for (int k = 0; k < K; ++k) {
      const uint32_t n = min(__ldg(dofmap + cell * K + k), last_node);
      for (int g = 0; g < GD; ++g)
        out[((int64_t)k * GD + g) * stride + c] = __ldg(nodes + (int64_t)n * GD + g);
    }
  }
}

}  // namespace tlg
