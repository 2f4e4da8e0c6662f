// Adjoint (vector-Jacobian product) of the geometric factors, codimension 0 (TD = GD = D).
//
// For a scalar L(x, J, det J, K) with cotangents xbar = dL/dx, dbar = dL/d(det J) and
// Kbar = dL/dK at every point, the cotangent of the node coordinates is
//   gbar(n, g) = sum over the (cell, k) with dofmap(cell, k) = n of
//                sum_q [ phi_k(q) xbar(q, g) + sum_d Jbar(q)(g, d) dphi_k(q)[d] ],
//   Jbar(g, d) = dbar det J K(d, g) - (K^T Kbar K^T)(g, d),
// from d det J = det J tr(K dJ) and dK = -K dJ K. J, det J and K are recomputed here, not read.
//
// vjp_kernel writes each cell's contributions L(cell, k, g), cell-major in rows of R values
// ([cell][k][R], R = 4 for D = 3 with a zero pad, else D), so that the entry e = cell * K + k
// of the node CSR owns the aligned row at e * R, read by one vector load; and, when asked, the
// forward fields of the same points in the same pass (the fused forward + adjoint). vjp_gather
// then sums, for every node, the contributions listed by the node's CSR entries in entry order,
// in f64: deterministic.
//
// Four lanes per cell split the cell's nodes: lane r owns the nodes k = r, r + 4, r + 8, ...
// with all D coordinates. Each lane forms the partial J (and x) over its nodes; a two-level
// butterfly (xor 1, then xor 2) sums the partials, and since IEEE addition commutes every lane
// of the group ends with the same bits. det J, K and Jbar are then formed by every lane, and
// each lane accumulates the contributions of its own nodes. One node row of the table (phi and
// dphi of one point, or of a point pair) is 32 bytes: two 16-byte shared-memory loads. The
// cotangents of the next step are loaded while the current step's contributions accumulate.
// The eight cells of a warp are consecutive: their contributions are staged in shared memory
// and written as one contiguous run.
//
// SPLIT: f64 nodes shifted by node 0 in f64, FP32 arithmetic on two points at a time (FFMA2,
// FMUL2 and FADD2 over the pair (q, q + 1)), f32 cotangents, contributions and fields.
// Otherwise f64 throughout, one point at a time.
#pragma once

#include <cstdint>
#include <type_traits>

#include "eval.cuh"

namespace tlg {

// Arguments of the adjoint below codimension 0 (vjp_surface.cu).
struct VjpSurfArgs {
  const void* nodes;
  const uint32_t* dofmap;
  const uint32_t* flags;
  const unsigned char* tab;  // phi [Q][K] at 0, dphi [Q][K][TD] at off_dphi (staged unless tab_global)
  const void* ct[4];         // cotangents: points, detj (area element), pinv, normals, or null
  void* out[5];              // fused forward: points, jacobian, detj, pinv, normals, or null
  void* local;               // contributions [cell][K][R]
  int* err;
  int64_t first_cell, padded, out_first_cell, last_cell, range_end, last_flag;
  double origin[3];
  uint32_t last_node, tab_bytes, off_dphi;
  int k, num_points, tab_global;
};

struct VjpArgs {
  const void* nodes;
  const uint32_t* dofmap;
  const unsigned char* tab;  // node rows [QV][K][4] of V: phi, dphi_0 .. dphi_{D-1}, padding
  const void* ct[3];         // cotangents: points, detj, pinv (tile 16 chunks) or null
  void* out[4];              // fused forward fields: points, jacobian, detj, pinv, or null
  void* local;               // contributions [cell][K][R] of the arithmetic's scalar type
  int* err;
  int64_t first_cell, padded, out_first_cell, last_cell, range_end;
  double origin[3];
  uint32_t last_node, tab_bytes;
  int num_points;
  int k_runtime;  // K (vjp_tile_kernel)
  int group;      // nodes per item (vjp_tile_kernel)
};

constexpr int kVjpGroup = 4;
constexpr int kVjpCellsPerWarp = 32 / kVjpGroup;

// Values per contribution row: D, padded to 4 for D = 3 so that rows are 16- or 32-byte aligned.
__host__ __device__ constexpr int vjp_row(int d) { return d == 3 ? 4 : d; }

// CTAs per SM the register allocation is bounded for: 4 where the kernel fits 128 registers
// without spills, else 3 (168 registers; the 27-node hexahedron spills a few words there).
__host__ __device__ constexpr int vjp_min_blocks(bool split, int d, int k) {
  return d == 2 || k <= 8 || (split && k <= 10) ? 4 : 3;
}

template <bool SPLIT>
struct VjpScalar;
template <>
struct VjpScalar<true> {
  using S = float;
  using V = float2;  // a point pair
  static constexpr int P = 2;
  __device__ static void row(const float2* p, float2 (&v)[4]) {
    const float4 a = reinterpret_cast<const float4*>(p)[0];
    const float4 b = reinterpret_cast<const float4*>(p)[1];
    v[0] = make_float2(a.x, a.y);
    v[1] = make_float2(a.z, a.w);
    v[2] = make_float2(b.x, b.y);
    v[3] = make_float2(b.z, b.w);
  }
  __device__ static float2 shfl_xor(float2 v, int m) {
    return make_float2(__shfl_xor_sync(0xFFFFFFFFu, v.x, m), __shfl_xor_sync(0xFFFFFFFFu, v.y, m));
  }
};
template <>
struct VjpScalar<false> {
  using S = double;
  using V = double;
  static constexpr int P = 1;
  __device__ static void row(const double* p, double (&v)[4]) {
    const double2 a = reinterpret_cast<const double2*>(p)[0];
    const double2 b = reinterpret_cast<const double2*>(p)[1];
    v[0] = a.x;
    v[1] = a.y;
    v[2] = b.x;
    v[3] = b.y;
  }
  __device__ static double shfl_xor(double v, int m) { return __shfl_xor_sync(0xFFFFFFFFu, v, m); }
};

// Shared memory past the staged table: one slot of 8 cells x K rows of contributions per warp.
inline size_t vjp_stage_bytes(bool split, int d, int k) {
  return (size_t)(kEvalThreads / 32) * kVjpCellsPerWarp * k * vjp_row(d) * (split ? 4 : 8);
}

template <bool SPLIT, int D, int K>
__global__ void __launch_bounds__(kEvalThreads, vjp_min_blocks(SPLIT, D, K))
    vjp_kernel(const __grid_constant__ VjpArgs a) {
  using T = VjpScalar<SPLIT>;
  using S = typename T::S;
  using V = typename T::V;
  using A = Ar<V>;
  using M = Factors<V, D, D>;
  constexpr int P = T::P;
  constexpr int G = kVjpGroup;
  constexpr int NK = (K + G - 1) / G;  // node slots per lane
  constexpr int TILE = 16;
  constexpr int LJ = D * D;
  constexpr int R = vjp_row(D);
  __shared__ uint64_t bar;
  extern __shared__ __align__(16) unsigned char smem[];
  if (!stage_table(a.tab, smem, a.tab_bytes, &bar, a.err)) return;
  const V* tab = reinterpret_cast<const V*>(smem);
  S* stage = reinterpret_cast<S*>(smem + (a.tab_bytes + 15) / 16 * 16) +
             (threadIdx.x / 32) * (kVjpCellsPerWarp * K * R);
  const int nq = a.num_points;
  const int nqv = (nq + P - 1) / P;
  const int lane = threadIdx.x % 32;
  const int r = lane % G;               // this lane's nodes: k = r + G j, j < nown
  const int nown = (K - r + G - 1) / G;
  const int rl = r < D ? r : D - 1;     // the row of the forward fields this lane stores
  const int slot = lane / G;
  const int cells_per_cta = kEvalThreads / G;
  const S* ctx = static_cast<const S*>(a.ct[0]);
  const S* ctd = static_cast<const S*>(a.ct[1]);
  const S* ctk = static_cast<const S*>(a.ct[2]);
  const double* nodes = static_cast<const double*>(a.nodes);

  // The trip count is uniform over a warp: padded is a multiple of 16 and a warp's cells are the
  // 8 consecutive c of one aligned run.
  for (int64_t c = (int64_t)blockIdx.x * cells_per_cta + threadIdx.x / G; c < a.padded;
       c += (int64_t)gridDim.x * cells_per_cta) {
    const int64_t cell = min(a.first_cell + c, a.last_cell);
    const uint32_t* drow = a.dofmap + cell * K;
    double x0[D];
#pragma unroll
    for (int g = 0; g < D; ++g) x0[g] = 0.0;
    if constexpr (SPLIT) {
      const int64_t n0 = min(__ldg(drow), a.last_node);
#pragma unroll
      for (int g = 0; g < D; ++g) x0[g] = __ldg(nodes + n0 * D + g);
    }
    S xk[NK][D];
#pragma unroll
    for (int j = 0; j < NK; ++j) {
      const bool own = j < nown;
      const int64_t n = min(__ldg(drow + min(r + G * j, K - 1)), a.last_node);
#pragma unroll
      for (int g = 0; g < D; ++g) {
        const double v = __ldg(nodes + n * D + g);
        if constexpr (SPLIT) xk[j][g] = own ? d2f_rn(v - x0[g]) : 0.0f;
        else xk[j][g] = own ? v : 0.0;
      }
    }
    // Absolute offset of this lane's row: split into two f32 values with SPLIT.
    double xo = x0[0] + a.origin[0];
#pragma unroll
    for (int g = 1; g < D; ++g)
      if (rl == g) xo = x0[g] + a.origin[g];
    S xh, xl;
    if constexpr (SPLIT) {
      xh = d2f_rn(xo);
      xl = d2f_rn(xo - f2d_exact(xh));
    } else {
      xh = xo;
      xl = 0.0;
    }

    const int64_t o = a.out_first_cell + c;
    const int64_t tq = (o / TILE) * nq;
    const int l16 = (int)(o % TILE);
    // Element (tile, q, comp, l16) of a tiled field with `len` components.
#define TLG_AT(q, len, comp) (((tq + (q)) * (len) + (comp)) * TILE + l16)
    // Cotangents of step qv (zero for the repeated odd last point of a pair).
    auto ld = [&](const S* p, int qv, int len, int comp) -> V {
      if constexpr (SPLIT) {
        const int q0 = qv * 2;
        return make_float2(__ldg(p + TLG_AT(q0, len, comp)),
                           q0 + 1 < nq ? __ldg(p + TLG_AT(q0 + 1, len, comp)) : 0.0f);
      } else {
        return __ldg(p + TLG_AT(qv, len, comp));
      }
    };
    V cx[D], cd, ck[LJ];
    auto load_ct = [&](int qv) {
#pragma unroll
      for (int g = 0; g < D; ++g) cx[g] = ctx ? ld(ctx, qv, D, g) : A::splat(S(0));
      cd = ctd ? ld(ctd, qv, 1, 0) : A::splat(S(0));
#pragma unroll
      for (int i = 0; i < LJ; ++i) ck[i] = ctk ? ld(ctk, qv, LJ, i) : A::splat(S(0));
    };
    load_ct(0);
    V lacc[NK][D];
#pragma unroll
    for (int j = 0; j < NK; ++j)
#pragma unroll
      for (int g = 0; g < D; ++g) lacc[j][g] = A::splat(S(0));

    for (int qv = 0; qv < nqv; ++qv) {
      const V* tv = tab + (int64_t)qv * K * 4;
      // Partial J(g, d) (at d * D + g) and x(g) over this lane's nodes.
      V jp[LJ], xp[D];
#pragma unroll
      for (int i = 0; i < LJ; ++i) jp[i] = A::splat(S(0));
#pragma unroll
      for (int g = 0; g < D; ++g) xp[g] = A::splat(S(0));
#pragma unroll
      for (int j = 0; j < NK; ++j) {
        V t[4];
        T::row(tv + min(r + G * j, K - 1) * 4, t);
#pragma unroll
        for (int d = 0; d < D; ++d)
#pragma unroll
          for (int g = 0; g < D; ++g) jp[d * D + g] = A::fma(A::splat(xk[j][g]), t[1 + d], jp[d * D + g]);
        if (a.out[0])
#pragma unroll
          for (int g = 0; g < D; ++g) xp[g] = A::fma(A::splat(xk[j][g]), t[0], xp[g]);
      }
#pragma unroll
      for (int m = 1; m < G; m *= 2) {
#pragma unroll
        for (int i = 0; i < LJ; ++i) jp[i] = A::add(jp[i], T::shfl_xor(jp[i], m));
        if (a.out[0])
#pragma unroll
          for (int g = 0; g < D; ++g) xp[g] = A::add(xp[g], T::shfl_xor(xp[g], m));
      }
      V kinv[LJ];
      M::pinv(jp, kinv);
      const V det = M::detj(jp);
      if (r < D) {
        // Row rl of x, J and K^T, selected with compile-time indices (no local memory).
        V xr = xp[0], jr[D], kr[D];
#pragma unroll
        for (int d = 0; d < D; ++d) {
          jr[d] = jp[d * D];
          kr[d] = kinv[d];
        }
#pragma unroll
        for (int g = 1; g < D; ++g)
          if (rl == g) {
            xr = xp[g];
#pragma unroll
            for (int d = 0; d < D; ++d) {
              jr[d] = jp[d * D + g];
              kr[d] = kinv[g * D + d];
            }
          }
        auto st = [&](void* p, int len, int comp, V v) {
          S* f = static_cast<S*>(p);
          if constexpr (SPLIT) {
            f[TLG_AT(2 * qv, len, comp)] = v.x;
            if (2 * qv + 1 < nq) f[TLG_AT(2 * qv + 1, len, comp)] = v.y;
          } else {
            f[TLG_AT(qv, len, comp)] = v;
          }
        };
        if (a.out[0])
          st(a.out[0], D, rl,
             SPLIT ? A::add(A::splat(xh), A::add(A::splat(xl), xr)) : A::add(xr, A::splat(xh)));
        if (a.out[1])
#pragma unroll
          for (int d = 0; d < D; ++d) st(a.out[1], LJ, d * D + rl, jr[d]);
        if (a.out[2] && r == 0) st(a.out[2], 1, 0, det);
        if (a.out[3])
#pragma unroll
          for (int t = 0; t < D; ++t) st(a.out[3], LJ, rl * D + t, kr[t]);
      }
      // Jbar(g, d) at g * D + d: dbar det K(d, g) - sum_t K(t, g) Mt(t, d), with
      // Mt(t, d) = sum_h Kbar(t, h) K(d, h); K(t, h) and Kbar(t, h) at h * D + t.
      V jb[LJ];
      const V s = A::mul(cd, det);
#pragma unroll
      for (int g = 0; g < D; ++g)
#pragma unroll
        for (int d = 0; d < D; ++d) jb[g * D + d] = A::mul(s, kinv[g * D + d]);
#pragma unroll
      for (int t = 0; t < D; ++t)
#pragma unroll
        for (int d = 0; d < D; ++d) {
          V mt = A::mul(ck[t], kinv[d]);
#pragma unroll
          for (int h = 1; h < D; ++h) mt = A::fma(ck[h * D + t], kinv[h * D + d], mt);
#pragma unroll
          for (int g = 0; g < D; ++g) jb[g * D + d] = A::fma(A::neg(kinv[g * D + t]), mt, jb[g * D + d]);
        }
      // The next step's cotangents load while this step's contributions are accumulated.
      V xb[D];
#pragma unroll
      for (int g = 0; g < D; ++g) xb[g] = cx[g];
      if (qv + 1 < nqv) load_ct(qv + 1);
#pragma unroll
      for (int j = 0; j < NK; ++j) {
        V t[4];
        T::row(tv + min(r + G * j, K - 1) * 4, t);
#pragma unroll
        for (int g = 0; g < D; ++g) {
          V acc = A::fma(t[0], xb[g], lacc[j][g]);
#pragma unroll
          for (int d = 0; d < D; ++d) acc = A::fma(jb[g * D + d], t[1 + d], acc);
          lacc[j][g] = acc;
        }
      }
    }
#undef TLG_AT
    // Stage the group's contributions; the warp then writes its cells' rows as one run of
    // 16-byte (8-byte for 2D f32 rows) stores.
#pragma unroll
    for (int j = 0; j < NK; ++j)
      if (j < nown)
#pragma unroll
        for (int g = 0; g < R; ++g) {
          S v = S(0);
          if (g < D) {
            if constexpr (SPLIT) v = __fadd_rn(lacc[j][g].x, lacc[j][g].y);
            else v = lacc[j][g];
          }
          stage[(slot * K + r + G * j) * R + g] = v;
        }
    __syncwarp();
    const int64_t cell0 = __shfl_sync(0xFFFFFFFFu, a.first_cell + c, 0);
    const int64_t nreal = min((int64_t)kVjpCellsPerWarp, a.range_end - cell0);
    if (nreal > 0) {
      using U = typename std::conditional<(R * sizeof(S)) % 16 == 0, uint4, uint2>::type;
      constexpr int UPR = (int)(R * sizeof(S) / sizeof(U));  // units per row
      const U* src = reinterpret_cast<const U*>(stage);
      U* dst = reinterpret_cast<U*>(static_cast<S*>(a.local) + cell0 * (K * R));
      for (int i = lane; i < nreal * (K * UPR); i += 32) dst[i] = src[i];
    }
    __syncwarp();
  }
}

// One contribution row (R values of L) as one vector value.
template <typename L, int R>
struct VjpRow;
template <>
struct VjpRow<float, 4> {
  using T = float4;
  __device__ static T load(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
  __device__ static float get(const T& v, int g) { return g == 0 ? v.x : g == 1 ? v.y : v.z; }
};
template <>
struct VjpRow<float, 2> {
  using T = float2;
  __device__ static T load(const float* p) { return __ldg(reinterpret_cast<const float2*>(p)); }
  __device__ static float get(const T& v, int g) { return g == 0 ? v.x : v.y; }
};
template <>
struct VjpRow<double, 4> {
  struct T {
    double2 a, b;
  };
  __device__ static T load(const double* p) {
    return {__ldg(reinterpret_cast<const double2*>(p)), __ldg(reinterpret_cast<const double2*>(p) + 1)};
  }
  __device__ static double get(const T& v, int g) { return g == 0 ? v.a.x : g == 1 ? v.a.y : v.b.x; }
};
template <>
struct VjpRow<double, 2> {
  using T = double2;
  __device__ static T load(const double* p) { return __ldg(reinterpret_cast<const double2*>(p)); }
  __device__ static double get(const T& v, int g) { return g == 0 ? v.x : v.y; }
};
template <typename L>
struct VjpRow<L, 1> {
  using T = L;
  __device__ static T load(const L* p) { return __ldg(p); }
  __device__ static L get(const T& v, int) { return v; }
};

// A node's running sum of f32 contributions: f64 adds for f64 rows; for f32 rows an unevaluated
// pair hi + lo kept by TwoSum (Knuth) in FP32, whose error per add is captured exactly, so the
// FP64 pipe sees one add per coordinate and node instead of a conversion and an add per entry.
template <typename L>
struct GatherSum {
  double s = 0.0;
  __device__ __forceinline__ void add(L x) { s = __dadd_rn(s, x); }
  __device__ __forceinline__ double value() const { return s; }
};
template <>
struct GatherSum<float> {
  float hi = 0.0f, lo = 0.0f;
  __device__ __forceinline__ void add(float x) {
    const float s = __fadd_rn(hi, x);
    const float bv = __fsub_rn(s, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bv)), __fsub_rn(x, bv));
    hi = s;
    lo = __fadd_rn(lo, err);
  }
  __device__ __forceinline__ double value() const { return __dadd_rn(f2d_exact(hi), f2d_exact(lo)); }
};

// gbar(n, g) = sum over the CSR entries e of node n, in entry order, of local[e * R + g]: in f64
// for f64 rows, as an FP32 TwoSum pair rounded once to f64 for f32 rows.
// A CTA owns 256 consecutive nodes, whose entries are contiguous in the CSR: all its threads
// load the rows of up to 1024 of those entries at a time into shared memory (independent
// vector loads, so many are in flight), then the thread of each node adds the rows of its own
// entries in order. The sums, and their order, do not depend on the launch shape.
constexpr int kGatherNodes = 256;
constexpr int kGatherChunk = 1024;

template <typename L, int D>
__global__ void __launch_bounds__(kGatherNodes) vjp_gather_kernel(const uint32_t* offsets, const uint32_t* entries,
                                                                  int64_t num_nodes, const L* local, double* grad,
                                                                  int add) {
  constexpr int R = vjp_row(D);
  using Row = VjpRow<L, R>;
  __shared__ typename Row::T rows[kGatherChunk];
  for (int64_t n0 = (int64_t)blockIdx.x * kGatherNodes; n0 < num_nodes; n0 += (int64_t)gridDim.x * kGatherNodes) {
    const int64_t n = n0 + threadIdx.x;
    const int64_t n_end = min(n0 + kGatherNodes, num_nodes);
    const uint32_t e0 = offsets[n0], e1 = offsets[n_end];
    uint32_t b = 0, e = 0;
    if (n < num_nodes) {
      b = offsets[n];
      e = offsets[n + 1];
    }
    GatherSum<L> acc[D];
    for (uint32_t c = e0; c < e1; c += kGatherChunk) {
      const uint32_t cn = min((uint32_t)kGatherChunk, e1 - c);
      uint32_t ent[kGatherChunk / kGatherNodes];
#pragma unroll
      for (int u = 0; u < kGatherChunk / kGatherNodes; ++u) {
        const uint32_t i = threadIdx.x + kGatherNodes * u;
        ent[u] = i < cn ? entries[c + i] : 0u;
      }
#pragma unroll
      for (int u = 0; u < kGatherChunk / kGatherNodes; ++u) {
        const uint32_t i = threadIdx.x + kGatherNodes * u;
        if (i < cn) rows[i] = Row::load(local + (int64_t)ent[u] * R);
      }
      __syncthreads();
      const uint32_t lo = max(b, c), hi = min(e, c + cn);
      for (uint32_t i = lo; i < hi; ++i)
#pragma unroll
        for (int g = 0; g < D; ++g) acc[g].add(Row::get(rows[i - c], g));
      __syncthreads();
    }
    // add: the block's sums go onto grad (one f64 addition each), nodes without entries untouched.
    if (n < num_nodes && (!add || e > b))
#pragma unroll
      for (int g = 0; g < D; ++g) grad[n * D + g] = add ? __dadd_rn(grad[n * D + g], acc[g].value()) : acc[g].value();
  }
}

// The adjoint from forward fields already written, for volume cells of any kind (D = 3, K at run
// time): det J and K read back instead of recomputed, so no coordinates and no forward
// contraction. A 16-cell tile of the fields per CTA step: one item per (point, cell) reads the
// cotangents, det J and K (coalesced, the cell fastest) and puts x̄ and J̄ (J̄(g, d) = d̄ det J
// K(d, g) - (K^T K̄ K^T)(g, d)) in shared memory as a record of three 4-vectors (x̄_g, J̄(g, 0..2));
// one item per (cell, group of a.group consecutive nodes), the group fastest, sums over the points
// phi_k x̄ + sum_d dphi_k[d] J̄(., d) from the staged node rows (the record read once per point for
// the group's nodes; split precision's point pairs as two 16-byte loads) and writes the group's
// rows. The host picks the group size and the CTA size (blockDim.x) so that the items fill whole
// warps. Two barriers per tile.
constexpr int kVjpTileMaxGroup = 6;
constexpr int kVjpTileRec = 12;

template <typename F>
__global__ void __launch_bounds__(256) vjp_tile_kernel(const __grid_constant__ VjpArgs a) {
  using A = Ar<F>;
  constexpr int D = 3, LJ = 9, TILE = 16, R = 4, G = kVjpTileMaxGroup, RS = kVjpTileRec;
  constexpr int PN = sizeof(F) == 4 ? 2 : 1;  // points per node row (split: point pairs)
  const int T = blockDim.x;
  __shared__ uint64_t bar;
  extern __shared__ __align__(16) unsigned char smem[];
  if (!stage_table(a.tab, smem, a.tab_bytes, &bar, a.err)) return;
  const F* tab = reinterpret_cast<const F*>(smem);
  F* V = reinterpret_cast<F*>(smem + (a.tab_bytes + 15) / 16 * 16);
  const int K = a.k_runtime, nq = a.num_points, grp = a.group;
  const int ngroups = (K + grp - 1) / grp;
  const F* ctx = static_cast<const F*>(a.ct[0]);
  const F* ctd = static_cast<const F*>(a.ct[1]);
  const F* ctk = static_cast<const F*>(a.ct[2]);
  const F* fdet = static_cast<const F*>(a.out[2]);
  const F* fk = static_cast<const F*>(a.out[3]);
  const int64_t ntiles = a.padded / TILE;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t tq = (a.out_first_cell / TILE + tile) * nq;
    for (int it = threadIdx.x; it < nq * TILE; it += T) {
      const int q = it / TILE, l = it % TILE;
#define TLG_AT(len, comp) (((tq + q) * (len) + (comp)) * TILE + l)
      F xb[D], kb[LJ], kinv[LJ], jb[LJ];
#pragma unroll
      for (int g = 0; g < D; ++g) xb[g] = ctx ? __ldg(ctx + TLG_AT(D, g)) : F(0);
      const F db = ctd ? __ldg(ctd + TLG_AT(1, 0)) : F(0);
#pragma unroll
      for (int i = 0; i < LJ; ++i) kb[i] = ctk ? __ldg(ctk + TLG_AT(LJ, i)) : F(0);
      const F det = __ldg(fdet + TLG_AT(1, 0));
#pragma unroll
      for (int i = 0; i < LJ; ++i) kinv[i] = __ldg(fk + TLG_AT(LJ, i));
#undef TLG_AT
      // J̄(g, d) at g * D + d; K(t, h) and K̄(t, h) at h * D + t.
      const F s = A::mul(db, det);
#pragma unroll
      for (int g = 0; g < D; ++g)
#pragma unroll
        for (int d = 0; d < D; ++d) jb[g * D + d] = A::mul(s, kinv[g * D + d]);
      if (ctk) {
#pragma unroll
        for (int t = 0; t < D; ++t)
#pragma unroll
          for (int d = 0; d < D; ++d) {
            F mt = A::mul(kb[t], kinv[d]);
#pragma unroll
            for (int h = 1; h < D; ++h) mt = A::fma(kb[h * D + t], kinv[h * D + d], mt);
#pragma unroll
            for (int g = 0; g < D; ++g) jb[g * D + d] = A::fma(A::neg(kinv[g * D + t]), mt, jb[g * D + d]);
          }
      }
      F* rec = V + ((size_t)q * TILE + l) * RS;
#pragma unroll
      for (int g = 0; g < D; ++g) Vec4<F>::put(rec + 4 * g, xb[g], jb[g * D], jb[g * D + 1], jb[g * D + 2]);
    }
    __syncthreads();
    const int64_t cell0 = a.first_cell + tile * TILE;
    for (int it = threadIdx.x; it < ngroups * TILE; it += T) {
      const int l = it / ngroups, gi = it - (it / ngroups) * ngroups;
      const int k0 = gi * grp;
      const int64_t cell = cell0 + l;
      if (cell >= a.range_end) continue;
      F acc[G][D];
#pragma unroll
      for (int u = 0; u < G; ++u)
#pragma unroll
        for (int g = 0; g < D; ++g) acc[u][g] = F(0);
      for (int r = 0; r < (nq + PN - 1) / PN; ++r) {
#pragma unroll
        for (int h = 0; h < PN; ++h) {
          const int q = r * PN + h;
          if (q >= nq) break;
          F v[RS];
          const F* rec = V + ((size_t)q * TILE + l) * RS;
#pragma unroll
          for (int g = 0; g < D; ++g) Vec4<F>::get(rec + 4 * g, v + 4 * g);
#pragma unroll
          for (int u = 0; u < G; ++u) {
            if (u < grp && k0 + u < K) {
              // Node k0 + u's row at pair r: phi, dphi_0..2, PN points each.
              F t[4 * PN];
              const F* row = tab + ((size_t)r * K + k0 + u) * 4 * PN;
              Vec4<F>::get(row, t);
              if constexpr (PN == 2) Vec4<F>::get(row + 4, t + 4);
#pragma unroll
              for (int g = 0; g < D; ++g) {
                F s0 = A::fma(t[h], v[4 * g], acc[u][g]);
#pragma unroll
                for (int d = 0; d < D; ++d) s0 = A::fma(t[(1 + d) * PN + h], v[4 * g + 1 + d], s0);
                acc[u][g] = s0;
              }
            }
          }
        }
      }
      F* base = static_cast<F*>(a.local) + (cell * K + k0) * R;
#pragma unroll
      for (int u = 0; u < G; ++u)
        if (u < grp && k0 + u < K) Vec4<F>::put(base + u * R, acc[u][0], acc[u][1], acc[u][2], F(0));
    }
    __syncthreads();
  }
}

// The group size and CTA size of vjp_tile_kernel for K nodes: the pair with the most useful work
// per issued instruction — the share of whole warps its items (16 cells x groups) fill, times the
// share of its groups' node slots that are nodes, times the share of a node's per-point
// instructions (12 FMA and a row load) that are not the record's three loads split over the group —
// ties to the larger group.
inline void vjp_tile_shape(int k, int* group, int* threads) {
  double best = -1.0;
  *group = 1;
  *threads = 32;
  for (int g = 1; g <= kVjpTileMaxGroup; ++g) {
    const int groups = (k + g - 1) / g;
    const int items = 16 * groups;
    const int t = items >= 256 ? 256 : (items + 31) / 32 * 32;
    const int rounds = (items + t - 1) / t;
    const double score = (double)items / (rounds * t) * ((double)k / (groups * g)) * (13.0 / (13.0 + 3.0 / g));
    if (score >= best - 1e-12) {
      best = score;
      *group = g;
      *threads = t;
    }
  }
}

// The node sums of several blocks in one pass over the nodes (an adjoint batch's blocks in block
// order): per node, the first block's sum (zero without entries) or, with `add`, the gradient's
// value, then each further block's sum added where the node has entries, with the sums and their
// order of vjp_gather_kernel's launches one block after another, so the gradient is the same bit
// for bit; written once. A CTA skips a block none of its nodes has entries in.
constexpr int kGatherMaxBlocks = 8;

struct GatherBlocks {
  const uint32_t* offsets[kGatherMaxBlocks];
  const uint32_t* entries[kGatherMaxBlocks];
  const void* local[kGatherMaxBlocks];
  int count;
};

template <typename L, int D>
__global__ void __launch_bounds__(kGatherNodes, 6) vjp_gather_blocks_kernel(const __grid_constant__ GatherBlocks gb,
                                                                         int64_t num_nodes, double* grad, int add) {
  constexpr int R = vjp_row(D);
  using Row = VjpRow<L, R>;
  __shared__ typename Row::T rows[kGatherChunk];
  for (int64_t n0 = (int64_t)blockIdx.x * kGatherNodes; n0 < num_nodes; n0 += (int64_t)gridDim.x * kGatherNodes) {
    const int64_t n = n0 + threadIdx.x;
    const int64_t n_end = min(n0 + kGatherNodes, num_nodes);
    double v[D];
#pragma unroll
    for (int g = 0; g < D; ++g) v[g] = 0.0;
    bool have = false;  // add: v holds the gradient's value
    // The blocks' CSR ranges of this CTA's nodes, loaded together before the blocks' passes (one
    // latency, not one per block: most blocks of a batch have no entries in most CTAs' ranges).
    uint32_t E0[kGatherMaxBlocks], E1[kGatherMaxBlocks];
#pragma unroll
    for (int bi = 0; bi < kGatherMaxBlocks; ++bi) {
      E0[bi] = E1[bi] = 0u;
      if (bi < gb.count) {
        E0[bi] = gb.offsets[bi][n0];
        E1[bi] = gb.offsets[bi][n_end];
      }
    }
#pragma unroll
    for (int bi = 0; bi < kGatherMaxBlocks; ++bi) {
      if (bi >= gb.count) break;
      const uint32_t* offsets = gb.offsets[bi];
      const uint32_t* entries = gb.entries[bi];
      const L* local = static_cast<const L*>(gb.local[bi]);
      const uint32_t e0 = E0[bi], e1 = E1[bi];
      uint32_t b = e0, e = e0;
      if (e1 > e0 && n < num_nodes) {
        b = offsets[n];
        e = offsets[n + 1];
      }
      GatherSum<L> acc[D];
      for (uint32_t c = e0; c < e1; c += kGatherChunk) {
        const uint32_t cn = min((uint32_t)kGatherChunk, e1 - c);
        uint32_t ent[kGatherChunk / kGatherNodes];
#pragma unroll
        for (int u = 0; u < kGatherChunk / kGatherNodes; ++u) {
          const uint32_t i = threadIdx.x + kGatherNodes * u;
          ent[u] = i < cn ? entries[c + i] : 0u;
        }
#pragma unroll
        for (int u = 0; u < kGatherChunk / kGatherNodes; ++u) {
          const uint32_t i = threadIdx.x + kGatherNodes * u;
          if (i < cn) rows[i] = Row::load(local + (int64_t)ent[u] * R);
        }
        __syncthreads();
        const uint32_t lo = max(b, c), hi = min(e, c + cn);
        for (uint32_t i = lo; i < hi; ++i)
#pragma unroll
          for (int g = 0; g < D; ++g) acc[g].add(Row::get(rows[i - c], g));
        __syncthreads();
      }
      if (n >= num_nodes) continue;
      if (bi == 0 && !add) {
#pragma unroll
        for (int g = 0; g < D; ++g) v[g] = acc[g].value();
      } else if (e > b) {
        if (add && !have) {
#pragma unroll
          for (int g = 0; g < D; ++g) v[g] = grad[n * D + g];
          have = true;
        }
#pragma unroll
        for (int g = 0; g < D; ++g) v[g] = __dadd_rn(v[g], acc[g].value());
      }
    }
    if (n < num_nodes && (!add || have))
#pragma unroll
      for (int g = 0; g < D; ++g) grad[n * D + g] = v[g];
  }
}

}  // namespace tlg
