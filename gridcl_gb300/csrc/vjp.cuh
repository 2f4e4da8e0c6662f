// Adjoint (vector-Jacobian product) of the geometric factors, codimension 0 (TD = GD = D).
//
// For a scalar L(x, J, det J, K) with cotangents xbar = dL/dx, dbar = dL/d(det J) and
// Kbar = dL/dK at every point, the cotangent of the node coordinates is
//   gbar(n, g) = sum over the (cell, k) with dofmap(cell, k) = n of
//                sum_q [ phi_k(q) xbar(q, g) + sum_d Jbar(q)(g, d) dphi_k(q)[d] ],
//   Jbar(g, d) = dbar det J K(d, g) - (K^T Kbar K^T)(g, d),
// from d det J = det J tr(K dJ) and dK = -K dJ K. J, det J and K are recomputed here, not read.
//
// vjp_kernel writes each cell's contributions L(cell, k, g) (layout [k][g][cell], cells fastest,
// as the E-vector) and, when asked, the forward fields of the same points in the same pass (the
// fused forward + adjoint). vjp_gather then sums, for every node, the contributions listed by the
// node's CSR entries in entry order, in f64: deterministic.
//
// Four lanes per cell: lane g < D owns coordinate g (its node coordinates, row g of J, its
// contributions); J is assembled from the rows by shuffles inside the group, det J and K are
// computed by every lane of the group. SPLIT: f64 nodes shifted by node 0 in f64, FP32
// arithmetic, f32 cotangents, contributions and fields; otherwise f64 throughout.
#pragma once

#include <cstdint>
#include <type_traits>

#include "eval.cuh"

namespace tlg {

struct VjpArgs {
  const void* nodes;
  const uint32_t* dofmap;
  const unsigned char* tab;  // phi [Q][K] | dphi [Q][K][D] in F (F = float with SPLIT)
  const void* ct[3];         // cotangents: points, detj, pinv (tile 16 chunks) or null
  void* out[4];              // fused forward fields: points, jacobian, detj, pinv, or null
  void* local;               // contributions [K][D][local_stride] of F
  int* err;
  int64_t first_cell, padded, out_first_cell, last_cell, range_end, local_stride;
  double origin[3];
  uint32_t last_node, tab_bytes, off_dphi;
  int num_points;
};

constexpr int kVjpGroup = 4;

template <bool SPLIT, int D, int K>
__global__ void __launch_bounds__(kEvalThreads) vjp_kernel(const __grid_constant__ VjpArgs a) {
  using F = typename std::conditional<SPLIT, float, double>::type;
  using A = Ar<F>;
  using M = Factors<F, D, D>;
  constexpr int TILE = 16;
  constexpr int LJ = D * D;
  constexpr int K0 = SPLIT ? 1 : 0;
  __shared__ uint64_t bar;
  extern __shared__ __align__(16) unsigned char smem[];
  stage_table(a.tab, smem, a.tab_bytes, &bar, a.err);
  const F* phi = reinterpret_cast<const F*>(smem);
  const F* dphi = reinterpret_cast<const F*>(smem + a.off_dphi);
  const int nq = a.num_points;
  const int lane = threadIdx.x % 32;
  const int g = threadIdx.x % kVjpGroup;
  const int gl = g < D ? g : D - 1;  // idle lanes mirror the last coordinate
  const int group_base = lane & ~(kVjpGroup - 1);
  const int cells_per_cta = kEvalThreads / kVjpGroup;
  const F* ctx = static_cast<const F*>(a.ct[0]);
  const F* ctd = static_cast<const F*>(a.ct[1]);
  const F* ctk = static_cast<const F*>(a.ct[2]);

  for (int64_t c = (int64_t)blockIdx.x * cells_per_cta + threadIdx.x / kVjpGroup; c < a.padded;
       c += (int64_t)gridDim.x * cells_per_cta) {
    const int64_t cell = min(a.first_cell + c, a.last_cell);
    const bool real = a.first_cell + c < a.range_end;
    uint32_t idx[K];
    load_row<K>(a.dofmap + cell * K, idx);
    F xk[K];
    F xh = F(0), xl = F(0);
    if constexpr (SPLIT) {
      const double* nodes = static_cast<const double*>(a.nodes);
      const double x0 = __ldg(nodes + (int64_t)min(idx[0], a.last_node) * D + gl);
      xk[0] = 0.0f;
#pragma unroll
      for (int k = 1; k < K; ++k)
        xk[k] = __double2float_rn(__ldg(nodes + (int64_t)min(idx[k], a.last_node) * D + gl) - x0);
      const double v = x0 + a.origin[gl];
      xh = __double2float_rn(v);
      xl = __double2float_rn(v - (double)xh);
    } else {
      const double* nodes = static_cast<const double*>(a.nodes);
#pragma unroll
      for (int k = 0; k < K; ++k) xk[k] = __ldg(nodes + (int64_t)min(idx[k], a.last_node) * D + gl);
      xh = (F)a.origin[gl];
    }
    const int64_t o = a.out_first_cell + c;
    const int64_t tile_idx = o / TILE;
    const int l16 = (int)(o % TILE);
    // Element (tile, q, comp, l16) of a tiled field with `len` components:
    // ((tile * Q + q) * len + comp) * 16 + l16.
    const int64_t tq = tile_idx * nq;
#define TLG_AT(q, len, comp) (((tq + (q)) * (len) + (comp)) * TILE + l16)
    F lacc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) lacc[k] = F(0);

    for (int q = 0; q < nq; ++q) {
      const F* dq = dphi + q * K * D;
      F jr[D];
#pragma unroll
      for (int d = 0; d < D; ++d) jr[d] = A::mul(xk[K0], dq[K0 * D + d]);
#pragma unroll
      for (int k = K0 + 1; k < K; ++k)
#pragma unroll
        for (int d = 0; d < D; ++d) jr[d] = A::fma(xk[k], dq[k * D + d], jr[d]);
      F j[LJ];
#pragma unroll
      for (int gg = 0; gg < D; ++gg)
#pragma unroll
        for (int d = 0; d < D; ++d) j[d * D + gg] = __shfl_sync(0xFFFFFFFFu, jr[d], group_base + gg);
      F kinv[LJ];
      M::pinv(j, kinv);
      const F det = M::detj(j);
      // Row gl of K^T: krow[t] = K(t, gl), selected with compile-time indices (no local memory).
      F krow[D];
#pragma unroll
      for (int t = 0; t < D; ++t) krow[t] = kinv[t];
#pragma unroll
      for (int gg = 1; gg < D; ++gg)
        if (gl == gg)
#pragma unroll
          for (int t = 0; t < D; ++t) krow[t] = kinv[gg * D + t];
      if (g < D) {
        if (a.out[0]) {
          const F* w = phi + q * K;
          F s = A::mul(xk[K0], w[K0]);
#pragma unroll
          for (int k = K0 + 1; k < K; ++k) s = A::fma(xk[k], w[k], s);
          s = SPLIT ? A::add(xh, A::add(xl, s)) : A::add(s, xh);
          static_cast<F*>(a.out[0])[TLG_AT(q, D, g)] = s;
        }
        if (a.out[1])
#pragma unroll
          for (int d = 0; d < D; ++d) static_cast<F*>(a.out[1])[TLG_AT(q, LJ, d * D + g)] = jr[d];
        if (a.out[2] && g == 0) static_cast<F*>(a.out[2])[TLG_AT(q, 1, 0)] = det;
        if (a.out[3])
#pragma unroll
          for (int t = 0; t < D; ++t) static_cast<F*>(a.out[3])[TLG_AT(q, LJ, g * D + t)] = krow[t];
      }
      // Jbar(gl, d) = dbar det K(d, gl) - sum_t K(t, gl) M(t, d), M(t, d) = sum_h Kbar(t, h) K(d, h).
      F jbar[D];
#pragma unroll
      for (int d = 0; d < D; ++d) jbar[d] = F(0);
      if (ctd) {
        const F s = A::mul(__ldg(ctd + TLG_AT(q, 1, 0)), det);
#pragma unroll
        for (int d = 0; d < D; ++d) jbar[d] = A::mul(s, krow[d]);
      }
      if (ctk) {
        F kb[LJ];
#pragma unroll
        for (int i = 0; i < LJ; ++i) kb[i] = __ldg(ctk + TLG_AT(q, LJ, i));
#pragma unroll
        for (int d = 0; d < D; ++d) {
          F acc = jbar[d];
#pragma unroll
          for (int t = 0; t < D; ++t) {
            F m = A::mul(kb[t], kinv[d]);  // Kbar(t, 0) K(d, 0); K(t, h) at h * D + t
#pragma unroll
            for (int h = 1; h < D; ++h) m = A::fma(kb[h * D + t], kinv[h * D + d], m);
            acc = A::fma(A::neg(krow[t]), m, acc);
          }
          jbar[d] = acc;
        }
      }
      F xb = F(0);
      if (ctx) xb = __ldg(ctx + TLG_AT(q, D, gl));
      const F* w = phi + q * K;
#pragma unroll
      for (int k = 0; k < K; ++k) {
        F acc = A::fma(w[k], xb, lacc[k]);
#pragma unroll
        for (int d = 0; d < D; ++d) acc = A::fma(jbar[d], dq[k * D + d], acc);
        lacc[k] = acc;
      }
    }
#undef TLG_AT
    if (real && g < D) {
      F* loc = static_cast<F*>(a.local);
#pragma unroll
      for (int k = 0; k < K; ++k) loc[((int64_t)k * D + g) * a.local_stride + cell] = lacc[k];
    }
  }
}

// gbar(n, g) = sum over the CSR entries e of node n, in entry order, of L(e / K, e % K, g), in f64.
template <typename L, int D>
__global__ void __launch_bounds__(256) vjp_gather_kernel(const uint32_t* offsets, const uint32_t* entries,
                                                         int64_t num_nodes, int K, const L* local,
                                                         int64_t local_stride, double* grad) {
  for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < num_nodes;
       n += (int64_t)gridDim.x * blockDim.x) {
    double acc[D];
#pragma unroll
    for (int g = 0; g < D; ++g) acc[g] = 0.0;
    const uint32_t b = offsets[n], e = offsets[n + 1];
    for (uint32_t i = b; i < e; ++i) {
      const uint32_t ent = entries[i];
      const int64_t cell = ent / (uint32_t)K;
      const int k = (int)(ent - (uint32_t)cell * (uint32_t)K);
#pragma unroll
      for (int g = 0; g < D; ++g) acc[g] += (double)local[((int64_t)k * D + g) * local_stride + cell];
    }
#pragma unroll
    for (int g = 0; g < D; ++g) grad[n * D + g] = acc[g];
  }
}

}  // namespace tlg
