// The cooperative evaluation kernel (the reference's cooperative strategy,
// tetraloma-geometry/src/cooperative/mod.rs:1-30 and cooperative/factors.rs:29-93): the node sums
// of a cell split over a group of lanes.
//
// Four lanes per cell (eight cells per warp). Lane l of a group holds the coordinates of the
// cell's nodes l, l + 4, l + 8, ... in registers (up to KPL of them, K at run time), loaded once
// per cell; each lane's partial sums run over its nodes in ascending order. Points go in groups of
// four: every lane forms the partial X and J of the four points, then a reduce-scatter over the
// group (two butterfly steps, lanes 2 apart then 1 apart) leaves lane p with the complete sums of
// point p of the group, (s0 + s2) + (s1 + s3) over the lanes' partials, and lane p runs that
// point's epilogue (det J, K, normals, facet normals, the stores; in split precision the condition
// estimate and the FP64 recompute). phi, dphi and the reference normals are read from shared
// memory where they take at most a third of it, else from global memory (L1-cached).
//
// Compared with the loops kernel (one cell per thread, each node's coordinates gathered again at
// every point) the coordinates are gathered once, and a lane keeps K / 4 of them instead of K.
#pragma once

#include <cstdint>
#include <type_traits>

#include "eval.cuh"

namespace tlg {

struct CoopArgs {
  const void* nodes;
  const uint32_t* dofmap;
  const uint32_t* flags;
  const unsigned char* tab;  // phi [Q][K] at 0, dphi [Q][K][TD] at off_dphi, refn [Q][TD] at off_refn
                             // (the arithmetic's type; the first tab_bytes staged unless tab_global);
                             // split: the f64 dphi [Q][K][TD] at off_dphi64, read from global memory
  void* out[6];              // points, jacobian, detj, pinv, normals, facet normals
  int* err;
  unsigned long long* recomputed;
  int64_t first_cell, padded, range_cells, out_first_cell, last_cell, last_flag;
  double origin[3];
  float cond_limit;
  uint32_t last_node, tab_bytes, off_dphi, off_refn, off_dphi64, mask;
  int num_points, k, tile_shift, tab_global;
};

constexpr int kCoopLanes = 4;

template <typename F, bool SPLIT, int TD, int GD, int KPL>
__global__ void __launch_bounds__(kEvalThreads) coop_kernel(const __grid_constant__ CoopArgs a) {
  using NT = typename std::conditional<SPLIT, double, F>::type;
  using A = Ar<F>;
  using M = Factors<F, TD, GD>;
  constexpr int LJ = TD * GD, NV = GD + LJ, G = kCoopLanes;
  __shared__ uint64_t bar;
  extern __shared__ __align__(16) unsigned char smem[];
  const unsigned char* tabs = a.tab;
  if (!a.tab_global) {
    if (!stage_table(a.tab, smem, a.tab_bytes, &bar, a.err)) return;
    tabs = smem;
  }
  const F* phi = reinterpret_cast<const F*>(tabs);
  const F* dphi = reinterpret_cast<const F*>(tabs + a.off_dphi);
  const F* refn = reinterpret_cast<const F*>(tabs + a.off_refn);
  const NT* nodes = static_cast<const NT*>(a.nodes);
  const int K = a.k, nq = a.num_points;
  const uint32_t mask = a.mask;
  const int sub = threadIdx.x & (G - 1);
  const int warp_lane = threadIdx.x & 31;
  const int64_t cells_per_cta = kEvalThreads / G;

  // Warps walk runs of 8 cells together (the shuffles need the whole warp); lanes past the
  // padded range work on the last cell and store nothing.
  for (int64_t cw = (int64_t)blockIdx.x * cells_per_cta + (threadIdx.x & ~31) / G; cw < a.padded;
       cw += (int64_t)gridDim.x * cells_per_cta) {
    const int64_t c = cw + warp_lane / G;
    const bool live = c < a.padded;
    const int64_t cell = min(a.first_cell + min(c, a.padded - 1), a.last_cell);
    const uint32_t* row = a.dofmap + cell * K;
    double x0[GD];
    F xh[GD], xl[GD];
    if constexpr (SPLIT) {
      const uint32_t n0 = min(__ldg(row), a.last_node);
#pragma unroll
      for (int g = 0; g < GD; ++g) {
        x0[g] = __ldg(nodes + (int64_t)n0 * GD + g);
        const double v = x0[g] + a.origin[g];
        xh[g] = d2f_rn(v);
        xl[g] = d2f_rn(v - f2d_exact(xh[g]));
      }
    } else {
#pragma unroll
      for (int g = 0; g < GD; ++g) {
        x0[g] = 0.0;
        xh[g] = (F)a.origin[g];
        xl[g] = F(0);
      }
    }
    F xk[KPL][GD];
#pragma unroll
    for (int i = 0; i < KPL; ++i) {
      const int k = sub + G * i;
#pragma unroll
      for (int g = 0; g < GD; ++g) xk[i][g] = F(0);
      if (k < K) {
        const uint32_t n = min(__ldg(row + k), a.last_node);
#pragma unroll
        for (int g = 0; g < GD; ++g) {
          const NT v = __ldg(nodes + (int64_t)n * GD + g);
          if constexpr (SPLIT) xk[i][g] = d2f_rn(v - x0[g]);
          else xk[i][g] = v;
        }
      }
    }
    F sign = F(1);
    if ((mask & kOutNormals) && a.flags != nullptr && a.last_flag >= 0) {
      const uint32_t f = __ldg(a.flags + min(a.first_cell + min(c, a.padded - 1), a.last_flag));
      sign = (f & 1u) ? F(-1) : F(1);
    }
    const int64_t o = a.out_first_cell + min(c, a.padded - 1);
    const int64_t tile_idx = o >> a.tile_shift;
    const int tlane = (int)(o & ((1 << a.tile_shift) - 1));

    for (int q0 = 0; q0 < nq; q0 += G) {
      // Partial X and J of the group's four points over this lane's nodes.
      F s[G][NV];
#pragma unroll
      for (int p = 0; p < G; ++p) {
        const int q = min(q0 + p, nq - 1);
#pragma unroll
        for (int v = 0; v < NV; ++v) s[p][v] = F(0);
#pragma unroll
        for (int i = 0; i < KPL; ++i) {
          const int k = sub + G * i;
          if (k < K) {
            const F w = phi[q * K + k];
#pragma unroll
            for (int g = 0; g < GD; ++g) s[p][g] = A::fma(xk[i][g], w, s[p][g]);
#pragma unroll
            for (int d = 0; d < TD; ++d) {
              const F wd = dphi[(q * K + k) * TD + d];
#pragma unroll
              for (int g = 0; g < GD; ++g) s[p][GD + d * GD + g] = A::fma(xk[i][g], wd, s[p][GD + d * GD + g]);
            }
          }
        }
      }
      // Reduce-scatter: lanes 2 apart exchange the halves they do not keep (lane bit 1 keeps
      // points 2-3), then lanes 1 apart (lane bit 0 keeps the odd point).
      const bool hi2 = (sub & 2) != 0, hi1 = (sub & 1) != 0;
      F h[2][NV];
#pragma unroll
      for (int p = 0; p < 2; ++p)
#pragma unroll
        for (int v = 0; v < NV; ++v) {
          const F keep = hi2 ? s[2 + p][v] : s[p][v];
          const F send = hi2 ? s[p][v] : s[2 + p][v];
          h[p][v] = A::add(keep, __shfl_xor_sync(0xFFFFFFFFu, send, 2));
        }
      F t[NV];
#pragma unroll
      for (int v = 0; v < NV; ++v) {
        const F keep = hi1 ? h[1][v] : h[0][v];
        const F send = hi1 ? h[0][v] : h[1][v];
        t[v] = A::add(keep, __shfl_xor_sync(0xFFFFFFFFu, send, 1));
      }
      const int q = q0 + sub;
      if (!live || q >= nq) continue;
      F* x = t;
      F* j = t + GD;
      if (mask & kOutPoints) {
        F xp[GD];
#pragma unroll
        for (int g = 0; g < GD; ++g) xp[g] = SPLIT ? A::add(xh[g], A::add(xl[g], x[g])) : A::add(x[g], xh[g]);
        store_point(static_cast<F*>(a.out[0]), tile_idx, q, nq, GD, tlane, a.tile_shift, xp, GD);
      }
      if ((mask & ~kOutPoints) == 0) continue;
      F kk[LJ];
      M::pinv(j, kk);
      F dj = M::detj(j);
      if constexpr (SPLIT) {
        const F kap = M::condition(j, kk);
        if (!(kap <= a.cond_limit) && (mask & (kOutJacobian | kOutDetJ | kOutPinv))) {
          float jr[LJ], kr[LJ], dr;
          recompute_f64_rt<TD, GD>(static_cast<const double*>(a.nodes), row, K, a.last_node,
                                   reinterpret_cast<const double*>(a.tab + a.off_dphi64) + (int64_t)q * K * TD,
                                   jr, &dr, kr, 1);
#pragma unroll
          for (int i = 0; i < LJ; ++i) {
            j[i] = jr[i];
            kk[i] = kr[i];
          }
          dj = dr;
          if (a.recomputed && c < a.range_cells) atomicAdd(a.recomputed, 1ull);
        }
      }
      if (mask & kOutJacobian) store_point(static_cast<F*>(a.out[1]), tile_idx, q, nq, LJ, tlane, a.tile_shift, j, LJ);
      if (mask & kOutDetJ) store_point(static_cast<F*>(a.out[2]), tile_idx, q, nq, 1, tlane, a.tile_shift, &dj, 1);
      if (mask & kOutPinv) store_point(static_cast<F*>(a.out[3]), tile_idx, q, nq, LJ, tlane, a.tile_shift, kk, LJ);
      if constexpr (TD == GD) {
        if (mask & kOutFacetNormals) {
          F n[GD];
          M::facet_normal(kk, refn + q * TD, n);
          store_point(static_cast<F*>(a.out[5]), tile_idx, q, nq, GD, tlane, a.tile_shift, n, GD);
        }
      }
      if constexpr (TD + 1 == GD) {
        if (mask & kOutNormals) {
          F n[GD];
          M::normal(j, sign, n);
          store_point(static_cast<F*>(a.out[4]), tile_idx, q, nq, GD, tlane, a.tile_shift, n, GD);
        }
      }
    }
  }
}

}  // namespace tlg
