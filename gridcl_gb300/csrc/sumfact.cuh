// Sum-factorised evaluation for quadrilaterals and hexahedra at tensor-product point sets
// (the reference's sum-factorised strategy, tetraloma-geometry/src/sumfact/tensor.rs:66-432).
//
// A Q_{N-1} Lagrange basis is the product of 1D Lagrange bases, phi_{ijk}(x, y, z) =
// l_i(x) l_j(y) l_k(z), and a tensor rule's point (a, b, c) is (u0_a, u1_b, u2_c). X and J at all
// points then follow by contracting one direction at a time:
//   U_g[j][i] = sum_k x_{ijk,g} B2[c][k],  V_g[j][i] = sum_k x_{ijk,g} D2[c][k]     (plane c)
//   UU_g[i] = sum_j U_g[j][i] B1[b][j], UD_g[i] = sum_j U_g[j][i] D1[b][j],
//   VU_g[i] = sum_j V_g[j][i] B1[b][j]                                                 (row b)
//   X_g = sum_i UU_g[i] B0[a][i], J(g, 0) = sum_i UU_g[i] D0[a][i],
//   J(g, 1) = sum_i UD_g[i] B0[a][i], J(g, 2) = sum_i VU_g[i] B0[a][i]                (point a)
// with B_d[a][i] = l_i(u_d[a]) and D_d[a][i] = l_i'(u_d[a]): N^3 M (2) + N^2 M^2 (3) + N M^3 (4)
// multiply-adds per coordinate instead of N^3 M^3 (4). Quadrilaterals contract two directions.
//
// One cell per thread, as the other evaluation kernels (consecutive threads write consecutive
// tile lanes). The cell's coordinates in lexicographic node order (the table's permutation maps
// a lexicographic index to the Lagrange node) go to the thread's slots in shared memory,
// interleaved over threads so that the slot accesses of a warp fall in distinct banks; one
// plane's intermediates live in registers. The point epilogue (det J, K, normals, the condition
// estimate and the FP64 recompute of split precision) is that of the other kernels.
#pragma once

#include <cstdint>
#include <type_traits>

#include "eval.cuh"

namespace tlg {

struct SfArgs {
  const void* nodes;
  const uint32_t* dofmap;
  const uint32_t* flags;
  const unsigned char* tab;  // staged: B_d [m_d][N], D_d [m_d][N] per direction, perm [K] u32
  const double* dphi64;      // split: the f64 derivative table [Q][K][TD] (global) of the recompute
  void* out[6];              // points, jacobian, detj, pinv, normals (facet normals: no tensor rule)
  int* err;
  unsigned long long* recomputed;
  int64_t first_cell, padded, range_cells, out_first_cell, last_cell, last_flag;
  double origin[3];
  float cond_limit;
  uint32_t last_node, tab_bytes, off_b[3], off_d[3], off_perm, mask;
  int m[3];  // points per direction
  int num_points;
  int tile_shift;  // log2 of the output tile
};

// Shared memory of the coordinate slots: K * GD values of F per thread.
inline size_t sumfact_slot_bytes(int k, int gd, size_t f_bytes) { return (size_t)k * gd * kEvalThreads * f_bytes; }

// One point's outputs from X (relative, before the origin) and J.
template <typename F, bool SPLIT, int TD, int GD>
__device__ __forceinline__ void sf_point(const SfArgs& a, int q, int64_t tile_idx, int lane, F* x, F* j, F sign,
                                         const F* xh, const F* xl, const uint32_t* row, int K, int64_t c) {
  constexpr int LJ = TD * GD;
  using A = Ar<F>;
  using M = Factors<F, TD, GD>;
  const int nq = a.num_points;
  const uint32_t mask = a.mask;
  if (mask & kOutPoints) {
#pragma unroll
    for (int g = 0; g < GD; ++g) x[g] = SPLIT ? A::add(xh[g], A::add(xl[g], x[g])) : A::add(x[g], xh[g]);
    store_point(static_cast<F*>(a.out[0]), tile_idx, q, nq, GD, lane, a.tile_shift, x, GD);
  }
  if ((mask & ~kOutPoints) == 0) return;
  F kk[LJ];
  if ((mask & kOutPinv) || SPLIT) M::pinv(j, kk);
  F dj = (mask & kOutDetJ) || SPLIT ? M::detj(j) : F(0);
  if constexpr (SPLIT) {
    const F kap = M::condition(j, kk);
    if (!(kap <= a.cond_limit) && (mask & (kOutJacobian | kOutDetJ | kOutPinv))) {
      float jr[LJ], kr[LJ], dr;
      recompute_f64_rt<TD, GD>(static_cast<const double*>(a.nodes), row, K, a.last_node,
                               a.dphi64 + (int64_t)q * K * TD, jr, &dr, kr, 1);
#pragma unroll
      for (int i = 0; i < LJ; ++i) {
        j[i] = jr[i];
        kk[i] = kr[i];
      }
      dj = dr;
      if (a.recomputed && c < a.range_cells) atomicAdd(a.recomputed, 1ull);
    }
  }
  if (mask & kOutJacobian) store_point(static_cast<F*>(a.out[1]), tile_idx, q, nq, LJ, lane, a.tile_shift, j, LJ);
  if (mask & kOutDetJ) store_point(static_cast<F*>(a.out[2]), tile_idx, q, nq, 1, lane, a.tile_shift, &dj, 1);
  if (mask & kOutPinv) store_point(static_cast<F*>(a.out[3]), tile_idx, q, nq, LJ, lane, a.tile_shift, kk, LJ);
  if constexpr (TD + 1 == GD) {
    if (mask & kOutNormals) {
      F n[GD];
      M::normal(j, sign, n);
      store_point(static_cast<F*>(a.out[4]), tile_idx, q, nq, GD, lane, a.tile_shift, n, GD);
    }
  }
}

// F: arithmetic and output type; SPLIT: f64 nodes shifted by node 0 and rounded to F = float.
template <typename F, bool SPLIT, int TD, int GD, int N>
__global__ void __launch_bounds__(kEvalThreads) sumfact_kernel(const __grid_constant__ SfArgs a) {
  using NT = typename std::conditional<SPLIT, double, F>::type;  // node type
  using A = Ar<F>;
  constexpr int K = TD == 3 ? N * N * N : N * N;
  constexpr int LJ = TD * GD;
  constexpr int T = kEvalThreads;
  __shared__ uint64_t bar;
  extern __shared__ __align__(16) unsigned char smem[];
  stage_table(a.tab, smem, a.tab_bytes, &bar, a.err);
  F* xs = reinterpret_cast<F*>(smem + (a.tab_bytes + 15) / 16 * 16) + threadIdx.x;
  const uint32_t* perm = reinterpret_cast<const uint32_t*>(smem + a.off_perm);
  const F* B0 = reinterpret_cast<const F*>(smem + a.off_b[0]);
  const F* D0 = reinterpret_cast<const F*>(smem + a.off_d[0]);
  const F* B1 = reinterpret_cast<const F*>(smem + a.off_b[1]);
  const F* D1 = reinterpret_cast<const F*>(smem + a.off_d[1]);
  const F* B2 = reinterpret_cast<const F*>(smem + a.off_b[2]);
  const F* D2 = reinterpret_cast<const F*>(smem + a.off_d[2]);
  const NT* nodes = static_cast<const NT*>(a.nodes);
  const int m0 = a.m[0], m1 = a.m[1], m2 = TD == 3 ? a.m[2] : 1;
  const uint32_t mask = a.mask;

  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < a.padded;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cell = min(a.first_cell + c, a.last_cell);
    const uint32_t* row = a.dofmap + cell * K;
    F xh[GD], xl[GD];
    double x0[GD];
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
    // The cell's coordinates, lexicographic node order, into this thread's slots.
#pragma unroll 4
    for (int l = 0; l < K; ++l) {
      const uint32_t n = min(__ldg(row + perm[l]), a.last_node);
#pragma unroll
      for (int g = 0; g < GD; ++g) {
        const NT v = __ldg(nodes + (int64_t)n * GD + g);
        F y;
        if constexpr (SPLIT) y = d2f_rn(v - x0[g]);
        else y = v;
        xs[(l * GD + g) * T] = y;
      }
    }
    F sign = F(1);
    if ((mask & kOutNormals) && a.flags != nullptr && a.last_flag >= 0) {
      const uint32_t f = __ldg(a.flags + min(a.first_cell + c, a.last_flag));
      sign = (f & 1u) ? F(-1) : F(1);
    }
    const int64_t o = a.out_first_cell + c;
    const int64_t tile_idx = o >> a.tile_shift;
    const int lane = (int)(o & ((1 << a.tile_shift) - 1));

    if constexpr (TD == 3) {
      for (int c2 = 0; c2 < m2; ++c2) {
        F U[GD][N][N], V[GD][N][N];
#pragma unroll
        for (int g = 0; g < GD; ++g)
#pragma unroll
          for (int jj = 0; jj < N; ++jj)
#pragma unroll
            for (int i = 0; i < N; ++i) U[g][jj][i] = V[g][jj][i] = F(0);
#pragma unroll
        for (int k = 0; k < N; ++k) {
          const F bk = B2[c2 * N + k], dk = D2[c2 * N + k];
#pragma unroll
          for (int jj = 0; jj < N; ++jj)
#pragma unroll
            for (int i = 0; i < N; ++i)
#pragma unroll
              for (int g = 0; g < GD; ++g) {
                const F xv = xs[((i + N * (jj + N * k)) * GD + g) * T];
                U[g][jj][i] = A::fma(xv, bk, U[g][jj][i]);
                V[g][jj][i] = A::fma(xv, dk, V[g][jj][i]);
              }
        }
        for (int b1 = 0; b1 < m1; ++b1) {
          F UU[GD][N], UD[GD][N], VU[GD][N];
#pragma unroll
          for (int g = 0; g < GD; ++g)
#pragma unroll
            for (int i = 0; i < N; ++i) UU[g][i] = UD[g][i] = VU[g][i] = F(0);
#pragma unroll
          for (int jj = 0; jj < N; ++jj) {
            const F bj = B1[b1 * N + jj], dj = D1[b1 * N + jj];
#pragma unroll
            for (int g = 0; g < GD; ++g)
#pragma unroll
              for (int i = 0; i < N; ++i) {
                UU[g][i] = A::fma(U[g][jj][i], bj, UU[g][i]);
                UD[g][i] = A::fma(U[g][jj][i], dj, UD[g][i]);
                VU[g][i] = A::fma(V[g][jj][i], bj, VU[g][i]);
              }
          }
          for (int a0 = 0; a0 < m0; ++a0) {
            F x[GD], j[LJ];
#pragma unroll
            for (int g = 0; g < GD; ++g) {
              F s = F(0), j0 = F(0), j1 = F(0), j2 = F(0);
#pragma unroll
              for (int i = 0; i < N; ++i) {
                const F bi = B0[a0 * N + i], di = D0[a0 * N + i];
                s = A::fma(UU[g][i], bi, s);
                j0 = A::fma(UU[g][i], di, j0);
                j1 = A::fma(UD[g][i], bi, j1);
                j2 = A::fma(VU[g][i], bi, j2);
              }
              x[g] = s;
              j[0 * GD + g] = j0;
              j[1 * GD + g] = j1;
              j[2 * GD + g] = j2;
            }
            sf_point<F, SPLIT, TD, GD>(a, a0 + m0 * (b1 + m1 * c2), tile_idx, lane, x, j, sign, xh, xl, row, K, c);
          }
        }
      }
    } else {
      for (int b1 = 0; b1 < m1; ++b1) {
        F U[GD][N], V[GD][N];
#pragma unroll
        for (int g = 0; g < GD; ++g)
#pragma unroll
          for (int i = 0; i < N; ++i) U[g][i] = V[g][i] = F(0);
#pragma unroll
        for (int jj = 0; jj < N; ++jj) {
          const F bj = B1[b1 * N + jj], dj = D1[b1 * N + jj];
#pragma unroll
          for (int i = 0; i < N; ++i)
#pragma unroll
            for (int g = 0; g < GD; ++g) {
              const F xv = xs[((i + N * jj) * GD + g) * T];
              U[g][i] = A::fma(xv, bj, U[g][i]);
              V[g][i] = A::fma(xv, dj, V[g][i]);
            }
        }
        for (int a0 = 0; a0 < m0; ++a0) {
          F x[GD], j[LJ];
#pragma unroll
          for (int g = 0; g < GD; ++g) {
            F s = F(0), j0 = F(0), j1 = F(0);
#pragma unroll
            for (int i = 0; i < N; ++i) {
              const F bi = B0[a0 * N + i], di = D0[a0 * N + i];
              s = A::fma(U[g][i], bi, s);
              j0 = A::fma(U[g][i], di, j0);
              j1 = A::fma(V[g][i], bi, j1);
            }
            x[g] = s;
            j[0 * GD + g] = j0;
            j[1 * GD + g] = j1;
          }
          sf_point<F, SPLIT, TD, GD>(a, a0 + m0 * b1, tile_idx, lane, x, j, sign, xh, xl, row, K, c);
        }
      }
    }
  }
}

}  // namespace tlg
