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
#include "eval_launch.cuh"

namespace tlg {

// One tensor block of a point set: point q = o + a s[0] + b s[1] + c s[2] for a < m[0], b < m[1],
// c < m[2]; per direction d the tables B_d [m_d][N] at off_b[d] and D_d at off_d[d] (bytes from the
// section's start). Prisms: direction 0 the (x, y) points with psi at off_b[0], d_x psi at
// off_d[0], d_y psi at off_d[1]; direction 2 the z points.
struct SfBlock {
  int o, m[3], s[3];
  uint32_t off_b[3], off_d[3];
  int pad[3];
};
static_assert(sizeof(SfBlock) == 64, "block headers are 64 bytes");

struct SfArgs {
  const void* nodes;
  const uint32_t* dofmap;
  const uint32_t* flags;
  const unsigned char* tab;  // staged: nblocks SfBlock headers, the blocks' tables, perm [K] u32,
                             // reference normals [Q][TD] (facet rules) at off_refn
  const double* dphi64;      // split: the f64 derivative table [Q][K][TD] (global) of the recompute
  void* out[6];              // points, jacobian, detj, pinv, normals, facet normals
  int* err;
  unsigned long long* recomputed;
  int64_t first_cell, padded, range_cells, out_first_cell, last_cell, last_flag;
  double origin[3];
  float cond_limit;
  uint32_t last_node, tab_bytes, off_perm, off_refn, mask;
  int nblocks;
  int prism;  // the table is a prism's
  int num_points;
  int tile_shift;  // log2 of the output tile
};

// Shared memory of the coordinate slots: K * GD values of F per thread.
inline size_t sumfact_slot_bytes(int k, int gd, size_t f_bytes) { return (size_t)k * gd * kEvalThreads * f_bytes; }

// One point's outputs from X (relative, before the origin) and J. FN: the facet normals are among
// them (a separate instantiation: their epilogue costs up to 60 registers).
template <typename F, bool SPLIT, int TD, int GD, bool FN>
__device__ __forceinline__ void sf_point(const SfArgs& a, int q, int64_t tile_idx, int lane, F* x, F* j, F sign,
                                         const F* xh, const F* xl, const uint32_t* row, int K, int64_t c,
                                         const F* refn) {
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
  if ((mask & kOutPinv) || SPLIT || FN) M::pinv(j, kk);
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
  if constexpr (FN && TD == GD) {
    if (mask & kOutFacetNormals) {
      F n[GD];
      M::facet_normal(kk, refn + q * TD, n);
      store_point(static_cast<F*>(a.out[5]), tile_idx, q, nq, GD, lane, a.tile_shift, n, GD);
    }
  }
  if constexpr (TD + 1 == GD) {
    if (mask & kOutNormals) {
      F n[GD];
      M::normal(j, sign, n);
      store_point(static_cast<F*>(a.out[4]), tile_idx, q, nq, GD, lane, a.tile_shift, n, GD);
    }
  }
}

// F: arithmetic and output type; SPLIT: f64 nodes shifted by node 0 and rounded to F = float.
template <typename F, bool SPLIT, int TD, int GD, int N, bool FN>
__global__ void __launch_bounds__(kEvalThreads) sumfact_kernel(const __grid_constant__ SfArgs a) {
  using NT = typename std::conditional<SPLIT, double, F>::type;  // node type
  using A = Ar<F>;
  constexpr int K = TD == 3 ? N * N * N : N * N;
  constexpr int LJ = TD * GD;
  constexpr int T = kEvalThreads;
  __shared__ uint64_t bar;
  extern __shared__ __align__(16) unsigned char smem[];
  if (!stage_table(a.tab, smem, a.tab_bytes, &bar, a.err)) return;
  F* xs = reinterpret_cast<F*>(smem + (a.tab_bytes + 15) / 16 * 16) + threadIdx.x;
  const uint32_t* perm = reinterpret_cast<const uint32_t*>(smem + a.off_perm);
  const SfBlock* blocks = reinterpret_cast<const SfBlock*>(smem);
  const F* refn = reinterpret_cast<const F*>(smem + a.off_refn);
  const NT* nodes = static_cast<const NT*>(a.nodes);
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

    for (int bk = 0; bk < a.nblocks; ++bk) {
      const SfBlock& h = blocks[bk];
      const F* B0 = reinterpret_cast<const F*>(smem + h.off_b[0]);
      const F* D0 = reinterpret_cast<const F*>(smem + h.off_d[0]);
      const F* B1 = reinterpret_cast<const F*>(smem + h.off_b[1]);
      const F* D1 = reinterpret_cast<const F*>(smem + h.off_d[1]);
      const F* B2 = reinterpret_cast<const F*>(smem + h.off_b[2]);
      const F* D2 = reinterpret_cast<const F*>(smem + h.off_d[2]);
      const int m0 = h.m[0], m1 = h.m[1], m2 = TD == 3 ? h.m[2] : 1;
      const int s0 = h.s[0], s1 = h.s[1], s2 = h.s[2], qo = h.o;
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
              sf_point<F, SPLIT, TD, GD, FN>(a, qo + a0 * s0 + b1 * s1 + c2 * s2, tile_idx, lane, x, j, sign, xh, xl, row, K,
                                         c, refn);
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
            sf_point<F, SPLIT, TD, GD, FN>(a, qo + a0 * s0 + b1 * s1, tile_idx, lane, x, j, sign, xh, xl, row, K, c, refn);
          }
        }
      }
    }  // blocks
  }
}

// Prisms (the reference's prism blocks, tetraloma-geometry/src/sumfact/prism.rs:23-136). The
// prism's Lagrange basis is the product of the triangle's (NT = N (N + 1) / 2 nodes) and the
// interval's (N nodes), and a tensor rule is a triangle rule times points in z. Per triangle point
// i the cell's coordinates are contracted with the triangle basis and its two derivatives,
//   BV_g[c] = sum_t x_{(c, t), g} psi_t(i),  BX_g[c] = ... d_x psi_t(i),  BY_g[c] = ... d_y psi_t(i),
// then per z point j with the interval basis:
//   X_g = sum_c BV_g[c] l_c(z_j), J(g, 0) = sum_c BX_g[c] l_c(z_j), J(g, 1) = sum_c BY_g[c] l_c(z_j),
//   J(g, 2) = sum_c BV_g[c] l_c'(z_j):
// 3 NT N per triangle point and 4 N per point and coordinate instead of 4 NT N per point. Per
// block: psi [m_t][NT] at off_b[0], d_x psi at off_d[0], d_y psi at off_d[1], l [m_z][N] at
// off_b[2], l' at off_d[2]; perm maps the index c NT + t to the Lagrange node; point
// q = o + i s[0] + j s[2].
template <typename F, bool SPLIT, int N, bool FN>
__global__ void __launch_bounds__(kEvalThreads) sumfact_prism_kernel(const __grid_constant__ SfArgs a) {
  using NT_ = typename std::conditional<SPLIT, double, F>::type;  // node type
  using A = Ar<F>;
  constexpr int TD = 3, GD = 3, NT = N * (N + 1) / 2, K = NT * N, LJ = TD * GD;
  constexpr int T = kEvalThreads;
  __shared__ uint64_t bar;
  extern __shared__ __align__(16) unsigned char smem[];
  if (!stage_table(a.tab, smem, a.tab_bytes, &bar, a.err)) return;
  F* xs = reinterpret_cast<F*>(smem + (a.tab_bytes + 15) / 16 * 16) + threadIdx.x;
  const uint32_t* perm = reinterpret_cast<const uint32_t*>(smem + a.off_perm);
  const SfBlock* blocks = reinterpret_cast<const SfBlock*>(smem);
  const F* refn = reinterpret_cast<const F*>(smem + a.off_refn);
  const NT_* nodes = static_cast<const NT_*>(a.nodes);

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
#pragma unroll 4
    for (int l = 0; l < K; ++l) {
      const uint32_t n = min(__ldg(row + perm[l]), a.last_node);
#pragma unroll
      for (int g = 0; g < GD; ++g) {
        const NT_ v = __ldg(nodes + (int64_t)n * GD + g);
        F y;
        if constexpr (SPLIT) y = d2f_rn(v - x0[g]);
        else y = v;
        xs[(l * GD + g) * T] = y;
      }
    }
    const int64_t o = a.out_first_cell + c;
    const int64_t tile_idx = o >> a.tile_shift;
    const int lane = (int)(o & ((1 << a.tile_shift) - 1));

    for (int bk = 0; bk < a.nblocks; ++bk) {
      const SfBlock& h = blocks[bk];
      const F* PV = reinterpret_cast<const F*>(smem + h.off_b[0]);
      const F* PX = reinterpret_cast<const F*>(smem + h.off_d[0]);
      const F* PY = reinterpret_cast<const F*>(smem + h.off_d[1]);
      const F* LV = reinterpret_cast<const F*>(smem + h.off_b[2]);
      const F* LD = reinterpret_cast<const F*>(smem + h.off_d[2]);
      const int mt = h.m[0], mz = h.m[2], st = h.s[0], sz = h.s[2], qo = h.o;
      for (int i = 0; i < mt; ++i) {
        F bv[GD][N], bx[GD][N], by[GD][N];
#pragma unroll
        for (int g = 0; g < GD; ++g)
#pragma unroll
          for (int cc = 0; cc < N; ++cc) bv[g][cc] = bx[g][cc] = by[g][cc] = F(0);
        // (f64 P3: a rolled loop, the unrolled one spills.)
#pragma unroll(sizeof(F) == 8 && N >= 4 ? 1 : NT)
        for (int t = 0; t < NT; ++t) {
          const F w = PV[i * NT + t], wx = PX[i * NT + t], wy = PY[i * NT + t];
#pragma unroll
          for (int cc = 0; cc < N; ++cc)
#pragma unroll
            for (int g = 0; g < GD; ++g) {
              const F xv = xs[((cc * NT + t) * GD + g) * T];
              bv[g][cc] = A::fma(xv, w, bv[g][cc]);
              bx[g][cc] = A::fma(xv, wx, bx[g][cc]);
              by[g][cc] = A::fma(xv, wy, by[g][cc]);
            }
        }
        for (int jz = 0; jz < mz; ++jz) {
          F x[GD], j[LJ];
#pragma unroll
          for (int g = 0; g < GD; ++g) {
            F s0 = F(0), j0 = F(0), j1 = F(0), j2 = F(0);
#pragma unroll
            for (int cc = 0; cc < N; ++cc) {
              const F l = LV[jz * N + cc], ld = LD[jz * N + cc];
              s0 = A::fma(bv[g][cc], l, s0);
              j0 = A::fma(bx[g][cc], l, j0);
              j1 = A::fma(by[g][cc], l, j1);
              j2 = A::fma(bv[g][cc], ld, j2);
            }
            x[g] = s0;
            j[0 * GD + g] = j0;
            j[1 * GD + g] = j1;
            j[2 * GD + g] = j2;
          }
          sf_point<F, SPLIT, TD, GD, FN>(a, qo + i * st + jz * sz, tile_idx, lane, x, j, F(1), xh, xl, row, K, c, refn);
        }
      }
    }  // blocks
  }
}


// Dispatch of the forward sum-factorised kernels (instantiated in sumfact.cu without, and in
// sumfact_fn.cu with, facet normals).
template <typename F, bool SPLIT, bool FN>
cudaError_t launch_sf(int td, int gd, int n, const SfArgs& a, size_t smem, cudaStream_t s, bool* found) {
  *found = true;
  if (a.prism) {
    if (n == 2) return launch_persistent(sumfact_prism_kernel<F, SPLIT, 2, FN>, a, a.padded, smem, s);
    if (n == 3) return launch_persistent(sumfact_prism_kernel<F, SPLIT, 3, FN>, a, a.padded, smem, s);
    if (n == 4) return launch_persistent(sumfact_prism_kernel<F, SPLIT, 4, FN>, a, a.padded, smem, s);
    *found = false;
    return cudaSuccess;
  }
#define TLG_SF(TD, GD, NN) \
  if (td == TD && gd == GD && n == NN) \
    return launch_persistent(sumfact_kernel<F, SPLIT, TD, GD, NN, FN>, a, a.padded, smem, s);
  TLG_SF(3, 3, 2)
  TLG_SF(3, 3, 3)
  TLG_SF(3, 3, 4)
  TLG_SF(2, 2, 2)
  TLG_SF(2, 2, 3)
  TLG_SF(2, 2, 4)
  TLG_SF(2, 2, 5)
  TLG_SF(2, 2, 6)
  if constexpr (!FN) {  // facet normals need codimension 0
    TLG_SF(2, 3, 2)
    TLG_SF(2, 3, 3)
    TLG_SF(2, 3, 4)
    TLG_SF(2, 3, 5)
    TLG_SF(2, 3, 6)
  }
#undef TLG_SF
  *found = false;
  return cudaSuccess;
}

}  // namespace tlg


namespace tlg {

// ----------------------------------------------------------------------------------------
// The sum-factorised adjoint of hexahedra (TD = GD = 3) at tensor-product rules.
//
// Per cell (one thread): the forward contraction as sumfact_kernel, plane by plane and row by
// row; at every point K, det J, the fused forward outputs when asked, and from the cotangents
// xbar, Jbar = dbar det J K^T - K^T Kbar K^T. The node contributions
//   L_g(i, j, k) = sum_{a,b,c} [B0 B1 B2 xbar_g + D0 B1 B2 Jbar(g, 0) + B0 D1 B2 Jbar(g, 1)
//                               + B0 B1 D2 Jbar(g, 2)]
// are the transposed contraction, accumulated in the reverse order: over a row's points into
// RU = sum_a (B0 xbar + D0 Jbar0), RD1 = sum_a B0 Jbar1, RD2 = sum_a B0 Jbar2 (registers), over a
// plane's rows into PU += B1 RU + D1 RD1, PV += B1 RD2 (shared-memory slots), over the planes
// into L += B2 PU + D2 PV (shared-memory slots). The 32 cells of a warp then write their rows
// (Lagrange node order, R = 4 values, the fourth zero) as one contiguous run.

struct VjpSfArgs {
  const void* nodes;
  const uint32_t* dofmap;
  const unsigned char* tab;  // the sum-factorisation section: B_d, D_d, perm
  const void* ct[3];         // cotangents: points, detj, pinv (tile 16 chunks) or null
  void* out[4];              // fused forward fields: points, jacobian, detj, pinv, or null
  void* local;               // contributions [cell][K][4]
  int* err;
  int64_t first_cell, padded, out_first_cell, last_cell, range_end;
  double origin[3];
  uint32_t last_node, tab_bytes, off_b[3], off_d[3], off_perm;
  int m[3];
  int num_points;
};

// Shared memory past the tables: the inverse permutation (K u32, rounded to 16 bytes), then per
// thread the coordinate slots (K * 3, stride `threads`), the plane accumulators (2 * 3 * N^2,
// stride `threads`) and the contribution slots (K * 3, stride threads + 1, so that the final
// write-out, whose lanes read one cell's slots, spreads over the banks), of F.
inline size_t vjp_sumfact_extra_bytes(int n, int threads, size_t f_bytes) {
  const size_t k = (size_t)n * n * n;
  return (k * 4 + 15) / 16 * 16 +
         f_bytes * ((size_t)threads * (k * 3 + 2 * 3 * (size_t)n * n) + (size_t)(threads + 1) * k * 3);
}

// M0 > 0: the rule has M0 points in direction 0 (the point loop of a row unrolled, so that the
// rows' points overlap); 0: at run time.
#ifndef TLG_VJP_PF
#define TLG_VJP_PF 2
#endif

template <typename F, bool SPLIT, int N, int M0>
__global__ void __launch_bounds__(kEvalThreads) vjp_sumfact_kernel(const __grid_constant__ VjpSfArgs a) {
  using NT = typename std::conditional<SPLIT, double, F>::type;
  using A = Ar<F>;
  using M = Factors<F, 3, 3>;
  constexpr int D = 3, K = N * N * N, LJ = 9, R = 4, TILE = 16;
  constexpr int T = kEvalThreads;  // compile-time slot strides: shared-memory offsets are immediates
  __shared__ uint64_t bar;
  extern __shared__ __align__(16) unsigned char smem[];
  if (!stage_table(a.tab, smem, a.tab_bytes, &bar, a.err)) return;
  const uint32_t* perm = reinterpret_cast<const uint32_t*>(smem + a.off_perm);
  uint32_t* invperm = reinterpret_cast<uint32_t*>(smem + (a.tab_bytes + 15) / 16 * 16);
  for (int i = threadIdx.x; i < K; i += T) invperm[perm[i]] = i;
  __syncthreads();
  F* slots = reinterpret_cast<F*>(reinterpret_cast<unsigned char*>(invperm) + (K * 4 + 15) / 16 * 16);
  constexpr int S = T + 1;                                        // stride of the contribution slots
  F* xs = slots + threadIdx.x;                                    // [K][3] coordinates
  F* Ps = slots + (size_t)K * D * T + threadIdx.x;                // [2][3][N][N] plane accumulators
  F* Lw = slots + (size_t)K * D * T + (size_t)2 * D * N * N * T;  // [K][3] contributions
  F* Ls = Lw + threadIdx.x;
  const F* B0 = reinterpret_cast<const F*>(smem + a.off_b[0]);
  const F* D0 = reinterpret_cast<const F*>(smem + a.off_d[0]);
  const F* B1 = reinterpret_cast<const F*>(smem + a.off_b[1]);
  const F* D1 = reinterpret_cast<const F*>(smem + a.off_d[1]);
  const F* B2 = reinterpret_cast<const F*>(smem + a.off_b[2]);
  const F* D2 = reinterpret_cast<const F*>(smem + a.off_d[2]);
  const NT* nodes = static_cast<const NT*>(a.nodes);
  const F* ctx = static_cast<const F*>(a.ct[0]);
  const F* ctd = static_cast<const F*>(a.ct[1]);
  const F* ctk = static_cast<const F*>(a.ct[2]);
  const int m0 = a.m[0], m1 = a.m[1], m2 = a.m[2];
  const int nq = a.num_points;
  const int lane = threadIdx.x % 32;
  const int64_t step = (int64_t)gridDim.x * T;

  // A warp walks 32 consecutive cells; lanes past the padded range repeat the last cell and
  // store nothing.
  for (int64_t cw = (int64_t)blockIdx.x * T + (threadIdx.x & ~31); cw < a.padded; cw += step) {
    const int64_t c = cw + lane;
    const bool live = c < a.padded;
    const int64_t cell = min(a.first_cell + c, a.last_cell);
    const uint32_t* row = a.dofmap + cell * K;
    F xh[D], xl[D];
    double x0[D];
    if constexpr (SPLIT) {
      const uint32_t n0 = min(__ldg(row), a.last_node);
#pragma unroll
      for (int g = 0; g < D; ++g) {
        x0[g] = __ldg(nodes + (int64_t)n0 * D + g);
        const double v = x0[g] + a.origin[g];
        xh[g] = d2f_rn(v);
        xl[g] = d2f_rn(v - f2d_exact(xh[g]));
      }
    } else {
#pragma unroll
      for (int g = 0; g < D; ++g) {
        x0[g] = 0.0;
        xh[g] = (F)a.origin[g];
        xl[g] = F(0);
      }
    }
#pragma unroll 4
    for (int l = 0; l < K; ++l) {
      const uint32_t n = min(__ldg(row + perm[l]), a.last_node);
#pragma unroll
      for (int g = 0; g < D; ++g) {
        const NT v = __ldg(nodes + (int64_t)n * D + g);
        F y;
        if constexpr (SPLIT) y = d2f_rn(v - x0[g]);
        else y = v;
        xs[(l * D + g) * T] = y;
        Ls[(l * D + g) * S] = F(0);
      }
    }
    // Lanes past the padded range read the cotangents of the last padded cell.
    const int64_t o = a.out_first_cell + (live ? c : a.padded - 1);
    const int64_t tq = (o / TILE) * nq;
    const int l16 = (int)(o % TILE);
#define TLG_AT(q, len, comp) (((tq + (q)) * (len) + (comp)) * TILE + l16)
    // The cotangents of a point (xbar, dbar, Kbar; zero where absent), loaded PF points ahead
    // (points run in rule order) so that their latency overlaps the work of the points between:
    // two in f32 (registers to spare under the two CTAs per SM the slots allow), one in f64.
    auto load_ct = [&](int q, F* v) {
#pragma unroll
      for (int g = 0; g < D; ++g) v[g] = ctx ? __ldg(ctx + TLG_AT(q, D, g)) : F(0);
      v[D] = ctd ? __ldg(ctd + TLG_AT(q, 1, 0)) : F(0);
#pragma unroll
      for (int i = 0; i < LJ; ++i) v[D + 1 + i] = ctk ? __ldg(ctk + TLG_AT(q, LJ, i)) : F(0);
    };
    constexpr int PF = sizeof(F) == 4 ? TLG_VJP_PF : 1;
    F buf[PF][D + 1 + LJ];  // buf[p]: the cotangents of point q + p
#pragma unroll
    for (int p = 0; p < PF; ++p) load_ct(min(p, nq - 1), buf[p]);
    const F* cur = buf[0];

    for (int c2 = 0; c2 < m2; ++c2) {
      F U[D][N][N], V[D][N][N];
#pragma unroll
      for (int g = 0; g < D; ++g)
#pragma unroll
        for (int jj = 0; jj < N; ++jj)
#pragma unroll
          for (int i = 0; i < N; ++i) {
            U[g][jj][i] = V[g][jj][i] = F(0);
            Ps[((0 * D + g) * N * N + jj * N + i) * T] = F(0);
            Ps[((1 * D + g) * N * N + jj * N + i) * T] = F(0);
          }
#pragma unroll
      for (int k = 0; k < N; ++k) {
        const F bk = B2[c2 * N + k], dk = D2[c2 * N + k];
#pragma unroll
        for (int jj = 0; jj < N; ++jj)
#pragma unroll
          for (int i = 0; i < N; ++i)
#pragma unroll
            for (int g = 0; g < D; ++g) {
              const F xv = xs[((i + N * (jj + N * k)) * D + g) * T];
              U[g][jj][i] = A::fma(xv, bk, U[g][jj][i]);
              V[g][jj][i] = A::fma(xv, dk, V[g][jj][i]);
            }
      }
      for (int b1 = 0; b1 < m1; ++b1) {
        F UU[D][N], UD[D][N], VU[D][N], RU[D][N], RD1[D][N], RD2[D][N];
#pragma unroll
        for (int g = 0; g < D; ++g)
#pragma unroll
          for (int i = 0; i < N; ++i) UU[g][i] = UD[g][i] = VU[g][i] = RU[g][i] = RD1[g][i] = RD2[g][i] = F(0);
#pragma unroll
        for (int jj = 0; jj < N; ++jj) {
          const F bj = B1[b1 * N + jj], dj = D1[b1 * N + jj];
#pragma unroll
          for (int g = 0; g < D; ++g)
#pragma unroll
            for (int i = 0; i < N; ++i) {
              UU[g][i] = A::fma(U[g][jj][i], bj, UU[g][i]);
              UD[g][i] = A::fma(U[g][jj][i], dj, UD[g][i]);
              VU[g][i] = A::fma(V[g][jj][i], bj, VU[g][i]);
            }
        }
        #pragma unroll
        for (int a0 = 0; a0 < (M0 > 0 ? M0 : m0); ++a0) {
          const int q = a0 + m0 * (b1 + m1 * c2);
          F nxt[D + 1 + LJ];
          load_ct(min(q + PF, nq - 1), nxt);
          F x[D], j[LJ];
#pragma unroll
          for (int g = 0; g < D; ++g) {
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
            j[0 * D + g] = j0;
            j[1 * D + g] = j1;
            j[2 * D + g] = j2;
          }
          F kinv[LJ];
          M::pinv(j, kinv);
          const F det = M::detj(j);
          if (live) {
            if (a.out[0]) {
#pragma unroll
              for (int g = 0; g < D; ++g) {
                const F v = SPLIT ? A::add(xh[g], A::add(xl[g], x[g])) : A::add(x[g], xh[g]);
                static_cast<F*>(a.out[0])[TLG_AT(q, D, g)] = v;
              }
            }
            if (a.out[1])
#pragma unroll
              for (int i = 0; i < LJ; ++i) static_cast<F*>(a.out[1])[TLG_AT(q, LJ, i)] = j[i];
            if (a.out[2]) static_cast<F*>(a.out[2])[TLG_AT(q, 1, 0)] = det;
            if (a.out[3])
#pragma unroll
              for (int i = 0; i < LJ; ++i) static_cast<F*>(a.out[3])[TLG_AT(q, LJ, i)] = kinv[i];
          }
          // Jbar(g, d) at g * D + d; K(t, h) and Kbar(t, h) at h * D + t.
          F jb[LJ];
          const F s = A::mul(cur[D], det);
#pragma unroll
          for (int g = 0; g < D; ++g)
#pragma unroll
            for (int d = 0; d < D; ++d) jb[g * D + d] = A::mul(s, kinv[g * D + d]);
          if (ctk) {
            const F* kb = cur + D + 1;
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
          const F* xb = cur;
#pragma unroll
          for (int i = 0; i < N; ++i) {
            const F bi = B0[a0 * N + i], di = D0[a0 * N + i];
#pragma unroll
            for (int g = 0; g < D; ++g) {
              RU[g][i] = A::fma(bi, xb[g], A::fma(di, jb[g * D + 0], RU[g][i]));
              RD1[g][i] = A::fma(bi, jb[g * D + 1], RD1[g][i]);
              RD2[g][i] = A::fma(bi, jb[g * D + 2], RD2[g][i]);
            }
          }
#pragma unroll
          for (int i = 0; i < D + 1 + LJ; ++i) {
#pragma unroll
            for (int p = 0; p + 1 < PF; ++p) buf[p][i] = buf[p + 1][i];
            buf[PF - 1][i] = nxt[i];
          }
        }
        // The row into the plane accumulators.
#pragma unroll
        for (int jj = 0; jj < N; ++jj) {
          const F bj = B1[b1 * N + jj], dj = D1[b1 * N + jj];
#pragma unroll
          for (int g = 0; g < D; ++g)
#pragma unroll
            for (int i = 0; i < N; ++i) {
              F* pu = Ps + ((0 * D + g) * N * N + jj * N + i) * T;
              F* pv = Ps + ((1 * D + g) * N * N + jj * N + i) * T;
              *pu = A::fma(bj, RU[g][i], A::fma(dj, RD1[g][i], *pu));
              *pv = A::fma(bj, RD2[g][i], *pv);
            }
        }
      }
      // The plane into the contributions.
#pragma unroll
      for (int k = 0; k < N; ++k) {
        const F bk = B2[c2 * N + k], dk = D2[c2 * N + k];
#pragma unroll
        for (int jj = 0; jj < N; ++jj)
#pragma unroll
          for (int i = 0; i < N; ++i)
#pragma unroll
            for (int g = 0; g < D; ++g) {
              F* lp = Ls + ((i + N * (jj + N * k)) * D + g) * S;
              const F pu = Ps[((0 * D + g) * N * N + jj * N + i) * T];
              const F pv = Ps[((1 * D + g) * N * N + jj * N + i) * T];
              *lp = A::fma(bk, pu, A::fma(dk, pv, *lp));
            }
      }
    }
#undef TLG_AT
    // The warp's cells' rows, Lagrange node order, as one run.
    __syncwarp();
    const int64_t cell0 = a.first_cell + cw;
    const int64_t nreal = min((int64_t)32, a.range_end - cell0);
    if (nreal > 0) {
      // One (cell, node) row of R = 4 values per lane and step: a 16-byte (f32) or two 16-byte
      // (f64) stores, consecutive lanes consecutive rows.
      F* dst = static_cast<F*>(a.local) + cell0 * (K * R);
      const F* lw = Lw + (threadIdx.x & ~31);  // the warp's contribution slots
      for (int t = lane; t < nreal * K; t += 32) {
        const int cl = t / K;
        const int kk = t - cl * K;
        const F* src = lw + (int)invperm[kk] * D * S + cl;
        F* row4 = dst + (int64_t)t * R;
        if constexpr (sizeof(F) == 4) {
          *reinterpret_cast<float4*>(row4) = make_float4(src[0], src[S], src[2 * S], 0.0f);
        } else {
          reinterpret_cast<double2*>(row4)[0] = make_double2(src[0], src[S]);
          reinterpret_cast<double2*>(row4)[1] = make_double2(src[2 * S], 0.0);
        }
      }
    }
    __syncwarp();
  }
}


// The adjoint of hexahedra at tensor-product rules from forward fields already written: det J and
// K read back per point (the pinv layout K(t, h) at h * D + t, as the fused kernel writes it)
// instead of recomputed, so no coordinates, no forward contraction and no coordinate slots; the
// transposed contraction, its accumulation order and the contribution rows exactly as
// vjp_sumfact_kernel's. `a.out[2]` (det J) and `a.out[3]` (K) are the inputs here.
template <typename F, int N, int M0>
__global__ void __launch_bounds__(kEvalThreads) vjp_sumfact_bwd_kernel(const __grid_constant__ VjpSfArgs a) {
  using A = Ar<F>;
  constexpr int D = 3, K = N * N * N, LJ = 9, R = 4, TILE = 16;
  constexpr int T = kEvalThreads;
  constexpr int NV = D + 1 + LJ + 1 + LJ;  // xbar, dbar, Kbar, det J, K of a point
  __shared__ uint64_t bar;
  extern __shared__ __align__(16) unsigned char smem[];
  if (!stage_table(a.tab, smem, a.tab_bytes, &bar, a.err)) return;
  const uint32_t* perm = reinterpret_cast<const uint32_t*>(smem + a.off_perm);
  uint32_t* invperm = reinterpret_cast<uint32_t*>(smem + (a.tab_bytes + 15) / 16 * 16);
  for (int i = threadIdx.x; i < K; i += T) invperm[perm[i]] = i;
  __syncthreads();
  F* slots = reinterpret_cast<F*>(reinterpret_cast<unsigned char*>(invperm) + (K * 4 + 15) / 16 * 16);
  constexpr int S = T + 1;                              // stride of the contribution slots
  F* Ps = slots + threadIdx.x;                          // [2][3][N][N] plane accumulators
  F* Lw = slots + (size_t)2 * D * N * N * T;            // [K][3] contributions
  F* Ls = Lw + threadIdx.x;
  const F* B0 = reinterpret_cast<const F*>(smem + a.off_b[0]);
  const F* D0 = reinterpret_cast<const F*>(smem + a.off_d[0]);
  const F* B1 = reinterpret_cast<const F*>(smem + a.off_b[1]);
  const F* D1 = reinterpret_cast<const F*>(smem + a.off_d[1]);
  const F* B2 = reinterpret_cast<const F*>(smem + a.off_b[2]);
  const F* D2 = reinterpret_cast<const F*>(smem + a.off_d[2]);
  const F* ctx = static_cast<const F*>(a.ct[0]);
  const F* ctd = static_cast<const F*>(a.ct[1]);
  const F* ctk = static_cast<const F*>(a.ct[2]);
  const F* fdet = static_cast<const F*>(a.out[2]);
  const F* fk = static_cast<const F*>(a.out[3]);
  const int m0 = a.m[0], m1 = a.m[1], m2 = a.m[2];
  const int nq = a.num_points;
  const int lane = threadIdx.x % 32;
  const int64_t step = (int64_t)gridDim.x * T;

  for (int64_t cw = (int64_t)blockIdx.x * T + (threadIdx.x & ~31); cw < a.padded; cw += step) {
    const int64_t c = cw + lane;
    const bool live = c < a.padded;
#pragma unroll 4
    for (int l = 0; l < K; ++l)
#pragma unroll
      for (int g = 0; g < D; ++g) Ls[(l * D + g) * S] = F(0);
    // Lanes past the padded range read the values of the last padded cell.
    const int64_t o = a.out_first_cell + (live ? c : a.padded - 1);
    const int64_t tq = (o / TILE) * nq;
    const int l16 = (int)(o % TILE);
#define TLG_AT(q, len, comp) (((tq + (q)) * (len) + (comp)) * TILE + l16)
    // A point's values, loaded PF points ahead (points run in rule order).
    auto load_pt = [&](int q, F* v) {
#pragma unroll
      for (int g = 0; g < D; ++g) v[g] = ctx ? __ldg(ctx + TLG_AT(q, D, g)) : F(0);
      v[D] = ctd ? __ldg(ctd + TLG_AT(q, 1, 0)) : F(0);
#pragma unroll
      for (int i = 0; i < LJ; ++i) v[D + 1 + i] = ctk ? __ldg(ctk + TLG_AT(q, LJ, i)) : F(0);
      v[D + 1 + LJ] = __ldg(fdet + TLG_AT(q, 1, 0));
#pragma unroll
      for (int i = 0; i < LJ; ++i) v[D + 2 + LJ + i] = __ldg(fk + TLG_AT(q, LJ, i));
    };
    constexpr int PF = sizeof(F) == 4 ? 2 : 1;
    F buf[PF][NV];
#pragma unroll
    for (int p = 0; p < PF; ++p) load_pt(min(p, nq - 1), buf[p]);

    for (int c2 = 0; c2 < m2; ++c2) {
#pragma unroll
      for (int g = 0; g < D; ++g)
#pragma unroll
        for (int jj = 0; jj < N; ++jj)
#pragma unroll
          for (int i = 0; i < N; ++i) {
            Ps[((0 * D + g) * N * N + jj * N + i) * T] = F(0);
            Ps[((1 * D + g) * N * N + jj * N + i) * T] = F(0);
          }
      for (int b1 = 0; b1 < m1; ++b1) {
        F RU[D][N], RD1[D][N], RD2[D][N];
#pragma unroll
        for (int g = 0; g < D; ++g)
#pragma unroll
          for (int i = 0; i < N; ++i) RU[g][i] = RD1[g][i] = RD2[g][i] = F(0);
#pragma unroll
        for (int a0 = 0; a0 < (M0 > 0 ? M0 : m0); ++a0) {
          const int q = a0 + m0 * (b1 + m1 * c2);
          F nxt[NV];
          load_pt(min(q + PF, nq - 1), nxt);
          const F* cur = buf[0];
          const F det = cur[D + 1 + LJ];
          const F* kinv = cur + D + 2 + LJ;
          // Jbar(g, d) at g * D + d; K(t, h) and Kbar(t, h) at h * D + t.
          F jb[LJ];
          const F s = A::mul(cur[D], det);
#pragma unroll
          for (int g = 0; g < D; ++g)
#pragma unroll
            for (int d = 0; d < D; ++d) jb[g * D + d] = A::mul(s, kinv[g * D + d]);
          if (ctk) {
            const F* kb = cur + D + 1;
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
          const F* xb = cur;
#pragma unroll
          for (int i = 0; i < N; ++i) {
            const F bi = B0[a0 * N + i], di = D0[a0 * N + i];
#pragma unroll
            for (int g = 0; g < D; ++g) {
              RU[g][i] = A::fma(bi, xb[g], A::fma(di, jb[g * D + 0], RU[g][i]));
              RD1[g][i] = A::fma(bi, jb[g * D + 1], RD1[g][i]);
              RD2[g][i] = A::fma(bi, jb[g * D + 2], RD2[g][i]);
            }
          }
#pragma unroll
          for (int i = 0; i < NV; ++i) {
#pragma unroll
            for (int p = 0; p + 1 < PF; ++p) buf[p][i] = buf[p + 1][i];
            buf[PF - 1][i] = nxt[i];
          }
        }
        // The row into the plane accumulators.
#pragma unroll
        for (int jj = 0; jj < N; ++jj) {
          const F bj = B1[b1 * N + jj], dj = D1[b1 * N + jj];
#pragma unroll
          for (int g = 0; g < D; ++g)
#pragma unroll
            for (int i = 0; i < N; ++i) {
              F* pu = Ps + ((0 * D + g) * N * N + jj * N + i) * T;
              F* pv = Ps + ((1 * D + g) * N * N + jj * N + i) * T;
              *pu = A::fma(bj, RU[g][i], A::fma(dj, RD1[g][i], *pu));
              *pv = A::fma(bj, RD2[g][i], *pv);
            }
        }
      }
      // The plane into the contributions.
#pragma unroll
      for (int k = 0; k < N; ++k) {
        const F bk = B2[c2 * N + k], dk = D2[c2 * N + k];
#pragma unroll
        for (int jj = 0; jj < N; ++jj)
#pragma unroll
          for (int i = 0; i < N; ++i)
#pragma unroll
            for (int g = 0; g < D; ++g) {
              F* lp = Ls + ((i + N * (jj + N * k)) * D + g) * S;
              const F pu = Ps[((0 * D + g) * N * N + jj * N + i) * T];
              const F pv = Ps[((1 * D + g) * N * N + jj * N + i) * T];
              *lp = A::fma(bk, pu, A::fma(dk, pv, *lp));
            }
      }
    }
#undef TLG_AT
    // The warp's cells' rows, Lagrange node order, as one run.
    __syncwarp();
    const int64_t cell0 = a.first_cell + cw;
    const int64_t nreal = min((int64_t)32, a.range_end - cell0);
    if (nreal > 0) {
      F* dst = static_cast<F*>(a.local) + cell0 * (K * R);
      const F* lw = Lw + (threadIdx.x & ~31);
      for (int t = lane; t < nreal * K; t += 32) {
        const int cl = t / K;
        const int kk = t - cl * K;
        const F* src = lw + (int)invperm[kk] * D * S + cl;
        F* row4 = dst + (int64_t)t * R;
        if constexpr (sizeof(F) == 4) {
          *reinterpret_cast<float4*>(row4) = make_float4(src[0], src[S], src[2 * S], 0.0f);
        } else {
          reinterpret_cast<double2*>(row4)[0] = make_double2(src[0], src[S]);
          reinterpret_cast<double2*>(row4)[1] = make_double2(src[2 * S], 0.0);
        }
      }
    }
    __syncwarp();
  }
}

// Shared memory past the tables of the kernel above: the inverse permutation, the plane
// accumulators (2 * 3 * N^2, stride `threads`) and the contribution slots (K * 3, stride
// threads + 1), of F.
inline size_t vjp_sumfact_bwd_extra_bytes(int n, int threads, size_t f_bytes) {
  const size_t k = (size_t)n * n * n;
  return (k * 4 + 15) / 16 * 16 + f_bytes * ((size_t)threads * 2 * 3 * n * n + (size_t)(threads + 1) * k * 3);
}

// ----------------------------------------------------------------------------------------
// Tile kernels: the work of a 16-cell tile of the fields spread over the CTA, one phase after
// another with a barrier between, each phase's work items (point and cell, cell and node, ...)
// over the threads with the cell index fastest, so that the loads and stores of the fields are
// coalesced. A point's x̄ and J̄ of one cell are a record of three 4-vectors (x̄_g, J̄(g, 0),
// J̄(g, 1), J̄(g, 2)), [point][cell][12], each moved by one 16-byte access (f32); the plane sums
// of a cell sit at an odd stride. Every sum runs in vjp_sumfact_kernel's order, so the
// contribution rows are that kernel's bit for bit.

constexpr int kTileCells = 16;
constexpr int kTileRec = 12;                       // x̄ and J̄ of a point and cell
constexpr int kTileQS = kTileRec * kTileCells;     // per point: the tile's records

template <typename F>
__device__ __forceinline__ void tile_put_record(F* rec, const F* xb, const F* jb) {
#pragma unroll
  for (int g = 0; g < 3; ++g) Vec4<F>::put(rec + 4 * g, xb[g], jb[g * 3], jb[g * 3 + 1], jb[g * 3 + 2]);
}

// J̄(g, d) at g * 3 + d of a point from its cotangents (d̄ = db, K̄ = kb or null for zero) and its
// det J and K (K(t, h) at h * 3 + t).
template <typename F>
__device__ __forceinline__ void tile_jbar(F db, const F* kb, F det, const F* kinv, F* jb) {
  using A = Ar<F>;
  constexpr int D = 3;
  const F s = A::mul(db, det);
#pragma unroll
  for (int g = 0; g < D; ++g)
#pragma unroll
    for (int d = 0; d < D; ++d) jb[g * D + d] = A::mul(s, kinv[g * D + d]);
  if (kb) {
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
}

// The transposed contraction of a tile along ξ0 (rows of m0 points) and ξ1 (planes of m1 rows):
// one item per (cell, plane c2, coordinate g), all node indices (j, i) of the plane at once, so that
// each point's x̄ and J̄ are read once; from V into the plane sums P ([cell * ps + ((c2 * 3 + g)
// * N + j) * N + i) * 2 + (u, v)]).
template <typename F, int N, int M, int T>
__device__ __forceinline__ void tile_planes(const F* V, F* P, int ps, const F* B0, const F* D0, const F* B1,
                                            const F* D1, int m0, int m1, int m2) {
  using A = Ar<F>;
  constexpr int D = 3, TILE = kTileCells, QS = kTileQS;
  for (int it = threadIdx.x; it < m2 * D * TILE; it += T) {
    const int l = it % TILE, r = it / TILE;
    const int g = r % D, c2 = r / D;
    F pu[N][N], pv[N][N];
#pragma unroll
    for (int j = 0; j < N; ++j)
#pragma unroll
      for (int i = 0; i < N; ++i) pu[j][i] = pv[j][i] = F(0);
    for (int b1 = 0; b1 < m1; ++b1) {
      F ru[N], rd1[N], rd2[N];
#pragma unroll
      for (int i = 0; i < N; ++i) ru[i] = rd1[i] = rd2[i] = F(0);
#pragma unroll
      for (int a0 = 0; a0 < (M > 0 ? M : m0); ++a0) {
        F v[4];
        Vec4<F>::get(V + (size_t)(a0 + m0 * (b1 + m1 * c2)) * QS + l * kTileRec + 4 * g, v);
        const F xb = v[0], j0 = v[1], j1 = v[2], j2 = v[3];
#pragma unroll
        for (int i = 0; i < N; ++i) {
          const F bi = B0[a0 * N + i], di = D0[a0 * N + i];
          ru[i] = A::fma(bi, xb, A::fma(di, j0, ru[i]));
          rd1[i] = A::fma(bi, j1, rd1[i]);
          rd2[i] = A::fma(bi, j2, rd2[i]);
        }
      }
#pragma unroll
      for (int j = 0; j < N; ++j) {
        const F bj = B1[b1 * N + j], dj = D1[b1 * N + j];
#pragma unroll
        for (int i = 0; i < N; ++i) {
          pu[j][i] = A::fma(bj, ru[i], A::fma(dj, rd1[i], pu[j][i]));
          pv[j][i] = A::fma(bj, rd2[i], pv[j][i]);
        }
      }
    }
    F* pl = P + l * ps + (c2 * D + g) * N * N * 2;
#pragma unroll
    for (int j = 0; j < N; ++j)
#pragma unroll
      for (int i = 0; i < N; ++i) {
        pl[(j * N + i) * 2] = pu[j][i];
        pl[(j * N + i) * 2 + 1] = pv[j][i];
      }
  }
}

// Along ξ2: one item per (cell, node indices j, i), the cell slowest, which forms the rows of the
// N nodes (i, j, k) and writes them at their Lagrange positions (perm: tensor slot to Lagrange
// node).
template <typename F, int N, int M, int T>
__device__ __forceinline__ void tile_rows(const VjpSfArgs& a, const F* P, int ps, const uint32_t* perm,
                                          const F* B2, const F* D2, int m2, int64_t tile) {
  using A = Ar<F>;
  constexpr int D = 3, K = N * N * N, R = 4, TILE = kTileCells;
  const int64_t cell0 = a.first_cell + tile * TILE;
  for (int it = threadIdx.x; it < N * N * TILE; it += T) {
    const int l = it / (N * N), r = it % (N * N);
    const int i = r % N, j = r / N;
    const int64_t cell = cell0 + l;
    if (cell >= a.range_end) continue;
    F acc[N][D];
#pragma unroll
    for (int k = 0; k < N; ++k)
#pragma unroll
      for (int g = 0; g < D; ++g) acc[k][g] = F(0);
#pragma unroll
    for (int c2 = 0; c2 < (M > 0 ? M : m2); ++c2)
#pragma unroll
      for (int g = 0; g < D; ++g) {
        const F* pp = P + l * ps + ((c2 * D + g) * N * N + j * N + i) * 2;
        const F pu = pp[0], pv = pp[1];
#pragma unroll
        for (int k = 0; k < N; ++k) acc[k][g] = A::fma(B2[c2 * N + k], pu, A::fma(D2[c2 * N + k], pv, acc[k][g]));
      }
#pragma unroll
    for (int k = 0; k < N; ++k) {
      F* row4 = static_cast<F*>(a.local) + (cell * K + perm[i + N * (j + N * k)]) * R;
      if constexpr (sizeof(F) == 4) {
        *reinterpret_cast<float4*>(row4) = make_float4(acc[k][0], acc[k][1], acc[k][2], 0.0f);
      } else {
        reinterpret_cast<double2*>(row4)[0] = make_double2(acc[k][0], acc[k][1]);
        reinterpret_cast<double2*>(row4)[1] = make_double2(acc[k][2], 0.0);
      }
    }
  }
}

// The adjoint from forward fields already written (vjp_sumfact_bwd_kernel's work, tiled; 144
// threads, so that each phase of a Q2 tile at 27 points is whole rounds of items):
// `a.out[2]` (det J) and `a.out[3]` (K) are read per (point, cell) with the cotangents, x̄ and J̄
// put in shared memory; then tile_planes and tile_rows. Two barriers per tile. M > 0: M points
// in each direction.
constexpr int kTileBwdThreads = 144;

template <typename F, int N, int M>
__global__ void __launch_bounds__(kTileBwdThreads, sizeof(F) == 4 ? 5 : 3) vjp_sumfact_tile_kernel(const __grid_constant__ VjpSfArgs a) {
  constexpr int D = 3, LJ = 9, TILE = kTileCells, T = kTileBwdThreads, QS = kTileQS;
  __shared__ uint64_t bar;
  extern __shared__ __align__(16) unsigned char smem[];
  if (!stage_table(a.tab, smem, a.tab_bytes, &bar, a.err)) return;
  const uint32_t* perm = reinterpret_cast<const uint32_t*>(smem + a.off_perm);
  const int m0 = M > 0 ? M : a.m[0], m1 = M > 0 ? M : a.m[1], m2 = M > 0 ? M : a.m[2];
  const int nq = a.num_points;
  const int ps = m2 * D * N * N * 2 + 1;
  F* V = reinterpret_cast<F*>(smem + (a.tab_bytes + 15) / 16 * 16);
  F* P = V + (size_t)nq * QS;
  const F* B0 = reinterpret_cast<const F*>(smem + a.off_b[0]);
  const F* D0 = reinterpret_cast<const F*>(smem + a.off_d[0]);
  const F* B1 = reinterpret_cast<const F*>(smem + a.off_b[1]);
  const F* D1 = reinterpret_cast<const F*>(smem + a.off_d[1]);
  const F* B2 = reinterpret_cast<const F*>(smem + a.off_b[2]);
  const F* D2 = reinterpret_cast<const F*>(smem + a.off_d[2]);
  const F* ctx = static_cast<const F*>(a.ct[0]);
  const F* ctd = static_cast<const F*>(a.ct[1]);
  const F* ctk = static_cast<const F*>(a.ct[2]);
  const F* fdet = static_cast<const F*>(a.out[2]);
  const F* fk = static_cast<const F*>(a.out[3]);
  __syncthreads();
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
      tile_jbar<F>(db, ctk ? kb : nullptr, det, kinv, jb);
      tile_put_record<F>(V + (size_t)q * QS + l * kTileRec, xb, jb);
    }
    __syncthreads();
    tile_planes<F, N, M, T>(V, P, ps, B0, D0, B1, D1, m0, m1, m2);
    __syncthreads();
    tile_rows<F, N, M, T>(a, P, ps, perm, B2, D2, m2, tile);
  }
}

// Shared memory past the tables of the kernel above: x̄ and J̄ of a tile's points (12 * 16 per
// point) and the tile's plane sums (16 cells x (2 * 3 * N^2 * m2 + 1)), of F.
inline size_t vjp_sumfact_tile_extra_bytes(int n, int num_points, int m2, size_t f_bytes) {
  return f_bytes * ((size_t)num_points * kTileQS + 16 * ((size_t)m2 * 3 * n * n * 2 + 1));
}

}  // namespace tlg
