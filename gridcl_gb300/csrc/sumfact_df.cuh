// Sum-factorised evaluation in double-float arithmetic (f64 meshes and fields; df.cuh) for
// quadrilaterals, hexahedra and prisms at tensor-product point sets: the contractions of
// sumfact.cuh (tetraloma-geometry/src/sumfact/tensor.rs:66-432, sumfact/prism.rs:23-136) with every
// multiply-add a double-float one (DfAcc), on the tables' double-float sum-factorisation section
// (B_d, D_d as (head, tail) f32 pairs; the direction whose points go two at a time stored per point
// pair).
//
// Tile 16. The cell's coordinates relative to its node 0, y_l = x_l - x_0 in lexicographic node
// order, go to shared-memory slots as (head, tail) pairs; the plane and row stages run on single
// double-floats in registers, the point stage on point pairs (the paired FP32 instructions), and
// each pair's det J, K, normals and facet normals follow in double-float, assembled into f64 and
// stored.
//  - sumfact_df_kernel: one cell per thread (quadrilaterals, Q1 hexahedra, facet normals);
//  - sumfact_df3_kernel: hexahedra with three lanes per cell, lane g computing coordinate g;
//  - sumfact_prism_df_kernel: prisms, one cell per thread, the z points two at a time.
#pragma once

#include <cstdint>

#include "df.cuh"
#include "sumfact.cuh"

namespace tlg {

// Slots of the single-thread kernels: K * GD (head, tail) pairs per thread.
inline size_t sumfact_df_slot_bytes(int k, int gd) { return (size_t)k * gd * kEvalThreads * 8; }

// The address of component 0 of point q of a cell in an f64 field of `len` components (tile 16;
// tq = the cell's tile index times the point count, lane its lane); component c is 16 values on.
__device__ __forceinline__ double* df_at(double* out, int64_t tq, int q, int len, int lane) {
  return out + (((tq + q) * len) << 4) + lane;
}

// The entry (point pair p, column i) of a paired table: (head of a, head of a + 1, tail of a, tail
// of a + 1) as a double-float of pairs.
__device__ __forceinline__ DF<float2> df_pair_entry(const float4* t, int p, int cols, int i) {
  const float4 e = t[p * cols + i];
  DF<float2> r;
  r.h = make_float2(e.x, e.y);
  r.l = make_float2(e.z, e.w);
  return r;
}

// One point pair's outputs (q1 only when `both`): X relative to x_0 + origin, J.
template <int TD, int GD, bool FN>
__device__ __forceinline__ void sf_df_pair(const SfArgs& a, int q0, int q1, bool both, int64_t tq, int lane,
                                           const DF<float2>* xr, const DF<float2>* j, DF<float2> sign,
                                           const float* oh, const float* ol, const double* refn) {
  constexpr int LJ = TD * GD;
  using D = DF<float2>;
  using B = Ar<float2>;
  using A = Ar<D>;
  using M = Factors<D, TD, GD>;
  const uint32_t mask = a.mask;
  auto put = [&](int slot, int len, const D* v) {
    double* p0 = df_at(static_cast<double*>(a.out[slot]), tq, q0, len, lane);
#pragma unroll
    for (int c = 0; c < len; ++c) p0[c * 16] = df_to_f64(v[c].h.x, v[c].l.x);
    if (both) {
      double* p1 = df_at(static_cast<double*>(a.out[slot]), tq, q1, len, lane);
#pragma unroll
      for (int c = 0; c < len; ++c) p1[c * 16] = df_to_f64(v[c].h.y, v[c].l.y);
    }
  };
  if (mask & kOutPoints) {
    D x[GD];
#pragma unroll
    for (int g = 0; g < GD; ++g) x[g] = A::add(A::make(B::splat(oh[g]), B::splat(ol[g])), xr[g]);
    put(0, GD, x);
  }
  if ((mask & ~kOutPoints) == 0) return;
  if (mask & kOutJacobian) put(1, LJ, j);
  if (mask & kOutDetJ) {
    const D dj = M::detj(j);
    put(2, 1, &dj);
  }
  if (mask & (kOutPinv | kOutFacetNormals)) {
    D kk[LJ];
    M::pinv(j, kk);
    if (mask & kOutPinv) put(3, LJ, kk);
    if constexpr (FN && TD == GD) {
      if (mask & kOutFacetNormals) {
        D nr[TD], n[GD];
        const int qb = both ? q1 : q0;
#pragma unroll
        for (int t = 0; t < TD; ++t) {
          float h0, l0, h1, l1;
          df_split(refn[q0 * TD + t], h0, l0);
          df_split(refn[qb * TD + t], h1, l1);
          nr[t] = A::make(make_float2(h0, h1), make_float2(l0, l1));
        }
        M::facet_normal(kk, nr, n);
        put(5, GD, n);
      }
    }
  }
  if constexpr (TD + 1 == GD) {
    if (mask & kOutNormals) {
      D n[GD];
      M::normal(j, sign, n);
      put(4, GD, n);
    }
  }
}

// The cell's coordinates relative to node 0, lexicographic order, into this thread's slots; the
// double-float x_0 + origin into (oh, ol).
template <int K, int GD>
__device__ __forceinline__ void df_cell_slots(const SfArgs& a, const uint32_t* row, const uint32_t* perm, float2* ys,
                                              float* oh, float* ol) {
  const double* nodes = static_cast<const double*>(a.nodes);
  const uint32_t n0 = min(__ldg(row), a.last_node);
  double x0[GD];
#pragma unroll
  for (int g = 0; g < GD; ++g) {
    x0[g] = __ldg(nodes + (int64_t)n0 * GD + g);
    df_split(__dadd_rn(x0[g], a.origin[g]), oh[g], ol[g]);
  }
#pragma unroll 3
  for (int l = 0; l < K; ++l) {
    const uint32_t n = min(__ldg(row + perm[l]), a.last_node);
#pragma unroll
    for (int g = 0; g < GD; ++g) {
      float h, lo;
      df_split(__dsub_rn(__ldg(nodes + (int64_t)n * GD + g), x0[g]), h, lo);
      ys[(l * GD + g) * kEvalThreads] = make_float2(h, lo);
    }
  }
}

template <int TD, int GD, int N, bool FN>
__global__ void __launch_bounds__(kEvalThreads) sumfact_df_kernel(const __grid_constant__ SfArgs a) {
  using DS = DF<float>;
  using D = DF<float2>;
  using B = Ar<float2>;
  using A = Ar<D>;
  constexpr int K = TD == 3 ? N * N * N : N * N;
  constexpr int LJ = TD * GD;
  constexpr int T = kEvalThreads;
  __shared__ uint64_t bar;
  extern __shared__ __align__(16) unsigned char smem[];
  if (!stage_table(a.tab, smem, a.tab_bytes, &bar, a.err)) return;
  float2* ys = reinterpret_cast<float2*>(smem + (a.tab_bytes + 15) / 16 * 16) + threadIdx.x;
  const uint32_t* perm = reinterpret_cast<const uint32_t*>(smem + a.off_perm);
  const SfBlock* blocks = reinterpret_cast<const SfBlock*>(smem);
  const double* refn = reinterpret_cast<const double*>(smem + a.off_refn);
  const uint32_t mask = a.mask;
  const int nq = a.num_points;

  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < a.padded;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cell = min(a.first_cell + c, a.last_cell);
    const uint32_t* row = a.dofmap + cell * K;
    float oh[GD], ol[GD];
    df_cell_slots<K, GD>(a, row, perm, ys, oh, ol);
    D sign = A::splat(1.0f);
    if ((mask & kOutNormals) && a.flags != nullptr && a.last_flag >= 0) {
      const uint32_t f = __ldg(a.flags + min(a.first_cell + c, a.last_flag));
      sign = A::splat((f & 1u) ? -1.0f : 1.0f);
    }
    const int64_t o = a.out_first_cell + c;
    const int64_t tq = (o >> 4) * nq;
    const int lane = (int)(o & 15);

    for (int bk = 0; bk < a.nblocks; ++bk) {
      const SfBlock& h = blocks[bk];
      const float4* B0 = reinterpret_cast<const float4*>(smem + h.off_b[0]);  // point pairs
      const float4* D0 = reinterpret_cast<const float4*>(smem + h.off_d[0]);
      const float2* B1 = reinterpret_cast<const float2*>(smem + h.off_b[1]);
      const float2* D1 = reinterpret_cast<const float2*>(smem + h.off_d[1]);
      const float2* B2 = reinterpret_cast<const float2*>(smem + h.off_b[2]);
      const float2* D2 = reinterpret_cast<const float2*>(smem + h.off_d[2]);
      const int m0 = h.m[0], m1 = h.m[1], m2 = TD == 3 ? h.m[2] : 1;
      const int s0 = h.s[0], s1 = h.s[1], s2 = h.s[2], qo = h.o;
      for (int c2 = 0; c2 < m2; ++c2) {
        // Plane c2 (hexahedra): U = x B2[c2], V = x D2[c2] over direction 2; quadrilaterals take the
        // coordinates themselves as the plane (U = x, V unused).
        DS U[GD][N][N], V[GD][N][N];
        if constexpr (TD == 3) {
          DfAcc<float> au[GD][N][N], av[GD][N][N];
#pragma unroll
          for (int g = 0; g < GD; ++g)
#pragma unroll
            for (int jj = 0; jj < N; ++jj)
#pragma unroll
              for (int i = 0; i < N; ++i) {
                au[g][jj][i].zero();
                av[g][jj][i].zero();
              }
#pragma unroll
          for (int k = 0; k < N; ++k) {
            const float2 bk2 = B2[c2 * N + k], dk2 = D2[c2 * N + k];
#pragma unroll
            for (int jj = 0; jj < N; ++jj)
#pragma unroll
              for (int i = 0; i < N; ++i)
#pragma unroll
                for (int g = 0; g < GD; ++g) {
                  const float2 xv = ys[((i + N * (jj + N * k)) * GD + g) * T];
                  au[g][jj][i].add(xv.x, xv.y, bk2.x, bk2.y);
                  av[g][jj][i].add(xv.x, xv.y, dk2.x, dk2.y);
                }
          }
#pragma unroll
          for (int g = 0; g < GD; ++g)
#pragma unroll
            for (int jj = 0; jj < N; ++jj)
#pragma unroll
              for (int i = 0; i < N; ++i) {
                U[g][jj][i] = au[g][jj][i].value();
                V[g][jj][i] = av[g][jj][i].value();
              }
        } else {
#pragma unroll
          for (int g = 0; g < GD; ++g)
#pragma unroll
            for (int jj = 0; jj < N; ++jj)
#pragma unroll
              for (int i = 0; i < N; ++i) {
                const float2 xv = ys[((i + N * jj) * GD + g) * T];
                U[g][jj][i].h = xv.x;
                U[g][jj][i].l = xv.y;
              }
        }
        for (int b1 = 0; b1 < m1; ++b1) {
          // Row b1: UU = U B1[b1], UD = U D1[b1], VU = V B1[b1] over direction 1.
          DS UU[GD][N], UD[GD][N], VU[GD][N];
          {
            DfAcc<float> auu[GD][N], aud[GD][N], avu[GD][N];
#pragma unroll
            for (int g = 0; g < GD; ++g)
#pragma unroll
              for (int i = 0; i < N; ++i) {
                auu[g][i].zero();
                aud[g][i].zero();
                avu[g][i].zero();
              }
#pragma unroll
            for (int jj = 0; jj < N; ++jj) {
              const float2 bj = B1[b1 * N + jj], dj = D1[b1 * N + jj];
#pragma unroll
              for (int g = 0; g < GD; ++g)
#pragma unroll
                for (int i = 0; i < N; ++i) {
                  auu[g][i].add(U[g][jj][i].h, U[g][jj][i].l, bj.x, bj.y);
                  aud[g][i].add(U[g][jj][i].h, U[g][jj][i].l, dj.x, dj.y);
                  if constexpr (TD == 3) avu[g][i].add(V[g][jj][i].h, V[g][jj][i].l, bj.x, bj.y);
                }
            }
#pragma unroll
            for (int g = 0; g < GD; ++g)
#pragma unroll
              for (int i = 0; i < N; ++i) {
                UU[g][i] = auu[g][i].value();
                UD[g][i] = aud[g][i].value();
                if constexpr (TD == 3) VU[g][i] = avu[g][i].value();
              }
          }
          // Points along direction 0, two at a time.
          for (int a0 = 0; a0 < m0; a0 += 2) {
            const bool both = a0 + 1 < m0;
            D xr[GD], j[LJ];
            {
              DfAcc<float2> ax[GD], aj[LJ];
#pragma unroll
              for (int g = 0; g < GD; ++g) ax[g].zero();
#pragma unroll
              for (int r = 0; r < LJ; ++r) aj[r].zero();
#pragma unroll
              for (int i = 0; i < N; ++i) {
                const D bi = df_pair_entry(B0, a0 >> 1, N, i), di = df_pair_entry(D0, a0 >> 1, N, i);
#pragma unroll
                for (int g = 0; g < GD; ++g) {
                  const float2 uh = B::splat(UU[g][i].h), ul = B::splat(UU[g][i].l);
                  ax[g].add(uh, ul, bi.h, bi.l);
                  aj[0 * GD + g].add(uh, ul, di.h, di.l);
                  aj[1 * GD + g].add(B::splat(UD[g][i].h), B::splat(UD[g][i].l), bi.h, bi.l);
                  if constexpr (TD == 3) aj[2 * GD + g].add(B::splat(VU[g][i].h), B::splat(VU[g][i].l), bi.h, bi.l);
                }
              }
#pragma unroll
              for (int g = 0; g < GD; ++g) xr[g] = ax[g].value();
#pragma unroll
              for (int r = 0; r < LJ; ++r) j[r] = aj[r].value();
            }
            const int q = qo + a0 * s0 + b1 * s1 + c2 * s2;
            sf_df_pair<TD, GD, FN>(a, q, q + s0, both, tq, lane, xr, j, sign, oh, ol, refn);
          }
        }
      }
    }  // blocks
  }
}

// Prisms: per triangle point i the cell's coordinates against psi, d_x psi, d_y psi (BV, BX, BY),
// then per z point with l, l' (sumfact.cuh's sumfact_prism_kernel); the z points two at a time.
template <int N, bool FN>
__global__ void __launch_bounds__(kEvalThreads) sumfact_prism_df_kernel(const __grid_constant__ SfArgs a) {
  using DS = DF<float>;
  using D = DF<float2>;
  using B = Ar<float2>;
  using A = Ar<D>;
  constexpr int TD = 3, GD = 3, NT = N * (N + 1) / 2, K = NT * N, LJ = TD * GD;
  constexpr int T = kEvalThreads;
  __shared__ uint64_t bar;
  extern __shared__ __align__(16) unsigned char smem[];
  if (!stage_table(a.tab, smem, a.tab_bytes, &bar, a.err)) return;
  float2* ys = reinterpret_cast<float2*>(smem + (a.tab_bytes + 15) / 16 * 16) + threadIdx.x;
  const uint32_t* perm = reinterpret_cast<const uint32_t*>(smem + a.off_perm);
  const SfBlock* blocks = reinterpret_cast<const SfBlock*>(smem);
  const double* refn = reinterpret_cast<const double*>(smem + a.off_refn);
  const int nq = a.num_points;

  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < a.padded;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cell = min(a.first_cell + c, a.last_cell);
    const uint32_t* row = a.dofmap + cell * K;
    float oh[GD], ol[GD];
    df_cell_slots<K, GD>(a, row, perm, ys, oh, ol);
    const int64_t o = a.out_first_cell + c;
    const int64_t tq = (o >> 4) * nq;
    const int lane = (int)(o & 15);

    for (int bk = 0; bk < a.nblocks; ++bk) {
      const SfBlock& h = blocks[bk];
      const float2* PV = reinterpret_cast<const float2*>(smem + h.off_b[0]);
      const float2* PX = reinterpret_cast<const float2*>(smem + h.off_d[0]);
      const float2* PY = reinterpret_cast<const float2*>(smem + h.off_d[1]);
      const float4* LV = reinterpret_cast<const float4*>(smem + h.off_b[2]);  // point pairs
      const float4* LD = reinterpret_cast<const float4*>(smem + h.off_d[2]);
      const int mt = h.m[0], mz = h.m[2], st = h.s[0], sz = h.s[2], qo = h.o;
      for (int i = 0; i < mt; ++i) {
        DS bv[GD][N], bx[GD][N], by[GD][N];
        {
          DfAcc<float> av[GD][N], ax[GD][N], ay[GD][N];
#pragma unroll
          for (int g = 0; g < GD; ++g)
#pragma unroll
            for (int cc = 0; cc < N; ++cc) {
              av[g][cc].zero();
              ax[g][cc].zero();
              ay[g][cc].zero();
            }
#pragma unroll 1
          for (int t = 0; t < NT; ++t) {
            const float2 w = PV[i * NT + t], wx = PX[i * NT + t], wy = PY[i * NT + t];
#pragma unroll
            for (int cc = 0; cc < N; ++cc)
#pragma unroll
              for (int g = 0; g < GD; ++g) {
                const float2 xv = ys[((cc * NT + t) * GD + g) * T];
                av[g][cc].add(xv.x, xv.y, w.x, w.y);
                ax[g][cc].add(xv.x, xv.y, wx.x, wx.y);
                ay[g][cc].add(xv.x, xv.y, wy.x, wy.y);
              }
          }
#pragma unroll
          for (int g = 0; g < GD; ++g)
#pragma unroll
            for (int cc = 0; cc < N; ++cc) {
              bv[g][cc] = av[g][cc].value();
              bx[g][cc] = ax[g][cc].value();
              by[g][cc] = ay[g][cc].value();
            }
        }
        for (int jz = 0; jz < mz; jz += 2) {
          const bool both = jz + 1 < mz;
          D xr[GD], j[LJ];
          {
            DfAcc<float2> acx[GD], acj[LJ];
#pragma unroll
            for (int g = 0; g < GD; ++g) acx[g].zero();
#pragma unroll
            for (int r = 0; r < LJ; ++r) acj[r].zero();
#pragma unroll
            for (int cc = 0; cc < N; ++cc) {
              const D l = df_pair_entry(LV, jz >> 1, N, cc), ld = df_pair_entry(LD, jz >> 1, N, cc);
#pragma unroll
              for (int g = 0; g < GD; ++g) {
                const float2 vh = B::splat(bv[g][cc].h), vl = B::splat(bv[g][cc].l);
                acx[g].add(vh, vl, l.h, l.l);
                acj[0 * GD + g].add(B::splat(bx[g][cc].h), B::splat(bx[g][cc].l), l.h, l.l);
                acj[1 * GD + g].add(B::splat(by[g][cc].h), B::splat(by[g][cc].l), l.h, l.l);
                acj[2 * GD + g].add(vh, vl, ld.h, ld.l);
              }
            }
#pragma unroll
            for (int g = 0; g < GD; ++g) xr[g] = acx[g].value();
#pragma unroll
            for (int r = 0; r < LJ; ++r) j[r] = acj[r].value();
          }
          const int q = qo + i * st + jz * sz;
          sf_df_pair<TD, GD, FN>(a, q, q + sz, both, tq, lane, xr, j, A::splat(1.0f), oh, ol, refn);
        }
      }
    }  // blocks
  }
}

// Hexahedra with three lanes per cell: lane g of a cell's group computes coordinate g (its
// contractions only need that coordinate), so a lane holds a third of the cell's intermediates
// (the single-thread kernel needs more than 255 registers at Q2 and spills). Per point pair a lane
// has row g of J, (J(g, 0), J(g, 1), J(g, 2)); the group exchanges rows by shuffles, and lane g
// forms the cofactor row C_g = J_{g+1} x J_{g+2} (cyclic rows), so that K(t, g) = C_g[t] / det J
// (the adjugate over the determinant, tetraloma-geometry/src/layout.rs:218-268) is its own
// column of K, and det J = J_0 . C_0 (the expansion along the first row, as layout.rs:184-213)
// comes from lane 0 of the group. Ten cells per warp (lanes 30, 31 repeat the tenth cell's first two
// coordinates and store nothing); coordinates in shared-memory slots [K][thread]. No facet
// normals (the single-thread kernel runs those).
inline size_t sumfact_df3_slot_bytes(int k) { return (size_t)k * kEvalThreads * 8; }

template <int N, int MINB>
__global__ void __launch_bounds__(kEvalThreads, MINB) sumfact_df3_kernel(const __grid_constant__ SfArgs a) {
  using DS = DF<float>;
  using D = DF<float2>;
  using B = Ar<float2>;
  using A = Ar<D>;
  constexpr int K = N * N * N;
  constexpr int T = kEvalThreads;
  __shared__ uint64_t bar;
  extern __shared__ __align__(16) unsigned char smem[];
  if (!stage_table(a.tab, smem, a.tab_bytes, &bar, a.err)) return;
  float2* ys = reinterpret_cast<float2*>(smem + (a.tab_bytes + 15) / 16 * 16) + threadIdx.x;
  const uint32_t* perm = reinterpret_cast<const uint32_t*>(smem + a.off_perm);
  const SfBlock* blocks = reinterpret_cast<const SfBlock*>(smem);
  const double* nodes = static_cast<const double*>(a.nodes);
  const int lane = threadIdx.x & 31;
  const int cl = lane < 30 ? lane / 3 : 9;  // the warp's cell of this lane
  const int g = lane < 30 ? lane - 3 * cl : lane - 30;
  const int base = 3 * cl;  // the group's first lane
  const int src1 = base + (g + 1) % 3, src2 = base + (g + 2) % 3;
  const int nq = a.num_points;
  const uint32_t mask = a.mask;
  const int64_t warps = (int64_t)gridDim.x * (T / 32);
  double* outx = static_cast<double*>(a.out[0]);
  double* outj = static_cast<double*>(a.out[1]);
  double* outd = static_cast<double*>(a.out[2]);
  double* outk = static_cast<double*>(a.out[3]);

  for (int64_t w = (int64_t)blockIdx.x * (T / 32) + threadIdx.x / 32; w * 10 < a.padded; w += warps) {
    const int64_t c = w * 10 + cl;
    const bool live = lane < 30 && c < a.padded;
    const int64_t cc = min(c, a.padded - 1);
    const int64_t cell = min(a.first_cell + cc, a.last_cell);
    const uint32_t* row = a.dofmap + cell * K;
    // Coordinate g of the cell's nodes relative to node 0, lexicographic order.
    const uint32_t n0 = min(__ldg(row), a.last_node);
    const double x0 = __ldg(nodes + (int64_t)n0 * 3 + g);
    float oh, ol;
    df_split(__dadd_rn(x0, a.origin[g]), oh, ol);
#pragma unroll 3
    for (int l = 0; l < K; ++l) {
      const uint32_t n = min(__ldg(row + perm[l]), a.last_node);
      float h, lo;
      df_split(__dsub_rn(__ldg(nodes + (int64_t)n * 3 + g), x0), h, lo);
      ys[l * T] = make_float2(h, lo);
    }
    const int64_t o = a.out_first_cell + cc;
    const int64_t tq = (o >> 4) * nq;
    const int l16 = (int)(o & 15);

    for (int bk = 0; bk < a.nblocks; ++bk) {
      const SfBlock& h = blocks[bk];
      const float4* B0 = reinterpret_cast<const float4*>(smem + h.off_b[0]);  // point pairs
      const float4* D0 = reinterpret_cast<const float4*>(smem + h.off_d[0]);
      const float2* B1 = reinterpret_cast<const float2*>(smem + h.off_b[1]);
      const float2* D1 = reinterpret_cast<const float2*>(smem + h.off_d[1]);
      const float2* B2 = reinterpret_cast<const float2*>(smem + h.off_b[2]);
      const float2* D2 = reinterpret_cast<const float2*>(smem + h.off_d[2]);
      const int m0 = h.m[0], m1 = h.m[1], m2 = h.m[2];
      const int s0 = h.s[0], s1 = h.s[1], s2 = h.s[2], qo = h.o;
      for (int c2 = 0; c2 < m2; ++c2) {
        DS U[N][N], V[N][N];
        {
          DfAcc<float> au[N][N], av[N][N];
#pragma unroll
          for (int jj = 0; jj < N; ++jj)
#pragma unroll
            for (int i = 0; i < N; ++i) {
              au[jj][i].zero();
              av[jj][i].zero();
            }
#pragma unroll
          for (int k = 0; k < N; ++k) {
            const float2 bk2 = B2[c2 * N + k], dk2 = D2[c2 * N + k];
#pragma unroll
            for (int jj = 0; jj < N; ++jj)
#pragma unroll
              for (int i = 0; i < N; ++i) {
                const float2 xv = ys[(i + N * (jj + N * k)) * T];
                au[jj][i].add(xv.x, xv.y, bk2.x, bk2.y);
                av[jj][i].add(xv.x, xv.y, dk2.x, dk2.y);
              }
          }
#pragma unroll
          for (int jj = 0; jj < N; ++jj)
#pragma unroll
            for (int i = 0; i < N; ++i) {
              U[jj][i] = au[jj][i].value();
              V[jj][i] = av[jj][i].value();
            }
        }
        for (int b1 = 0; b1 < m1; ++b1) {
          DS UU[N], UD[N], VU[N];
          {
            DfAcc<float> auu[N], aud[N], avu[N];
#pragma unroll
            for (int i = 0; i < N; ++i) {
              auu[i].zero();
              aud[i].zero();
              avu[i].zero();
            }
#pragma unroll
            for (int jj = 0; jj < N; ++jj) {
              const float2 bj = B1[b1 * N + jj], dj = D1[b1 * N + jj];
#pragma unroll
              for (int i = 0; i < N; ++i) {
                auu[i].add(U[jj][i].h, U[jj][i].l, bj.x, bj.y);
                aud[i].add(U[jj][i].h, U[jj][i].l, dj.x, dj.y);
                avu[i].add(V[jj][i].h, V[jj][i].l, bj.x, bj.y);
              }
            }
#pragma unroll
            for (int i = 0; i < N; ++i) {
              UU[i] = auu[i].value();
              UD[i] = aud[i].value();
              VU[i] = avu[i].value();
            }
          }
          for (int a0 = 0; a0 < m0; a0 += 2) {
            const bool both = a0 + 1 < m0;
            D xr, r[3];  // X_g - x_0 - origin, row g of J
            {
              DfAcc<float2> ax, aj0, aj1, aj2;
              ax.zero();
              aj0.zero();
              aj1.zero();
              aj2.zero();
#pragma unroll
              for (int i = 0; i < N; ++i) {
                const D bi = df_pair_entry(B0, a0 >> 1, N, i), di = df_pair_entry(D0, a0 >> 1, N, i);
                const float2 uh = B::splat(UU[i].h), ul = B::splat(UU[i].l);
                ax.add(uh, ul, bi.h, bi.l);
                aj0.add(uh, ul, di.h, di.l);
                aj1.add(B::splat(UD[i].h), B::splat(UD[i].l), bi.h, bi.l);
                aj2.add(B::splat(VU[i].h), B::splat(VU[i].l), bi.h, bi.l);
              }
              xr = ax.value();
              r[0] = aj0.value();
              r[1] = aj1.value();
              r[2] = aj2.value();
            }
            // The other two rows of the group.
            D p[3], s[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
              p[d].h.x = __shfl_sync(0xffffffffu, r[d].h.x, src1);
              p[d].h.y = __shfl_sync(0xffffffffu, r[d].h.y, src1);
              p[d].l.x = __shfl_sync(0xffffffffu, r[d].l.x, src1);
              p[d].l.y = __shfl_sync(0xffffffffu, r[d].l.y, src1);
              s[d].h.x = __shfl_sync(0xffffffffu, r[d].h.x, src2);
              s[d].h.y = __shfl_sync(0xffffffffu, r[d].h.y, src2);
              s[d].l.x = __shfl_sync(0xffffffffu, r[d].l.x, src2);
              s[d].l.y = __shfl_sync(0xffffffffu, r[d].l.y, src2);
            }
            // Cofactor row g: J_{g+1} x J_{g+2}; det J from lane 0 of the group.
            D cof[3];
            cof[0] = A::fma(p[1], s[2], A::neg(A::mul(p[2], s[1])));
            cof[1] = A::fma(p[2], s[0], A::neg(A::mul(p[0], s[2])));
            cof[2] = A::fma(p[0], s[1], A::neg(A::mul(p[1], s[0])));
            D det = A::fma(r[2], cof[2], A::fma(r[0], cof[0], A::mul(r[1], cof[1])));
            det.h.x = __shfl_sync(0xffffffffu, det.h.x, base);
            det.h.y = __shfl_sync(0xffffffffu, det.h.y, base);
            det.l.x = __shfl_sync(0xffffffffu, det.l.x, base);
            det.l.y = __shfl_sync(0xffffffffu, det.l.y, base);
            if (!live) continue;
            const int q0 = qo + a0 * s0 + b1 * s1 + c2 * s2;
            const int q1 = both ? q0 + s0 : q0;  // (stores of q1 only when both)
            if (mask & kOutPoints) {
              const D x = A::add(A::make(B::splat(oh), B::splat(ol)), xr);
              df_at(outx, tq, q0, 3, l16)[g * 16] = df_to_f64(x.h.x, x.l.x);
              if (both) df_at(outx, tq, q1, 3, l16)[g * 16] = df_to_f64(x.h.y, x.l.y);
            }
            if (mask & kOutJacobian) {
              double* p0 = df_at(outj, tq, q0, 9, l16) + g * 16;
              double* p1 = df_at(outj, tq, q1, 9, l16) + g * 16;
#pragma unroll
              for (int d = 0; d < 3; ++d) {
                p0[d * 48] = df_to_f64(r[d].h.x, r[d].l.x);
                if (both) p1[d * 48] = df_to_f64(r[d].h.y, r[d].l.y);
              }
            }
            if ((mask & kOutDetJ) && g == 0) {
              df_at(outd, tq, q0, 1, l16)[0] = df_to_f64(det.h.x, det.l.x);
              if (both) df_at(outd, tq, q1, 1, l16)[0] = df_to_f64(det.h.y, det.l.y);
            }
            if (mask & kOutPinv) {
              const D inv = A::rcp(det);
              double* p0 = df_at(outk, tq, q0, 9, l16) + g * 48;
              double* p1 = df_at(outk, tq, q1, 9, l16) + g * 48;
#pragma unroll
              for (int t = 0; t < 3; ++t) {
                const D kt = A::mul(cof[t], inv);
                p0[t * 16] = df_to_f64(kt.h.x, kt.l.x);
                if (both) p1[t * 16] = df_to_f64(kt.h.y, kt.l.y);
              }
            }
          }
        }
      }
    }  // blocks
  }
}

}  // namespace tlg
