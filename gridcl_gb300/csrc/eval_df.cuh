// f64 geometry evaluation in double-float arithmetic on the FP32 pipe (df.cuh): f64 nodes in,
// f64 fields out, errors of a few 1e-14 relative to the fields' largest values (the reference's
// f64 tolerance is 1e-12, tetraloma-testing/src/lib.rs:127-130).
//
// eval_df_kernel<TD, GD, K>: one thread per cell, two quadrature points per instruction (the
// paired FP32 instructions on double-float pairs), tile 16, persistent CTAs that stage the tables
// in shared memory with one bulk copy (eval.cuh). Per cell the K node indices, node 0's f64
// coordinates x_0 and y_k = x_k - x_0 (one FP64 subtraction each) split into double-floats; per
// point pair and node one table row of 16 floats, (phi, dphi_0 .. dphi_{TD-1}) as heads and tails
// of both points. X - x_0 - origin and J accumulate term by term in DfAcc (k = 0 drops out: y_0 = 0),
// X adds x_0 + origin (a double-float per cell), and det J, K, normals and facet normals follow
// in double-float by the formulas of the other kernels (Factors<DF<float2>, TD, GD>); every value
// is assembled into its f64 (df_to_f64) and stored into its QuadField chunk.
#pragma once

#include <cstdint>

#include "df.cuh"
#include "eval.cuh"

namespace tlg {

struct DfArgs {
  const double* nodes;
  const uint32_t* dofmap;
  const uint32_t* flags;
  const unsigned char* tab;  // staged: df rows [QP][K][1 + TD] float4 at off_rows, refn [Q][TD] f64
  double* out[6];
  int* err;
  int64_t first_cell, padded, out_first_cell, last_cell, last_flag;
  double origin[3];
  uint32_t last_node, tab_bytes, off_rows, off_refn, mask;
  int num_points;
  // Monomial form (tetrahedra P1-P3): the rows at off_rows are those of the monomials x^a of the
  // Lagrange space, and off_mono holds the expansion C [k][m] (f32 head, tail) and per monomial
  // the mask of the directions it depends on (u32 bits).
  uint32_t off_mono;
  int mono;
};

// Output cursor of an f64 field (tile 16): point pairs of double-floats, assembled into f64.
template <int LEN>
struct DfCursor {
  double* p;
  __device__ __forceinline__ void init(double* out, int64_t tile_idx, int nq, int lane) {
    p = out + tile_idx * (int64_t)nq * (LEN * 16) + lane;
  }
  __device__ __forceinline__ void put2(const DF<float2>* v, bool both) {
#pragma unroll
    for (int c = 0; c < LEN; ++c) p[c * 16] = df_to_f64(v[c].h.x, v[c].l.x);
    if (both) {
#pragma unroll
      for (int c = 0; c < LEN; ++c) p[(LEN + c) * 16] = df_to_f64(v[c].h.y, v[c].l.y);
    }
    p += 2 * LEN * 16;
  }
};

// Shared memory past the staged tables: per thread the double-float coordinates y_k (k >= 1) as
// (head, tail) f32 pairs, [k - 1][g] with stride kEvalThreads (the lanes of a warp read
// consecutive 8-byte slots); in the monomial form the K coefficient vectors c_m, [m][g].
inline size_t df_slot_bytes(int k, int gd, bool mono = false) {
  return (size_t)(mono ? k : k - 1) * gd * kEvalThreads * 8;
}

// MONO: the monomial form. The map of a cell is x_0 + sum_m c_m x^(a_m) with c_m = sum_k C[m][k]
// y_k, formed once per cell (double-float sums over the nonzero C[m][k]; accumulated in the slots
// and normalised there). At a point J(:, d) = sum over the monomials that depend on x_d of
// c_m d(x^(a_m))/dx_d: for a P2 tetrahedron 12 (monomial, direction) terms instead of the 27 of
// the nine nodes k >= 1, about a third fewer double-float terms per point with x; the same
// epilogue.
template <int TD, int GD, int K, bool MONO = false>
__global__ void __launch_bounds__(kEvalThreads) eval_df_kernel(const __grid_constant__ DfArgs a) {
  constexpr int TILE = 16;
  constexpr int LJ = TD * GD;
  constexpr int RW = 1 + TD;  // float4 rows per node of a point pair
  constexpr int T = kEvalThreads;
  using V = float2;
  using D = DF<V>;
  using B = Ar<V>;
  using A = Ar<D>;
  using M = Factors<D, TD, GD>;
  __shared__ uint64_t bar;
  extern __shared__ __align__(16) unsigned char smem[];
  if (!stage_table(a.tab, smem, a.tab_bytes, &bar, a.err)) return;
  const float4* rows = reinterpret_cast<const float4*>(smem + a.off_rows);
  const double* refn = reinterpret_cast<const double*>(smem + a.off_refn);
  float2* ys = reinterpret_cast<float2*>(smem + (a.tab_bytes + 15) / 16 * 16) + threadIdx.x;
  const int nq = a.num_points;
  const int nqp = (nq + 1) / 2;
  const uint32_t mask = a.mask;
  const bool want_x = (mask & kOutPoints) != 0;
  const bool want_j = (mask & ~kOutPoints) != 0;

  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < a.padded;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cell = min(a.first_cell + c, a.last_cell);
    uint32_t idx[K];
    load_row<K>(a.dofmap + cell * K, idx);
    double x0[GD];
    const uint32_t n0 = min(idx[0], a.last_node);
#pragma unroll
    for (int g = 0; g < GD; ++g) x0[g] = __ldg(a.nodes + (int64_t)n0 * GD + g);
    if constexpr (MONO) {
      // c_m = sum_k C[m][k] y_k (y_0 = 0), accumulated in the slots as (sum, error) pairs.
      const float2* coef = reinterpret_cast<const float2*>(smem + a.off_mono);
#pragma unroll
      for (int i = 0; i < K * GD; ++i) ys[i * T] = make_float2(0.0f, 0.0f);
#pragma unroll 1
      for (int k = 1; k < K; ++k) {
        // The row again through L1 (a rolled loop cannot index idx[] in registers).
        const uint32_t n = min(__ldg(a.dofmap + cell * K + k), a.last_node);
        float yh[GD], yl[GD];
#pragma unroll
        for (int g = 0; g < GD; ++g) df_split(__dsub_rn(__ldg(a.nodes + (int64_t)n * GD + g), x0[g]), yh[g], yl[g]);
#pragma unroll
        for (int m = 0; m < K; ++m) {
          const float2 cm = coef[k * K + m];
          if (cm.x != 0.0f) {
#pragma unroll
            for (int g = 0; g < GD; ++g) {
              const float2 st = ys[(m * GD + g) * T];
              DfAcc<float> acc;
              acc.s = st.x;
              acc.c = st.y;
              acc.add(yh[g], yl[g], cm.x, cm.y);
              ys[(m * GD + g) * T] = make_float2(acc.s, acc.c);
            }
          }
        }
      }
#pragma unroll
      for (int i = 0; i < K * GD; ++i) {
        const float2 st = ys[i * T];
        const DF<float> v = Ar<DF<float>>::fast_two_sum(st.x, st.y);
        ys[i * T] = make_float2(v.h, v.l);
      }
    } else {
      // y_k = x_k - x_0 (k >= 1) into this thread's slots; the k = 0 term of every sum vanishes.
#pragma unroll
      for (int k = 1; k < K; ++k) {
        const uint32_t n = min(idx[k], a.last_node);
#pragma unroll
        for (int g = 0; g < GD; ++g) {
          float h, l;
          df_split(__dsub_rn(__ldg(a.nodes + (int64_t)n * GD + g), x0[g]), h, l);
          ys[((k - 1) * GD + g) * T] = make_float2(h, l);
        }
      }
    }
    float oh[GD], ol[GD];  // x_0 + origin
#pragma unroll
    for (int g = 0; g < GD; ++g) df_split(__dadd_rn(x0[g], a.origin[g]), oh[g], ol[g]);
    D sign = A::splat(1.0f);
    if ((mask & kOutNormals) && a.flags != nullptr && a.last_flag >= 0) {
      const uint32_t f = __ldg(a.flags + min(a.first_cell + c, a.last_flag));
      sign = A::splat((f & 1u) ? -1.0f : 1.0f);
    }
    const int64_t o = a.out_first_cell + c;
    const int64_t tile_idx = o / TILE;
    const int lane = (int)(o % TILE);
    DfCursor<GD> cx, cn, cf;
    DfCursor<LJ> cj, ck;
    DfCursor<1> cd;
    if (mask & kOutPoints) cx.init(a.out[0], tile_idx, nq, lane);
    if (mask & kOutJacobian) cj.init(a.out[1], tile_idx, nq, lane);
    if (mask & kOutDetJ) cd.init(a.out[2], tile_idx, nq, lane);
    if (mask & kOutPinv) ck.init(a.out[3], tile_idx, nq, lane);
    if (mask & kOutNormals) cn.init(a.out[4], tile_idx, nq, lane);
    if (mask & kOutFacetNormals) cf.init(a.out[5], tile_idx, nq, lane);

    for (int qp = 0; qp < nqp; ++qp) {
      const bool both = 2 * qp + 1 < nq;
      const float4* rq = rows + (int64_t)qp * K * RW;
      // X - x_0 - origin and J of the pair, one node per iteration (a rolled loop: the unrolled
      // one outgrows the instruction cache).
      DfAcc<V> ax[GD], aj[LJ];
#pragma unroll
      for (int g = 0; g < GD; ++g) ax[g].zero();
#pragma unroll
      for (int i = 0; i < LJ; ++i) aj[i].zero();
      // (MONO: monomial m's rows, its coefficients in slot m, the directions it depends on.)
      const uint32_t* mmask = reinterpret_cast<const uint32_t*>(smem + a.off_mono + K * K * 8);
#pragma unroll 1
      for (int k = MONO ? 0 : 1; k < K; ++k) {
        float2 y[GD];
#pragma unroll
        for (int g = 0; g < GD; ++g) y[g] = ys[((MONO ? k : k - 1) * GD + g) * T];
        if (want_x) {
          const float4 r = rq[k * RW];
#pragma unroll
          for (int g = 0; g < GD; ++g)
            ax[g].add(B::splat(y[g].x), B::splat(y[g].y), make_float2(r.x, r.y), make_float2(r.z, r.w));
        }
        if (want_j) {
          const uint32_t dep = MONO ? mmask[k] : ~0u;
#pragma unroll
          for (int d = 0; d < TD; ++d) {
            if (!((dep >> d) & 1u)) continue;
            const float4 r = rq[k * RW + 1 + d];
            const V th = make_float2(r.x, r.y), tl = make_float2(r.z, r.w);
#pragma unroll
            for (int g = 0; g < GD; ++g) aj[d * GD + g].add(B::splat(y[g].x), B::splat(y[g].y), th, tl);
          }
        }
      }
      if (want_x) {
        D xs[GD];
#pragma unroll
        for (int g = 0; g < GD; ++g) xs[g] = A::add(A::make(B::splat(oh[g]), B::splat(ol[g])), ax[g].value());
        cx.put2(xs, both);
      }
      if (!want_j) continue;
      D j[LJ];
#pragma unroll
      for (int i = 0; i < LJ; ++i) j[i] = aj[i].value();
      if (mask & kOutJacobian) cj.put2(j, both);
      if (mask & kOutDetJ) {
        const D dj = M::detj(j);
        cd.put2(&dj, both);
      }
      if (mask & (kOutPinv | kOutFacetNormals)) {
        D kk[LJ];
        M::pinv(j, kk);
        if (mask & kOutPinv) ck.put2(kk, both);
        if constexpr (TD == GD) {
          if (mask & kOutFacetNormals) {
            D nr[TD], n[GD];
            const int q1 = min(2 * qp + 1, nq - 1);
#pragma unroll
            for (int t = 0; t < TD; ++t) {
              float h0, l0, h1, l1;
              df_split(refn[(2 * qp) * TD + t], h0, l0);
              df_split(refn[q1 * TD + t], h1, l1);
              nr[t] = A::make(make_float2(h0, h1), make_float2(l0, l1));
            }
            M::facet_normal(kk, nr, n);
            cf.put2(n, both);
          }
        }
      }
      if constexpr (TD + 1 == GD) {
        if (mask & kOutNormals) {
          D n[GD];
          M::normal(j, sign, n);
          cn.put2(n, both);
        }
      }
    }
  }
}

}  // namespace tlg
