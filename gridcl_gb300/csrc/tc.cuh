// Tensor-core evaluation for cells of many nodes (geometry degree >= 3): the node-by-basis
// contraction as a GEMM on the tensor cores, X (cells x nodes, per coordinate) times
// Phi (nodes x points * 4: phi, dphi_0, dphi_1, dphi_2 per point), in 3xTF32: each operand split
// into a TF32 head and a TF32 tail, C = Ah Bh + Ah Bl + Al Bh accumulated in FP32, which keeps the
// error at the level of FP32 arithmetic (the dropped Al Bl term and the tails' rounding are
// O(2^-21) relative).
//
// One warp per output tile of 16 cells. The warp gathers its cells' coordinates relative to each
// cell's first node (an f32 mesh in f32; an f64 mesh in f64, rounded to f32, as split precision
// does), so that the TF32 rounding is relative to the cell's size, splits them into head and
// tail, and stores them in shared memory in fragment order: per k-step of 8 nodes and per
// coordinate, each lane's four A values (rows = cells lane/4 and lane/4 + 8, nodes lane%4 and
// lane%4 + 4), head and tail, as two 16-byte words. The basis table is in fragment order in global
// memory (L1/L2-resident): per column tile of 8 (two points) and k-step, each lane's two B values
// (node lane%4 and lane%4 + 4, column lane/4), head and tail, one 16-byte word. Per column tile the
// warp issues 3 x 3 mma.sync.m16n8k8 per k-step (three coordinates, three products); lane pairs
// (lane, lane ^ 1) then exchange halves so that each lane holds x and J of one (cell, point) and
// runs its epilogue (det J, K, normals, facet normals, the stores; in split precision the
// condition estimate and the FP64 recompute).
#pragma once

#include <cstdint>
#include <type_traits>

#include "convert.cuh"
#include "eval.cuh"

namespace tlg {

struct TcArgs {
  const void* nodes;
  const uint32_t* dofmap;
  const uint32_t* flags;
  const float4* bfrag;        // [col tile][k-step][lane] (b0 head, b1 head, b0 tail, b1 tail)
  const float* refn;          // reference normals [Q][TD] (facet rules), f32
  const double* dphi64;       // split: the f64 derivative table [Q][K][TD] of the recompute
  void* out[6];               // points, jacobian, detj, pinv, normals, facet normals (f32)
  unsigned long long* recomputed;
  int64_t first_cell, padded, range_cells, out_first_cell, last_cell, last_flag;
  double origin[3];
  float cond_limit;
  uint32_t last_node, mask;
  int k, ksteps, num_points, col_tiles;
};

// The TF32 head of a float (round to nearest, ties away, as cvt.rna.tf32.f32).
__device__ __forceinline__ uint32_t tf32_head(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void mma_tf32(float* d, const uint32_t* a, uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

constexpr int kTcWarps = 4;

// Shared memory per warp: ksteps x GD x 32 lanes x (4 head + 4 tail) floats.
inline size_t tc_smem_bytes(int ksteps, int gd) { return (size_t)kTcWarps * ksteps * gd * 32 * 8 * 4; }

template <bool SPLIT, int TD, int GD>
__global__ void __launch_bounds__(kTcWarps * 32) tc_eval_kernel(const __grid_constant__ TcArgs a) {
  using A = Ar<float>;
  using M = Factors<float, TD, GD>;
  using NT = typename std::conditional<SPLIT, double, float>::type;
  constexpr int LJ = TD * GD, TILE = 16;
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int K = a.k, KS = a.ksteps, nq = a.num_points;
  float4* frag = reinterpret_cast<float4*>(smem) + (size_t)warp * KS * GD * 32 * 2;  // [ks][g][lane][head, tail]
  const NT* nodes = static_cast<const NT*>(a.nodes);
  const uint32_t mask = a.mask;
  const int grp = lane >> 2, tig = lane & 3;
  const int64_t tiles = a.padded / TILE;

  for (int64_t w = (int64_t)blockIdx.x * kTcWarps + warp; w < tiles; w += (int64_t)gridDim.x * kTcWarps) {
    const int64_t c0 = w * TILE;  // first cell of the tile, relative to the range
    // The epilogue cell of this lane: row grp for even tig, grp + 8 for odd.
    const int my_row = grp + ((tig & 1) ? 8 : 0);
    const int64_t my_cell = min(a.first_cell + c0 + my_row, a.last_cell);
    const uint32_t* my_dof = a.dofmap + my_cell * K;
    // Gather: lane handles rows r = lane % 16, nodes k with k % 2 == lane / 16.
    {
      const int r = lane & 15;
      const int64_t cell = min(a.first_cell + c0 + r, a.last_cell);
      const uint32_t* row = a.dofmap + cell * K;
      // Coordinates relative to the cell's first node (f64 for split precision, f32 otherwise), so
      // that the TF32 splits round relative to the cell's size.
      NT x0[GD];
      {
        const uint32_t n0 = min(__ldg(row), a.last_node);
#pragma unroll
        for (int g = 0; g < GD; ++g) x0[g] = __ldg(nodes + (int64_t)n0 * GD + g);
      }
      for (int k = lane >> 4; k < KS * 8; k += 2) {
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
        // A element (row r, node k) belongs to k-step k / 8, lane (r % 8) * 4 + k % 4, slot
        // (r >= 8) + 2 * (k % 8 >= 4).
        const int ks = k >> 3, kk = k & 7;
        const int dst_lane = (r & 7) * 4 + (kk & 3);
        const int slot = (r >> 3) + 2 * (kk >> 2);
#pragma unroll
        for (int g = 0; g < GD; ++g) {
          const uint32_t h = tf32_head(y[g]);
          const uint32_t t = tf32_head(y[g] - __uint_as_float(h));
          float* base = reinterpret_cast<float*>(frag + (((size_t)ks * GD + g) * 32 + dst_lane) * 2);
          base[slot] = __uint_as_float(h);
          base[4 + slot] = __uint_as_float(t);
        }
      }
    }
    __syncwarp();
    // This lane's epilogue cell: x = xh + (xl + X) with the f32 pair of x_0 + origin (split), or
    // x = (X + x_0) + origin (f32 mesh).
    float xh[GD], xl[GD];
    if constexpr (SPLIT) {
      const uint32_t n0 = min(__ldg(my_dof), a.last_node);
#pragma unroll
      for (int g = 0; g < GD; ++g) {
        const double v = __ldg(static_cast<const double*>(a.nodes) + (int64_t)n0 * GD + g) + a.origin[g];
        xh[g] = d2f_rn(v);
        xl[g] = d2f_rn(v - f2d_exact(xh[g]));
      }
    } else {  // xh: the cell's first node, xl: the origin
      const uint32_t n0 = min(__ldg(my_dof), a.last_node);
#pragma unroll
      for (int g = 0; g < GD; ++g) {
        xh[g] = __ldg(static_cast<const float*>(a.nodes) + (int64_t)n0 * GD + g);
        xl[g] = (float)a.origin[g];
      }
    }
    float sign = 1.0f;
    if ((mask & kOutNormals) && a.flags != nullptr && a.last_flag >= 0) {
      const uint32_t f = __ldg(a.flags + min(a.first_cell + c0 + my_row, a.last_flag));
      sign = (f & 1u) ? -1.0f : 1.0f;
    }
    const int64_t o = a.out_first_cell + c0 + my_row;
    const int64_t tile_idx = o / TILE;
    const int tl = (int)(o % TILE);

    for (int j = 0; j < a.col_tiles; ++j) {
      // Three accumulators per coordinate (head x head, and the two cross terms), summed at the
      // end: nine independent mma chains per warp instead of three.
      float acc[GD][4], acx[GD][4], acy[GD][4];
#pragma unroll
      for (int g = 0; g < GD; ++g)
#pragma unroll
        for (int i = 0; i < 4; ++i) acc[g][i] = acx[g][i] = acy[g][i] = 0.0f;
      const float4* bj = a.bfrag + (size_t)j * KS * 32 + lane;
      for (int ks = 0; ks < KS; ++ks) {
        const float4 b = __ldg(bj + ks * 32);
        const uint32_t bh0 = __float_as_uint(b.x), bh1 = __float_as_uint(b.y);
        const uint32_t bt0 = __float_as_uint(b.z), bt1 = __float_as_uint(b.w);
#pragma unroll
        for (int g = 0; g < GD; ++g) {
          const float4* f = frag + (((size_t)ks * GD + g) * 32 + lane) * 2;
          const float4 ah = f[0], at = f[1];
          const uint32_t ahv[4] = {__float_as_uint(ah.x), __float_as_uint(ah.y), __float_as_uint(ah.z),
                                   __float_as_uint(ah.w)};
          const uint32_t atv[4] = {__float_as_uint(at.x), __float_as_uint(at.y), __float_as_uint(at.z),
                                   __float_as_uint(at.w)};
          mma_tf32(acx[g], atv, bh0, bh1);
          mma_tf32(acy[g], ahv, bt0, bt1);
          mma_tf32(acc[g], ahv, bh0, bh1);
        }
      }
#pragma unroll
      for (int g = 0; g < GD; ++g)
#pragma unroll
        for (int i = 0; i < 4; ++i) acc[g][i] = A::add(acc[g][i], A::add(acx[g][i], acy[g][i]));
      // acc[g] = C_g at (row grp, cols 2 tig, 2 tig + 1) and (row grp + 8, same cols). Column
      // 4 p + r of the tile is point 2 j + p, r = 0 phi, 1 + d dphi_d. Even tig holds (phi,
      // dphi_0), odd tig (dphi_1, dphi_2), of point tig / 2; the pair exchanges halves.
      const bool odd = tig & 1;
      float v[GD][4];  // phi, dphi_0, dphi_1, dphi_2 of this lane's cell and point
#pragma unroll
      for (int g = 0; g < GD; ++g) {
        const float s0 = odd ? acc[g][0] : acc[g][2];
        const float s1 = odd ? acc[g][1] : acc[g][3];
        const float r0 = __shfl_xor_sync(0xFFFFFFFFu, s0, 1);
        const float r1 = __shfl_xor_sync(0xFFFFFFFFu, s1, 1);
        if (odd) {
          v[g][0] = r0;
          v[g][1] = r1;
          v[g][2] = acc[g][2];
          v[g][3] = acc[g][3];
        } else {
          v[g][0] = acc[g][0];
          v[g][1] = acc[g][1];
          v[g][2] = r0;
          v[g][3] = r1;
        }
      }
      const int q = 2 * j + (tig >> 1);
      if (q >= nq) continue;
      float x[GD], jm[LJ];
#pragma unroll
      for (int g = 0; g < GD; ++g) {
        x[g] = v[g][0];
#pragma unroll
        for (int d = 0; d < TD; ++d) jm[d * GD + g] = v[g][1 + d];
      }
      if (mask & kOutPoints) {
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
      if constexpr (SPLIT) {
        const float kap = M::condition(jm, kk);
        if (!(kap <= a.cond_limit) && (mask & (kOutJacobian | kOutDetJ | kOutPinv))) {
          float jr[LJ], kr[LJ], dr;
          recompute_f64_rt<TD, GD>(static_cast<const double*>(a.nodes), my_dof, K, a.last_node,
                                   a.dphi64 + (int64_t)q * K * TD, jr, &dr, kr, 1);
#pragma unroll
          for (int i = 0; i < LJ; ++i) {
            jm[i] = jr[i];
            kk[i] = kr[i];
          }
          dj = dr;
          if (a.recomputed && c0 + my_row < a.range_cells) atomicAdd(a.recomputed, 1ull);
        }
      }
      if (mask & kOutJacobian) store_point(static_cast<float*>(a.out[1]), tile_idx, q, nq, LJ, tl, 4, jm, LJ);
      if (mask & kOutDetJ) store_point(static_cast<float*>(a.out[2]), tile_idx, q, nq, 1, tl, 4, &dj, 1);
      if (mask & kOutPinv) store_point(static_cast<float*>(a.out[3]), tile_idx, q, nq, LJ, tl, 4, kk, LJ);
      if constexpr (TD == GD) {
        if (mask & kOutFacetNormals) {
          float n[GD];
          M::facet_normal(kk, a.refn + q * TD, n);
          store_point(static_cast<float*>(a.out[5]), tile_idx, q, nq, GD, tl, 4, n, GD);
        }
      }
      if constexpr (TD + 1 == GD) {
        if (mask & kOutNormals) {
          float n[GD];
          M::normal(jm, sign, n);
          store_point(static_cast<float*>(a.out[4]), tile_idx, q, nq, GD, tl, 4, n, GD);
        }
      }
    }
    __syncwarp();
  }
}

}  // namespace tlg
