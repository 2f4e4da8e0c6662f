// Fused geometry-evaluation kernels for sm_103a.
//
// One thread per cell of a block range. Each CTA stages the element's tabulation (values
// [Q][K], derivatives [Q][K][TD], reference facet normals [Q][TD], all in F) from global memory
// into its own shared memory with one bulk asynchronous copy (cp.async.bulk completing on an
// mbarrier); every thread then reads table entries at warp-uniform addresses, which shared
// memory broadcasts. A thread gathers its cell's K nodes through the dofmap (index clamped to
// the last node, the cell clamped to the block's last cell, tetraloma-geometry/src/evector.rs:
// 221-222) into registers and walks the Q points: J, then every requested factor from J, each
// stored straight into its QuadField chunk at ((cell / tile) * Q * LEN + q * LEN + k) * tile +
// cell % tile (tetraloma-geometry/src/field.rs:121-162). Consecutive threads are consecutive
// cells, so each warp store covers whole tile rows.
//
// Arithmetic follows tetraloma-geometry/src/layout.rs:133-369: J(g, d) is the sum over the
// nodes in ascending k starting with the k = 0 product; det J and K by the same cofactor
// formulas; normals as s (J0 x J1) / |J0 x J1|. The CTAs are persistent (a grid-stride loop),
// so the table is staged once per CTA.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

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
  uint32_t off_dphi;         // byte offset of the derivative table
  uint32_t off_refn;         // byte offset of the reference normals
  uint32_t mask;             // kOut* bits
  int num_points;            // Q
  int tile_shift;            // log2(tile)
  int k_runtime;             // K for the loops kernel
};

// ----------------------------------------------------------------------------------------
// Table staging: one elected thread issues a bulk copy into shared memory; all threads wait on
// the mbarrier with a bounded number of polls. On expiry the CTA records an error and does a
// second bounded wait for its copy before it lets the caller continue.

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

__device__ __forceinline__ bool stage_table(const unsigned char* src, unsigned char* dst,
                                            uint32_t bytes, uint64_t* bar, int* err) {
  const uint32_t bar_s = (uint32_t)__cvta_generic_to_shared(bar);
  const uint32_t dst_s = (uint32_t)__cvta_generic_to_shared(dst);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar_s) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar_s), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(dst_s),
        "l"(src), "r"(bytes), "r"(bar_s)
        : "memory");
  }
  // Bounded poll: try_wait itself suspends for a hardware-defined interval per call.
  const int kPolls = 1 << 22;
  for (int i = 0; i < kPolls; ++i)
    if (mbar_try_wait(bar_s, 0)) return true;
  if (err) atomicExch(err, 1);
  for (int i = 0; i < kPolls; ++i)
    if (mbar_try_wait(bar_s, 0)) break;
  return false;
}

// ----------------------------------------------------------------------------------------
// Factor math on J (column-major GD x TD), tetraloma-geometry/src/layout.rs:166-369.

template <typename F, int TD, int GD>
struct Factors {
  __device__ static F column_dot(const F* j, int a, int b) {
    F acc = j[a * GD] * j[b * GD];
#pragma unroll
    for (int g = 1; g < GD; ++g) acc = fma(j[a * GD + g], j[b * GD + g], acc);
    return acc;
  }

  __device__ static F square_det(const F* j) {
    if constexpr (TD == 1) {
      return j[0];
    } else if constexpr (TD == 2) {
      return j[0] * j[3] - j[2] * j[1];
    } else {
      return j[0] * (j[4] * j[8] - j[7] * j[5]) - j[3] * (j[1] * j[8] - j[7] * j[2]) +
             j[6] * (j[1] * j[5] - j[4] * j[2]);
    }
  }

  __device__ static F detj(const F* j) {
    if constexpr (TD == GD) {
      return square_det(j);
    } else if constexpr (TD == 1) {
      return sqrt(column_dot(j, 0, 0));
    } else {
      const F a = column_dot(j, 0, 0), b = column_dot(j, 0, 1), c = column_dot(j, 1, 1);
      return sqrt(a * c - b * b);
    }
  }

  // K(t, g) at g * TD + t.
  __device__ static void pinv(const F* j, F* k) {
    if constexpr (TD == GD) {
      const F inv = F(1) / square_det(j);
      if constexpr (TD == 1) {
        k[0] = inv;
      } else if constexpr (TD == 2) {
        k[0] = j[3] * inv;
        k[2] = -j[2] * inv;
        k[1] = -j[1] * inv;
        k[3] = j[0] * inv;
      } else {
        k[0] = (j[4] * j[8] - j[7] * j[5]) * inv;
        k[3] = (j[6] * j[5] - j[3] * j[8]) * inv;
        k[6] = (j[3] * j[7] - j[6] * j[4]) * inv;
        k[1] = (j[7] * j[2] - j[1] * j[8]) * inv;
        k[4] = (j[0] * j[8] - j[6] * j[2]) * inv;
        k[7] = (j[6] * j[1] - j[0] * j[7]) * inv;
        k[2] = (j[1] * j[5] - j[4] * j[2]) * inv;
        k[5] = (j[3] * j[2] - j[0] * j[5]) * inv;
        k[8] = (j[0] * j[4] - j[3] * j[1]) * inv;
      }
    } else if constexpr (TD == 1) {
      const F inv = F(1) / column_dot(j, 0, 0);
#pragma unroll
      for (int g = 0; g < GD; ++g) k[g] = j[g] * inv;
    } else {
      const F a = column_dot(j, 0, 0), b = column_dot(j, 0, 1), c = column_dot(j, 1, 1);
      const F inv = F(1) / (a * c - b * b);
      const F g00 = c * inv, g01 = -b * inv, g11 = a * inv;
#pragma unroll
      for (int g = 0; g < GD; ++g) {
        k[g * TD] = g00 * j[g] + g01 * j[GD + g];
        k[g * TD + 1] = g01 * j[g] + g11 * j[GD + g];
      }
    }
  }

  // Codimension 1: s (J0_y, -J0_x) / |J0| or s (J0 x J1) / |J0 x J1|.
  __device__ static void normal(const F* j, F s, F* n) {
    F v[GD];
    if constexpr (GD == 2) {
      v[0] = j[1];
      v[1] = -j[0];
    } else {
      v[0] = j[1] * j[5] - j[2] * j[4];
      v[1] = j[2] * j[3] - j[0] * j[5];
      v[2] = j[0] * j[4] - j[1] * j[3];
    }
    F s2 = v[0] * v[0];
#pragma unroll
    for (int g = 1; g < GD; ++g) s2 = fma(v[g], v[g], s2);
    const F norm = sqrt(s2);
#pragma unroll
    for (int g = 0; g < GD; ++g) n[g] = (s * v[g]) / norm;
  }

  // Codimension 0: m = K^T n_ref, m / |m|.
  __device__ static void facet_normal(const F* k, const F* nref, F* n) {
    F m[GD];
#pragma unroll
    for (int g = 0; g < GD; ++g) {
      F acc = k[g * TD] * nref[0];
#pragma unroll
      for (int t = 1; t < TD; ++t) acc = fma(k[g * TD + t], nref[t], acc);
      m[g] = acc;
    }
    F s2 = m[0] * m[0];
#pragma unroll
    for (int g = 1; g < GD; ++g) s2 = fma(m[g], m[g], s2);
    const F norm = sqrt(s2);
#pragma unroll
    for (int g = 0; g < GD; ++g) n[g] = m[g] / norm;
  }
};

// Stores `len` components of one point of one cell: element (tile, q, comp, lane).
template <typename F>
__device__ __forceinline__ void store_point(F* out, int64_t tile_idx, int q, int nq, int len,
                                            int lane, int tile_shift, const F* v, int n) {
  F* base = out + ((((tile_idx * nq + q) * len) << tile_shift) + lane);
  for (int c = 0; c < n; ++c) base[(int64_t)c << tile_shift] = v[c];
}

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
// The direct kernel: K, TD, GD at compile time, everything unrolled over nodes and dimensions.

template <typename F, int TD, int GD, int K>
__global__ void __launch_bounds__(kEvalThreads) eval_direct_kernel(const __grid_constant__ EvalArgs<F> a) {
  __shared__ uint64_t bar;
  extern __shared__ __align__(16) unsigned char smem[];
  stage_table(a.tab, smem, a.tab_bytes, &bar, a.err);
  const F* phi = reinterpret_cast<const F*>(smem);
  const F* dphi = reinterpret_cast<const F*>(smem + a.off_dphi);
  const F* refn = reinterpret_cast<const F*>(smem + a.off_refn);
  const int nq = a.num_points;
  const uint32_t mask = a.mask;
  const bool want_j = (mask & ~kOutPoints) != 0;
  constexpr int LJ = TD * GD;
  const int tile_mask = (1 << a.tile_shift) - 1;

  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < a.padded;
       c += (int64_t)gridDim.x * blockDim.x) {
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
    const int64_t tile_idx = o >> a.tile_shift;
    const int lane = (int)(o & tile_mask);

    for (int q = 0; q < nq; ++q) {
      if (mask & kOutPoints) {
        F xp[GD];
        const F* w = phi + q * K;
#pragma unroll
        for (int g = 0; g < GD; ++g) xp[g] = x[0][g] * w[0];
#pragma unroll
        for (int k = 1; k < K; ++k) {
          const F wk = w[k];
#pragma unroll
          for (int g = 0; g < GD; ++g) xp[g] = fma(x[k][g], wk, xp[g]);
        }
#pragma unroll
        for (int g = 0; g < GD; ++g) xp[g] = xp[g] + a.origin[g];
        store_point(a.out[0], tile_idx, q, nq, GD, lane, a.tile_shift, xp, GD);
      }
      if (!want_j) continue;
      F j[LJ];
      const F* dq = dphi + q * K * TD;
#pragma unroll
      for (int d = 0; d < TD; ++d) {
        const F w0 = dq[d];
#pragma unroll
        for (int g = 0; g < GD; ++g) j[d * GD + g] = x[0][g] * w0;
      }
#pragma unroll
      for (int k = 1; k < K; ++k) {
#pragma unroll
        for (int d = 0; d < TD; ++d) {
          const F w = dq[k * TD + d];
#pragma unroll
          for (int g = 0; g < GD; ++g) j[d * GD + g] = fma(x[k][g], w, j[d * GD + g]);
        }
      }
      using M = Factors<F, TD, GD>;
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

// ----------------------------------------------------------------------------------------
// The split-precision kernel: f64 mesh in, FP32 arithmetic, f32 fields out.
//
// Each cell's nodes are shifted by its node 0 in f64 (x_k - x_0, FP64 subtractions once per
// cell), then rounded to f32: the shifted coordinates have the size of the cell, so their f32
// rounding is relative to the cell, not to the distance from the origin. J = sum_{k>=1} (x_k - x_0)
// dphi_k (the k = 0 term vanishes; sum_k dphi_k = 0), X = x_0 + sum_{k>=1} (x_k - x_0) phi_k with
// x_0 carried as an f32 pair. det J and K follow in f32. A condition estimate
// kappa = |J|_F |K|_F / TD flags near-degenerate points (kappa above `cond_limit`, or not
// finite); for those J, det J and K are recomputed in FP64 from the f64 nodes and the f64
// derivative table, then rounded to f32, and a device counter records how many points were
// recomputed.

struct SplitArgs {
  const double* nodes;
  const uint32_t* dofmap;
  const uint32_t* flags;
  const unsigned char* tab;  // phi32 | dphi32 | refn32 | dphi64
  float* out[6];
  int* err;
  unsigned long long* recomputed;  // may be null
  int64_t first_cell, padded, out_first_cell, last_cell, last_flag;
  double origin[3];
  float cond_limit;
  uint32_t last_node, tab_bytes, off_dphi, off_refn, off_dphi64, mask;
  int num_points, tile_shift;
};

template <int TD, int GD>
__device__ __forceinline__ float frob(const float* m) {
  float s = m[0] * m[0];
#pragma unroll
  for (int i = 1; i < TD * GD; ++i) s = fmaf(m[i], m[i], s);
  return sqrtf(s);
}

template <int TD, int GD, int K>
__global__ void __launch_bounds__(kEvalThreads) eval_split_kernel(const __grid_constant__ SplitArgs a) {
  __shared__ uint64_t bar;
  extern __shared__ __align__(16) unsigned char smem[];
  stage_table(a.tab, smem, a.tab_bytes, &bar, a.err);
  const float* phi = reinterpret_cast<const float*>(smem);
  const float* dphi = reinterpret_cast<const float*>(smem + a.off_dphi);
  const float* refn = reinterpret_cast<const float*>(smem + a.off_refn);
  const double* dphi64 = reinterpret_cast<const double*>(smem + a.off_dphi64);
  const int nq = a.num_points;
  const uint32_t mask = a.mask;
  const bool want_j = (mask & ~kOutPoints) != 0;
  constexpr int LJ = TD * GD;
  const int tile_mask = (1 << a.tile_shift) - 1;
  using M = Factors<float, TD, GD>;
  using M64 = Factors<double, TD, GD>;

  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < a.padded;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cell = min(a.first_cell + c, a.last_cell);
    uint32_t idx[K];
    load_row<K>(a.dofmap + cell * K, idx);
#pragma unroll
    for (int k = 0; k < K; ++k) idx[k] = min(idx[k], a.last_node);
    double x0[GD];
#pragma unroll
    for (int g = 0; g < GD; ++g) x0[g] = __ldg(a.nodes + (int64_t)idx[0] * GD + g);
    float y[K][GD];
#pragma unroll
    for (int k = 1; k < K; ++k)
#pragma unroll
      for (int g = 0; g < GD; ++g)
        y[k][g] = __double2float_rn(__ldg(a.nodes + (int64_t)idx[k] * GD + g) - x0[g]);
    // x_0 + origin as an f32 pair (hi + lo), for the physical points.
    float xh[GD], xl[GD];
    if (mask & kOutPoints) {
#pragma unroll
      for (int g = 0; g < GD; ++g) {
        const double v = x0[g] + a.origin[g];
        xh[g] = __double2float_rn(v);
        xl[g] = __double2float_rn(v - (double)xh[g]);
      }
    }
    float sign = 1.0f;
    if ((mask & kOutNormals) && a.flags != nullptr && a.last_flag >= 0) {
      const uint32_t f = __ldg(a.flags + min(a.first_cell + c, a.last_flag));
      sign = (f & 1u) ? -1.0f : 1.0f;
    }
    const int64_t o = a.out_first_cell + c;
    const int64_t tile_idx = o >> a.tile_shift;
    const int lane = (int)(o & tile_mask);

    for (int q = 0; q < nq; ++q) {
      if (mask & kOutPoints) {
        float s[GD];
        const float* w = phi + q * K;
#pragma unroll
        for (int g = 0; g < GD; ++g) s[g] = y[1][g] * w[1];
#pragma unroll
        for (int k = 2; k < K; ++k) {
          const float wk = w[k];
#pragma unroll
          for (int g = 0; g < GD; ++g) s[g] = fmaf(y[k][g], wk, s[g]);
        }
#pragma unroll
        for (int g = 0; g < GD; ++g) s[g] = xh[g] + (xl[g] + s[g]);
        store_point(a.out[0], tile_idx, q, nq, GD, lane, a.tile_shift, s, GD);
      }
      if (!want_j) continue;
      float j[LJ];
      const float* dq = dphi + q * K * TD;
#pragma unroll
      for (int d = 0; d < TD; ++d) {
        const float w1 = dq[TD + d];
#pragma unroll
        for (int g = 0; g < GD; ++g) j[d * GD + g] = y[1][g] * w1;
      }
#pragma unroll
      for (int k = 2; k < K; ++k) {
#pragma unroll
        for (int d = 0; d < TD; ++d) {
          const float w = dq[k * TD + d];
#pragma unroll
          for (int g = 0; g < GD; ++g) j[d * GD + g] = fmaf(y[k][g], w, j[d * GD + g]);
        }
      }
      float kk[LJ];
      M::pinv(j, kk);
      float dj = M::detj(j);
      const float kappa = frob<TD, GD>(j) * frob<TD, GD>(kk) * (1.0f / TD);
      if (!(kappa <= a.cond_limit)) {
        // Near-degenerate point: J, det J and K again in FP64 from the f64 nodes.
        double jd[LJ], kd[LJ];
#pragma unroll
        for (int i = 0; i < LJ; ++i) jd[i] = 0.0;
        const double* d64 = dphi64 + q * K * TD;
        for (int k = 1; k < K; ++k) {
#pragma unroll
          for (int g = 0; g < GD; ++g) {
            const double yk = __ldg(a.nodes + (int64_t)idx[k] * GD + g) - x0[g];
#pragma unroll
            for (int d = 0; d < TD; ++d) jd[d * GD + g] = fma(yk, d64[k * TD + d], jd[d * GD + g]);
          }
        }
        M64::pinv(jd, kd);
        dj = (float)M64::detj(jd);
#pragma unroll
        for (int i = 0; i < LJ; ++i) {
          j[i] = (float)jd[i];
          kk[i] = (float)kd[i];
        }
        if (a.recomputed) atomicAdd(a.recomputed, 1ull);
      }
      if (mask & kOutJacobian) store_point(a.out[1], tile_idx, q, nq, LJ, lane, a.tile_shift, j, LJ);
      if (mask & kOutDetJ) store_point(a.out[2], tile_idx, q, nq, 1, lane, a.tile_shift, &dj, 1);
      if (mask & kOutPinv) store_point(a.out[3], tile_idx, q, nq, LJ, lane, a.tile_shift, kk, LJ);
      if constexpr (TD == GD) {
        if (mask & kOutFacetNormals) {
          float n[GD];
          M::facet_normal(kk, refn + q * TD, n);
          store_point(a.out[5], tile_idx, q, nq, GD, lane, a.tile_shift, n, GD);
        }
      }
      if constexpr (TD + 1 == GD) {
        if (mask & kOutNormals) {
          float n[GD];
          M::normal(j, sign, n);
          store_point(a.out[4], tile_idx, q, nq, GD, lane, a.tile_shift, n, GD);
        }
      }
    }
  }
}

// ----------------------------------------------------------------------------------------
// The loops kernel: any K (run time), TD and GD at compile time; node coordinates re-read
// through L1 at each point. Same values as the direct kernel.

template <typename F, int TD, int GD>
__global__ void __launch_bounds__(kEvalThreads) eval_loops_kernel(const __grid_constant__ EvalArgs<F> a) {
  __shared__ uint64_t bar;
  extern __shared__ __align__(16) unsigned char smem[];
  stage_table(a.tab, smem, a.tab_bytes, &bar, a.err);
  const F* phi = reinterpret_cast<const F*>(smem);
  const F* dphi = reinterpret_cast<const F*>(smem + a.off_dphi);
  const F* refn = reinterpret_cast<const F*>(smem + a.off_refn);
  const int nq = a.num_points;
  const int K = a.k_runtime;
  const uint32_t mask = a.mask;
  const bool want_j = (mask & ~kOutPoints) != 0;
  constexpr int LJ = TD * GD;
  const int tile_mask = (1 << a.tile_shift) - 1;

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
          for (int g = 0; g < GD; ++g) xp[g] = k == 0 ? xk[g] * w : fma(xk[g], w, xp[g]);
        }
        if (want_j) {
#pragma unroll
          for (int d = 0; d < TD; ++d) {
            const F w = dphi[(q * K + k) * TD + d];
#pragma unroll
            for (int g = 0; g < GD; ++g)
              j[d * GD + g] = k == 0 ? xk[g] * w : fma(xk[g], w, j[d * GD + g]);
          }
        }
      }
      if (mask & kOutPoints) {
#pragma unroll
        for (int g = 0; g < GD; ++g) xp[g] = xp[g] + a.origin[g];
        store_point(a.out[0], tile_idx, q, nq, GD, lane, a.tile_shift, xp, GD);
      }
      if (!want_j) continue;
      using M = Factors<F, TD, GD>;
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
