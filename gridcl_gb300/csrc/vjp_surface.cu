// The adjoint with K at run time: below codimension 0 (curves in 2D or 3D and surfaces in 3D,
// TD < GD), and in codimension 0 for the elements without a node-row kernel (P4+ tetrahedra, Q3+
// hexahedra at other than tensor rules, ...), where P = 0 and the area element is det J. Below
// codimension 0, with
// cotangents on x, the area element a = sqrt(det(J^T J)), the pseudo-inverse K = G^-1 J^T
// (G = J^T J) and, for TD + 1 = GD, the unit normal n = s v / |v| (v = J0 x J1 in 3D,
// (J0_y, -J0_x) in 2D; s = -1 where bit 0 of the cell's flag is set). Per point
//   dL/dJ = dbar a K^T - K^T Kbar K^T + P Kbar^T G^-1 + (normal term),  P = I - J K,
// the normal term from w = s (nbar - (nbar . v^) v^) / |v|: dL/dJ0 += J1 x w, dL/dJ1 += w x J0
// (3D) or dL/dJ0 += (-w_y, w_x) (2D); the contributions L(cell, k, g) = sum_q phi_k xbar_g +
// sum_d dphi_k[d] dL/dJ(g, d) go to the rows the gather reads.
//
// One cell per thread; the cell's coordinates and its contributions sit in the thread's slots in
// shared memory (K x GD each, interleaved over the threads), K at run time. f64 with TLG_F64
// tables; with TLG_SPLIT32 tables FP32 arithmetic on coordinates shifted by the cell's first node
// (f32 cotangents, contributions and forward fields). The forward fields (x, J, a, K, n) can be
// written in the same pass.
#include <cstdint>
#include <type_traits>

#include "convert.cuh"
#include "eval.cuh"
#include "vjp.cuh"

namespace tlg {

template <typename F, bool SPLIT, int TD, int GD>
__global__ void __launch_bounds__(kEvalThreads) vjp_surface_kernel(const __grid_constant__ VjpSurfArgs a) {
  using NT = typename std::conditional<SPLIT, double, F>::type;
  using M = Factors<F, TD, GD>;
  using A = Ar<F>;
  constexpr int LJ = TD * GD, R = GD == 3 ? 4 : GD, TILE = 16;
  __shared__ uint64_t bar;
  extern __shared__ __align__(16) unsigned char smem[];
  const unsigned char* tabs = a.tab;
  size_t slot_base = 0;
  if (!a.tab_global) {
    if (!stage_table(a.tab, smem, a.tab_bytes, &bar, a.err)) return;
    tabs = smem;
    slot_base = (a.tab_bytes + 15) / 16 * 16;
  }
  const F* phi = reinterpret_cast<const F*>(tabs);
  const F* dphi = reinterpret_cast<const F*>(tabs + a.off_dphi);
  const int T = blockDim.x, K = a.k, nq = a.num_points;
  F* xs = reinterpret_cast<F*>(smem + slot_base) + threadIdx.x;  // [K][GD] coordinates
  F* ls = xs + (size_t)K * GD * T;                                  // [K][GD] contributions
  const NT* nodes = static_cast<const NT*>(a.nodes);
  const F* ctx = static_cast<const F*>(a.ct[0]);
  const F* ctd = static_cast<const F*>(a.ct[1]);
  const F* ctk = static_cast<const F*>(a.ct[2]);
  const F* ctn = static_cast<const F*>(a.ct[3]);

  for (int64_t c = (int64_t)blockIdx.x * T + threadIdx.x; c < a.padded; c += (int64_t)gridDim.x * T) {
    const int64_t cell = min(a.first_cell + c, a.last_cell);
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
    for (int l = 0; l < K; ++l) {
      const uint32_t n = min(__ldg(row + l), a.last_node);
#pragma unroll
      for (int g = 0; g < GD; ++g) {
        const NT v = __ldg(nodes + (int64_t)n * GD + g);
        if constexpr (SPLIT) xs[(l * GD + g) * T] = d2f_rn(v - x0[g]);
        else xs[(l * GD + g) * T] = v;
        ls[(l * GD + g) * T] = F(0);
      }
    }
    F sgn = F(1);
    if (a.flags != nullptr && a.last_flag >= 0) {
      const uint32_t f = __ldg(a.flags + min(a.first_cell + c, a.last_flag));
      sgn = (f & 1u) ? F(-1) : F(1);
    }
    const int64_t o = a.out_first_cell + c;
    const int64_t tq = (o / TILE) * nq;
    const int l16 = (int)(o % TILE);
#define TLG_AT(q, len, comp) (((tq + (q)) * (len) + (comp)) * TILE + l16)
    for (int q = 0; q < nq; ++q) {
      F x[GD], j[LJ];
#pragma unroll
      for (int g = 0; g < GD; ++g) x[g] = F(0);
#pragma unroll
      for (int i = 0; i < LJ; ++i) j[i] = F(0);
      for (int l = 0; l < K; ++l) {
        const F w = phi[q * K + l];
        F dw[TD];
#pragma unroll
        for (int d = 0; d < TD; ++d) dw[d] = dphi[(q * K + l) * TD + d];
#pragma unroll
        for (int g = 0; g < GD; ++g) {
          const F xv = xs[(l * GD + g) * T];
          x[g] = A::fma(xv, w, x[g]);
#pragma unroll
          for (int d = 0; d < TD; ++d) j[d * GD + g] = A::fma(xv, dw[d], j[d * GD + g]);
        }
      }
      // J(g, d) at d * GD + g; K(t, g) at g * TD + t.
      F kk[LJ], n[GD];
      M::pinv(j, kk);
      const F area = M::detj(j);
      if constexpr (TD + 1 == GD) M::normal(j, sgn, n);
      if (a.out[0]) {
#pragma unroll
        for (int g = 0; g < GD; ++g)
          static_cast<F*>(a.out[0])[TLG_AT(q, GD, g)] = SPLIT ? xh[g] + (xl[g] + x[g]) : x[g] + xh[g];
      }
      if (a.out[1])
#pragma unroll
        for (int i = 0; i < LJ; ++i) static_cast<F*>(a.out[1])[TLG_AT(q, LJ, i)] = j[i];
      if (a.out[2]) static_cast<F*>(a.out[2])[TLG_AT(q, 1, 0)] = area;
      if (a.out[3])
#pragma unroll
        for (int i = 0; i < LJ; ++i) static_cast<F*>(a.out[3])[TLG_AT(q, LJ, i)] = kk[i];
      if constexpr (TD + 1 == GD) {
        if (a.out[4])
#pragma unroll
          for (int g = 0; g < GD; ++g) static_cast<F*>(a.out[4])[TLG_AT(q, GD, g)] = n[g];
      }

      F jb[LJ];
      const F db = ctd ? ctd[TLG_AT(q, 1, 0)] : F(0);
#pragma unroll
      for (int g = 0; g < GD; ++g)
#pragma unroll
        for (int d = 0; d < TD; ++d) jb[d * GD + g] = db * area * kk[g * TD + d];
      if (ctk && TD == GD) {  // codimension 0: P = 0, Jbar -= K^T Kbar K^T
        F kb[LJ];
#pragma unroll
        for (int i = 0; i < LJ; ++i) kb[i] = ctk[TLG_AT(q, LJ, i)];
#pragma unroll
        for (int g = 0; g < GD; ++g)
#pragma unroll
          for (int d = 0; d < TD; ++d) {
            F v = F(0);
#pragma unroll
            for (int t = 0; t < TD; ++t) {
              F kt = F(0);
#pragma unroll
              for (int h = 0; h < GD; ++h) kt = A::fma(kb[h * TD + t], kk[h * TD + d], kt);
              v = A::fma(-kk[g * TD + t], kt, v);
            }
            jb[d * GD + g] += v;
          }
      } else if (ctk) {
        F kb[LJ], gi[TD * TD], pm[GD * GD];
#pragma unroll
        for (int i = 0; i < LJ; ++i) kb[i] = ctk[TLG_AT(q, LJ, i)];
        // G^-1 = K K^T (K = G^-1 J^T), P = I - J K.
#pragma unroll
        for (int t = 0; t < TD; ++t)
#pragma unroll
          for (int u = 0; u < TD; ++u) {
            F s = F(0);
#pragma unroll
            for (int g = 0; g < GD; ++g) s = A::fma(kk[g * TD + t], kk[g * TD + u], s);
            gi[t * TD + u] = s;
          }
#pragma unroll
        for (int g = 0; g < GD; ++g)
#pragma unroll
          for (int h = 0; h < GD; ++h) {
            F s = g == h ? F(1) : F(0);
#pragma unroll
            for (int t = 0; t < TD; ++t) s = A::fma(-j[t * GD + g], kk[h * TD + t], s);
            pm[g * GD + h] = s;
          }
#pragma unroll
        for (int g = 0; g < GD; ++g)
#pragma unroll
          for (int d = 0; d < TD; ++d) {
            F v = F(0);
#pragma unroll
            for (int t = 0; t < TD; ++t) {
              F kt = F(0), pt = F(0);
#pragma unroll
              for (int h = 0; h < GD; ++h) {
                kt = A::fma(kb[h * TD + t], kk[h * TD + d], kt);  // (Kbar K^T)(t, d)
                pt = A::fma(pm[g * GD + h], kb[h * TD + t], pt);  // (P Kbar^T)(g, t)
              }
              v = A::fma(-kk[g * TD + t], kt, v);
              v = A::fma(pt, gi[t * TD + d], v);
            }
            jb[d * GD + g] += v;
          }
      }
      if constexpr (TD + 1 == GD) {
        if (ctn) {
          F v[GD], w[GD], nb[GD];
          if constexpr (GD == 2) {
            v[0] = j[1];
            v[1] = -j[0];
          } else {
            v[0] = j[1] * j[5] - j[2] * j[4];
            v[1] = j[2] * j[3] - j[0] * j[5];
            v[2] = j[0] * j[4] - j[1] * j[3];
          }
          F len2 = F(0);
#pragma unroll
          for (int g = 0; g < GD; ++g) len2 = A::fma(v[g], v[g], len2);
          const F len = A::sqrt(len2), inv = A::rcp(len);
          F dot = F(0);
#pragma unroll
          for (int g = 0; g < GD; ++g) {
            nb[g] = ctn[TLG_AT(q, GD, g)];
            dot = A::fma(nb[g], v[g] * inv, dot);
          }
#pragma unroll
          for (int g = 0; g < GD; ++g) w[g] = sgn * (nb[g] - dot * v[g] * inv) * inv;
          if constexpr (GD == 2) {
            jb[0] += -w[1];
            jb[1] += w[0];
          } else {
            // J1 x w into column 0, w x J0 into column 1.
            jb[0] += j[4] * w[2] - j[5] * w[1];
            jb[1] += j[5] * w[0] - j[3] * w[2];
            jb[2] += j[3] * w[1] - j[4] * w[0];
            jb[3] += w[1] * j[2] - w[2] * j[1];
            jb[4] += w[2] * j[0] - w[0] * j[2];
            jb[5] += w[0] * j[1] - w[1] * j[0];
          }
        }
      }
      F xb[GD];
#pragma unroll
      for (int g = 0; g < GD; ++g) xb[g] = ctx ? ctx[TLG_AT(q, GD, g)] : F(0);
      for (int l = 0; l < K; ++l) {
        const F w = phi[q * K + l];
        F dw[TD];
#pragma unroll
        for (int d = 0; d < TD; ++d) dw[d] = dphi[(q * K + l) * TD + d];
#pragma unroll
        for (int g = 0; g < GD; ++g) {
          F v = w * xb[g];
#pragma unroll
          for (int d = 0; d < TD; ++d) v = A::fma(dw[d], jb[d * GD + g], v);
          ls[(l * GD + g) * T] += v;
        }
      }
    }
#undef TLG_AT
    if (a.first_cell + c < a.range_end) {
      F* dst = static_cast<F*>(a.local) + (a.first_cell + c) * ((int64_t)K * R);
      for (int l = 0; l < K; ++l)
#pragma unroll
        for (int g = 0; g < R; ++g) dst[l * R + g] = g < GD ? ls[(l * GD + g) * T] : F(0);
    }
  }
}

cudaError_t launch_vjp_surface(bool split, int td, int gd, const VjpSurfArgs& a, size_t smem, int threads,
                               cudaStream_t s, bool* found) {
  *found = true;
#define TLG_VS(F, SPLIT, TD, GD) \
  if (td == TD && gd == GD) { \
    auto kern = vjp_surface_kernel<F, SPLIT, TD, GD>; \
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
    if (e != cudaSuccess) return e; \
    int per_sm = 0, sms = 1, dev = 0; \
    cudaGetDevice(&dev); \
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev); \
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, smem) != cudaSuccess || per_sm < 1) \
      per_sm = 1; \
    const int64_t need = (a.padded + threads - 1) / threads; \
    const int64_t cap = (int64_t)sms * per_sm; \
    kern<<<(unsigned)(need < cap ? (need > 0 ? need : 1) : cap), threads, smem, s>>>(a); \
    return cudaGetLastError(); \
  }
  if (split) {
    TLG_VS(float, true, 1, 2)
    TLG_VS(float, true, 1, 3)
    TLG_VS(float, true, 2, 3)
    TLG_VS(float, true, 1, 1)
    TLG_VS(float, true, 2, 2)
    TLG_VS(float, true, 3, 3)
  } else {
    TLG_VS(double, false, 1, 2)
    TLG_VS(double, false, 1, 3)
    TLG_VS(double, false, 2, 3)
    TLG_VS(double, false, 1, 1)
    TLG_VS(double, false, 2, 2)
    TLG_VS(double, false, 3, 3)
  }
#undef TLG_VS
  *found = false;
  return cudaSuccess;
}

}  // namespace tlg
