// Pull-back: the reference point xi of a physical point y in a cell, by Newton's method on the
// cell's Lagrange map (tetraloma-geometry/src/pull_back.rs:94-330, 566).
//
// Semantics kept from the reference, because the outputs are specified by them: every point
// starts at the vertex centroid of the reference cell (rounded to f32, then to F); exactly
// `max_iterations` steps run for every point (no early exit, so results do not depend on how
// points are grouped); a step is delta = K(xi) (y - X(xi)) with K the (pseudo-)inverse of J;
// a point not yet frozen moves to xi + delta clamped to the box [-0.1, 1.1]^TD (bounds rounded
// to f32), records |delta|_inf (the largest finite value of F when a component is not finite)
// and freezes once that is at most the tolerance; frozen points keep xi and their last step.
//
// The basis at an arbitrary xi is evaluated in product form instead of the reference's
// orthonormal expansion with a coefficient matrix (the same Lagrange functions): on intervals,
// quadrilaterals and hexahedra the product of 1D Lagrange polynomials through the sorted 1D
// nodes; on triangles and tetrahedra (equispaced nodes) the barycentric product
//   phi_alpha = prod_i prod_{j < alpha_i} (p lambda_i - j) / (j + 1),   |alpha| = p,
// whose value is 1 at its node and 0 at the others; prisms multiply the triangle's by the
// line's. The host stores per node its 1D indices or barycentric multi-index. Pyramids (a
// rational space, no product form) go through the expansion, as the reference does: the host's
// orthogonal rationomials evaluated at xi by their recurrences, times the host's coefficient
// matrix (the inverse of their Vandermonde matrix at the nodes).
//
// One cell per thread: the cell's node coordinates (relative to the origin) go to the thread's
// interleaved slots in shared memory, then each point runs its iterations. Tile layout of the
// input points, xi and the steps as the evaluation outputs.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "convert.cuh"
#include "eval.cuh"
#include "refcell.h"
#include "status.h"

struct tlg_basis {
  int cell, degree, family, td;
  int64_t k;
  unsigned char* dev = nullptr;  // the basis header (tlg::BasisData)
};

namespace tlg {

constexpr int kBasisMaxN = 16;    // 1D nodes (degree + 1)
constexpr int kBasisMaxK = 1024;  // nodes per cell
constexpr int kPyramidMaxP = 4;   // pyramid degrees of the pull-back
constexpr int kPyramidMaxK = 55;  // (p + 1)(p + 2)(2p + 3) / 6 at p = 4

// Device copy of the basis description.
struct alignas(16) BasisData {
  int cell, p, k, n;        // cell type, degree, nodes per cell, 1D nodes (p + 1)
  const double* coef;       // pyramids: C [m][k] (m-major) after this header; else null
  double s[kBasisMaxN];     // sorted 1D nodes (tensor cells, the prism's line)
  uint8_t idx[kBasisMaxK][4];  // per node: 1D indices (tensor) or barycentric multi-index
                               // (simplex: lambda_0 .. lambda_TD; prism: alpha_0..2, line index)
};

struct PullBackArgs {
  const void* nodes;
  const uint32_t* dofmap;
  const BasisData* basis;
  const void* x;  // input points, GD components (absolute)
  void* xi;       // TD components
  void* step;     // 1 component
  int64_t first_cell, padded, out_first_cell, x_first_cell, last_cell;
  double origin[3];
  double tolerance;
  uint32_t last_node;
  int num_points, max_iterations, tile_shift, threads;
  int refinements;  // mixed precision: FP64-residual steps after the FP32 iteration (0: native)
};

template <typename F>
__device__ __forceinline__ F fmax_finite();
template <>
__device__ __forceinline__ float fmax_finite<float>() { return 3.402823466e38f; }
template <>
__device__ __forceinline__ double fmax_finite<double>() { return 1.7976931348623157e308; }

// 1D Lagrange values and derivatives l_i(t), l_i'(t), i < n, at the nodes s.
template <typename F>
__device__ void lagrange1d(const double* s, int n, F t, F* v, F* d) {
  for (int i = 0; i < n; ++i) {
    F val = F(1), der = F(0);
    for (int r = 0; r < n; ++r) {
      if (r == i) continue;
      const F w = F(1) / F(s[i] - s[r]);
      der = der * (t - F(s[r])) * w + val * w;
      val = val * (t - F(s[r])) * w;
    }
    v[i] = val;
    d[i] = der;
  }
}

// Barycentric factors f(m) = prod_{j < m} (p lam - j) / (j + 1) and df/dlam, m = 0..p.
template <typename F>
__device__ void simplex_factors(int p, F lam, F* f, F* df) {
  f[0] = F(1);
  df[0] = F(0);
  const F pl = F(p) * lam;
  for (int m = 1; m <= p; ++m) {
    const F inv = F(1) / F(m);
    const F t = (pl - F(m - 1)) * inv;
    df[m] = df[m - 1] * t + f[m - 1] * F(p) * inv;
    f[m] = f[m - 1] * t;
  }
}

// The pyramid's orthogonal rationomials at xi, in the host's order (i outer, then j, then k;
// max(i, j) + k <= p): e[0][m] the values, e[1 + d][m] the derivatives. With s = 1 - z,
//   Q_i(2x - s, s) Q_j(2y - s, s) / s^min(i,j) * P_k^(2 max(i,j) + 2, 0)(2z - 1),
// Q_i the homogeneous Legendre recurrence Q_n = ((2n - 1) f Q_{n-1} - (n - 1) s^2 Q_{n-2}) / n
// and P_k the Jacobi recurrence. At s = 0 the rational ones (min(i, j) >= 1) are 0 with a zero
// gradient, their limit along the axis.
template <typename F>
__device__ void pyramid_set(int p, const F* xi, F (*e)[kPyramidMaxK]) {
  const F s = F(1) - xi[2];
  F q[2][kPyramidMaxP + 1], qd[2][kPyramidMaxP + 1], qz[2][kPyramidMaxP + 1];
  for (int v = 0; v < 2; ++v) {
    const F f = F(2) * xi[v] - s;  // d/dx_v = 2, d/dz = 1
    q[v][0] = F(1);
    qd[v][0] = qz[v][0] = F(0);
    if (p >= 1) {
      q[v][1] = f;
      qd[v][1] = F(2);
      qz[v][1] = F(1);
    }
    for (int n = 2; n <= p; ++n) {
      const F a = F(2 * n - 1) / F(n), c = F(n - 1) / F(n);
      q[v][n] = a * f * q[v][n - 1] - c * s * s * q[v][n - 2];
      qd[v][n] = a * (F(2) * q[v][n - 1] + f * qd[v][n - 1]) - c * s * s * qd[v][n - 2];
      qz[v][n] = a * (q[v][n - 1] + f * qz[v][n - 1]) - c * (s * s * qz[v][n - 2] - F(2) * s * q[v][n - 2]);
    }
  }
  const F t = F(2) * xi[2] - F(1);
  int m = 0;
  for (int i = 0; i <= p; ++i)
    for (int j = 0; j <= p; ++j) {
      const int mx = i > j ? i : j, mn = i < j ? i : j;
      F f = F(0), fx = F(0), fy = F(0), fz = F(0);
      if (mn == 0 || s != F(0)) {
        F sn = F(1);
        for (int r = 0; r < mn; ++r) sn *= s;
        const F r = F(1) / sn;
        const F rz = mn ? F(mn) * r / s : F(0);  // d(s^-mn)/dz
        f = q[0][i] * q[1][j] * r;
        fx = qd[0][i] * q[1][j] * r;
        fy = q[0][i] * qd[1][j] * r;
        fz = (qz[0][i] * q[1][j] + q[0][i] * qz[1][j]) * r + q[0][i] * q[1][j] * rz;
      }
      const F al = F(2 * mx + 2);
      F j2 = F(0), dj2 = F(0), j1 = F(1), dj1 = F(0);  // P_{k-2}, P_{k-1}
      for (int k = 0; k + mx <= p; ++k) {
        F jk, djk;
        if (k == 0) {
          jk = F(1);
          djk = F(0);
        } else if (k == 1) {
          jk = F(0.5) * ((al + F(2)) * t + al);
          djk = al + F(2);
        } else {
          const F kk = F(k);
          const F D = F(2) * kk * (kk + al) * (F(2) * kk + al - F(2));
          const F A = (F(2) * kk + al - F(1)) * (F(2) * kk + al) * (F(2) * kk + al - F(2)) / D;
          const F B = (F(2) * kk + al - F(1)) * al * al / D;
          const F C = F(2) * (kk + al - F(1)) * (kk - F(1)) * (F(2) * kk + al) / D;
          jk = (A * t + B) * j1 - C * j2;
          djk = F(2) * A * j1 + (A * t + B) * dj1 - C * dj2;
        }
        if (k >= 1) {
          j2 = j1;
          dj2 = dj1;
        }
        j1 = jk;
        dj1 = djk;
        e[0][m] = f * jk;
        e[1][m] = fx * jk;
        e[2][m] = fy * jk;
        e[3][m] = fz * jk + f * djk;
        ++m;
      }
    }
}

// X and J of a pyramid at xi through the expansion coefficients.
template <typename F, int GD, bool WANT_J>
__device__ void map_at_pyramid(const BasisData& b, const F* xs, int T, const F* xi, F* X, F* J) {
  F e[4][kPyramidMaxK];
  pyramid_set<F>(b.p, xi, e);
#pragma unroll
  for (int g = 0; g < GD; ++g) X[g] = F(0);
  if constexpr (WANT_J)
#pragma unroll
    for (int i = 0; i < 3 * GD; ++i) J[i] = F(0);
  for (int k = 0; k < b.k; ++k) {
    F phi = F(0), grad[3] = {F(0), F(0), F(0)};
    for (int m = 0; m < b.k; ++m) {
      const F c = F(__ldg(b.coef + (size_t)m * b.k + k));
      phi = fma(e[0][m], c, phi);
      if constexpr (WANT_J)
#pragma unroll
        for (int d = 0; d < 3; ++d) grad[d] = fma(e[1 + d][m], c, grad[d]);
    }
#pragma unroll
    for (int g = 0; g < GD; ++g) {
      const F xk = xs[(k * GD + g) * T];
      X[g] = fma(xk, phi, X[g]);
      if constexpr (WANT_J)
#pragma unroll
        for (int d = 0; d < 3; ++d) J[d * GD + g] = fma(xk, grad[d], J[d * GD + g]);
    }
  }
}

// X (GD) and, with WANT_J, J (J(g, d) at d * GD + g) at xi from the node coordinates in the
// thread's slots.
template <typename F, int TD, int GD, bool WANT_J = true>
__device__ void map_at(const BasisData& b, const F* xs, int T, const F* xi, F* X, F* J) {
  if constexpr (TD == 3) {
    if (b.cell == kPyramid) {
      map_at_pyramid<F, GD, WANT_J>(b, xs, T, xi, X, J);
      return;
    }
  }
  constexpr int MAXN = kBasisMaxN;
  F v[3][MAXN], dv[3][MAXN];
  const int cell = b.cell;
  const bool tensor = cell == kInterval || cell == kQuadrilateral || cell == kHexahedron;
  const bool prism = cell == kPrism;
  if (tensor) {
    for (int d = 0; d < TD; ++d) lagrange1d<F>(b.s, b.n, xi[d], v[d], dv[d]);
  } else {
    // Barycentric coordinates: lambda_0 = 1 - sum, lambda_d = xi_d (the triangle of a prism
    // in (x, y)). Rows 0..2 of v / dv hold lambda_0 .. lambda_2; the tetrahedron's lambda_3 and
    // the prism's line factor go to f3 / df3.
    const int nl = prism ? 2 : TD;  // simplex dimension
    F lam0 = F(1);
    for (int d = 0; d < nl; ++d) lam0 -= xi[d];
    simplex_factors<F>(b.p, lam0, v[0], dv[0]);
    simplex_factors<F>(b.p, xi[0], v[1], dv[1]);
    if (nl >= 2) simplex_factors<F>(b.p, xi[1], v[2], dv[2]);
  }
  F f3[MAXN], df3[MAXN];
  if (!tensor) {
    if (cell == kTetrahedron) simplex_factors<F>(b.p, xi[2], f3, df3);
    if (prism) lagrange1d<F>(b.s, b.n, xi[2], f3, df3);
  }
#pragma unroll
  for (int g = 0; g < GD; ++g) X[g] = F(0);
  if constexpr (WANT_J)
#pragma unroll
    for (int i = 0; i < TD * GD; ++i) J[i] = F(0);
  for (int k = 0; k < b.k; ++k) {
    const uint8_t* id = b.idx[k];
    F phi, grad[3];
    if (tensor) {
      phi = F(1);
      for (int d = 0; d < TD; ++d) phi *= v[d][id[d]];
      for (int d = 0; d < TD; ++d) {
        F gd = dv[d][id[d]];
        for (int e = 0; e < TD; ++e)
          if (e != d) gd *= v[e][id[e]];
        grad[d] = gd;
      }
    } else if (cell == kTriangle || cell == kTetrahedron || prism) {
      // Simplex part: rows 0..nl with multi-index id[0..nl]; d(phi)/d(xi_d) =
      // d/dlam_{d+1} - d/dlam_0.
      const int nl = prism ? 2 : TD;
      F f[4], df[4];
      for (int r = 0; r <= nl; ++r) {
        if (r < 3) {
          f[r] = v[r][id[r]];
          df[r] = dv[r][id[r]];
        } else {
          f[r] = f3[id[r]];
          df[r] = df3[id[r]];
        }
      }
      F prod = F(1);
      for (int r = 0; r <= nl; ++r) prod *= f[r];
      F dl[4];
      for (int r = 0; r <= nl; ++r) {
        F t = df[r];
        for (int s = 0; s <= nl; ++s)
          if (s != r) t *= f[s];
        dl[r] = t;
      }
      phi = prod;
      for (int d = 0; d < nl; ++d) grad[d] = dl[d + 1] - dl[0];
      if (prism) {
        const F lz = f3[id[3]], dlz = df3[id[3]];
        grad[0] *= lz;
        grad[1] *= lz;
        grad[2] = phi * dlz;
        phi *= lz;
      }
    } else {
      phi = F(0);
      grad[0] = grad[1] = grad[2] = F(0);
    }
#pragma unroll
    for (int g = 0; g < GD; ++g) {
      const F xk = xs[(k * GD + g) * T];
      X[g] = fma(xk, phi, X[g]);
      if constexpr (WANT_J)
#pragma unroll
        for (int d = 0; d < TD; ++d) J[d * GD + g] = fma(xk, grad[d], J[d * GD + g]);
    }
  }
}

// One step of a point: delta = K r, s = |delta|_inf (the largest finite value when a component
// is not finite); a point not yet frozen moves to p + delta clamped to [lo, hi], records s and
// freezes once s <= tol. K(t, g) at g * TD + t (in KT's precision), r and p in P's.
template <typename P, typename KT, int TD, int GD>
__device__ __forceinline__ void newton_update(P* p, const KT* K, const P* r, P& last, bool& frozen, P tol, P lo,
                                              P hi, P big) {
  P delta[TD];
  P s = big;
  bool bad = false;
#pragma unroll
  for (int t = 0; t < TD; ++t) {
    P acc = P(K[t]) * r[0];
#pragma unroll
    for (int g = 1; g < GD; ++g) acc = fma(P(K[g * TD + t]), r[g], acc);
    delta[t] = acc;
    const P m = fabs(acc);
    s = t == 0 ? m : (m > s ? m : s);
    bad = bad || !(m <= big);
  }
  if (bad) s = big;
  if (!frozen) {
#pragma unroll
    for (int d = 0; d < TD; ++d) {
      P qd = p[d] + delta[d];
      qd = qd < lo ? lo : qd;
      qd = qd > hi ? hi : qd;
      p[d] = qd;
    }
    last = s;
    frozen = s <= tol;
  }
}

// The vertex centroid of the reference cell, rounded to f32.
__device__ __forceinline__ void centroid_f32(int cell, float* start) {
  const float third = 1.0f / 3.0f;
  if (cell == kTriangle) start[0] = start[1] = third;
  else if (cell == kTetrahedron) start[0] = start[1] = start[2] = 0.25f;
  else if (cell == kPrism) {
    start[0] = start[1] = third;
    start[2] = 0.5f;
  } else if (cell == kPyramid) {
    start[0] = start[1] = 0.4f;
    start[2] = 0.2f;
  } else start[0] = start[1] = start[2] = 0.5f;
}

template <typename F, int TD, int GD>
__global__ void pull_back_kernel(const __grid_constant__ PullBackArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ BasisData basis;
  // The basis description into shared memory (its size is a few KB).
  {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(a.basis);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&basis);
    for (int i = threadIdx.x; i < (int)(sizeof(BasisData) / 4); i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  using M = Factors<F, TD, GD>;
  constexpr int LJ = TD * GD;
  const int T = a.threads;
  F* xs = reinterpret_cast<F*>(smem) + threadIdx.x;
  const F* nodes = static_cast<const F*>(a.nodes);
  const F* xin = static_cast<const F*>(a.x);
  F* xi_out = static_cast<F*>(a.xi);
  F* step_out = static_cast<F*>(a.step);
  const int nq = a.num_points;
  const int K = basis.k;
  const int tmask = (1 << a.tile_shift) - 1;
  const F big = fmax_finite<F>();
  const F lo = F(-0.1f), hi = F(1.1f);
  const F tol = F(a.tolerance);
  float start[3];
  centroid_f32(basis.cell, start);
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < a.padded;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cell = min(a.first_cell + c, a.last_cell);
    const uint32_t* row = a.dofmap + cell * K;
    for (int k = 0; k < K; ++k) {
      const uint32_t n = min(__ldg(row + k), a.last_node);
#pragma unroll
      for (int g = 0; g < GD; ++g) xs[(k * GD + g) * T] = __ldg(nodes + (int64_t)n * GD + g);
    }
    const int64_t ox = a.x_first_cell + c, oo = a.out_first_cell + c;
    const int64_t tx = ox >> a.tile_shift, to = oo >> a.tile_shift;
    const int lx = (int)(ox & tmask), lo_ = (int)(oo & tmask);
    for (int q = 0; q < nq; ++q) {
      F y[GD];
#pragma unroll
      for (int g = 0; g < GD; ++g)
        y[g] = xin[(((tx * nq + q) * GD + g) << a.tile_shift) + lx] - F(a.origin[g]);
      F p[TD];
#pragma unroll
      for (int d = 0; d < TD; ++d) p[d] = start[d];
      F last = big;
      bool frozen = false;
      for (int it = 0; it < a.max_iterations; ++it) {
        F X[GD], J[LJ], K_[LJ];
        map_at<F, TD, GD>(basis, xs, T, p, X, J);
        M::pinv(J, K_);
        F r[GD];
#pragma unroll
        for (int g = 0; g < GD; ++g) r[g] = y[g] - X[g];
        newton_update<F, F, TD, GD>(p, K_, r, last, frozen, tol, lo, hi, big);
      }
#pragma unroll
      for (int d = 0; d < TD; ++d) xi_out[(((to * nq + q) * TD + d) << a.tile_shift) + lo_] = p[d];
      step_out[((to * nq + q) << a.tile_shift) + lo_] = last;
    }
  }
}

// Mixed precision for f64 meshes: the native iteration in FP32 on coordinates shifted by the
// cell's first node (rounding relative to the cell size, as the split evaluation), then
// `refinements` steps with the residual y - X(xi) in FP64 and the correction K r through the
// FP32 inverse Jacobian at xi: an iteration with an approximate Jacobian, converging linearly
// at a rate of the FP32 rounding of K times the condition of J, so that a few steps reach the
// FP64 tolerance. xi and the step (of the last refinement) are f64; a point whose FP32 phase
// left its cell does not converge in the refinement either.
template <int TD, int GD>
__global__ void pull_back_split_kernel(const __grid_constant__ PullBackArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ BasisData basis;
  {
    const uint32_t* src = reinterpret_cast<const uint32_t*>(a.basis);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&basis);
    for (int i = threadIdx.x; i < (int)(sizeof(BasisData) / 4); i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  using M = Factors<float, TD, GD>;
  constexpr int LJ = TD * GD;
  const int T = a.threads;
  const int K = basis.k;
  // Slots: the f64 shifted coordinates, then their f32 roundings.
  double* xs64 = reinterpret_cast<double*>(smem) + threadIdx.x;
  float* xs32 = reinterpret_cast<float*>(smem + (size_t)K * GD * T * sizeof(double)) + threadIdx.x;
  const double* nodes = static_cast<const double*>(a.nodes);
  const double* xin = static_cast<const double*>(a.x);
  double* xi_out = static_cast<double*>(a.xi);
  double* step_out = static_cast<double*>(a.step);
  const int nq = a.num_points;
  const int tmask = (1 << a.tile_shift) - 1;
  const float big32 = fmax_finite<float>();
  const double big = fmax_finite<double>();
  const float tol32 = 1e-5f;
  const double tol = a.tolerance;
  float start[3];
  centroid_f32(basis.cell, start);
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < a.padded;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cell = min(a.first_cell + c, a.last_cell);
    const uint32_t* row = a.dofmap + cell * K;
    double x0[GD];
    const uint32_t n0 = min(__ldg(row), a.last_node);
#pragma unroll
    for (int g = 0; g < GD; ++g) x0[g] = __ldg(nodes + (int64_t)n0 * GD + g);
    for (int k = 0; k < K; ++k) {
      const uint32_t n = min(__ldg(row + k), a.last_node);
#pragma unroll
      for (int g = 0; g < GD; ++g) {
        const double v = __ldg(nodes + (int64_t)n * GD + g) - x0[g];
        xs64[(k * GD + g) * T] = v;
        xs32[(k * GD + g) * T] = d2f_rn(v);
      }
    }
    const int64_t ox = a.x_first_cell + c, oo = a.out_first_cell + c;
    const int64_t tx = ox >> a.tile_shift, to = oo >> a.tile_shift;
    const int lx = (int)(ox & tmask), lo_ = (int)(oo & tmask);
    for (int q = 0; q < nq; ++q) {
      double y[GD];
      float y32[GD];
#pragma unroll
      for (int g = 0; g < GD; ++g) {
        y[g] = (xin[(((tx * nq + q) * GD + g) << a.tile_shift) + lx] - a.origin[g]) - x0[g];
        y32[g] = d2f_rn(y[g]);
      }
      float p32[TD];
#pragma unroll
      for (int d = 0; d < TD; ++d) p32[d] = start[d];
      float last32 = big32;
      bool frozen32 = false;
      for (int it = 0; it < a.max_iterations; ++it) {
        float X[GD], J[LJ], K_[LJ];
        map_at<float, TD, GD>(basis, xs32, T, p32, X, J);
        M::pinv(J, K_);
        float r[GD];
#pragma unroll
        for (int g = 0; g < GD; ++g) r[g] = y32[g] - X[g];
        newton_update<float, float, TD, GD>(p32, K_, r, last32, frozen32, tol32, -0.1f, 1.1f, big32);
      }
      double p[TD];
#pragma unroll
      for (int d = 0; d < TD; ++d) p[d] = f2d_exact(p32[d]);
      double last = big;
      bool frozen = false;
      for (int it = 0; it < a.refinements; ++it) {
        double X[GD], Jd[1];
        map_at<double, TD, GD, false>(basis, xs64, T, p, X, Jd);
        float pf[TD], X32[GD], J[LJ], K_[LJ];
#pragma unroll
        for (int d = 0; d < TD; ++d) pf[d] = d2f_rn(p[d]);
        map_at<float, TD, GD>(basis, xs32, T, pf, X32, J);
        M::pinv(J, K_);
        double r[GD];
#pragma unroll
        for (int g = 0; g < GD; ++g) r[g] = y[g] - X[g];
        newton_update<double, float, TD, GD>(p, K_, r, last, frozen, tol, double(-0.1f), double(1.1f), big);
      }
#pragma unroll
      for (int d = 0; d < TD; ++d) xi_out[(((to * nq + q) * TD + d) << a.tile_shift) + lo_] = p[d];
      step_out[((to * nq + q) << a.tile_shift) + lo_] = last;
    }
  }
}

}  // namespace tlg

namespace {

tlg_status basis_fail(tlg_status s, const std::string& m) { return tlg::fail(s, m); }

}  // namespace

tlg_status tlg_basis_create(int cell, int degree, int family, tlg_basis** out) {
  if (!out) return basis_fail(TLG_ERR_INVALID_ARGUMENT, "tlg_basis_create: out is NULL");
  *out = nullptr;
  if (!tlg::valid_cell(cell) || cell == tlg::kPoint)
    return basis_fail(TLG_ERR_UNSUPPORTED, "tlg_basis_create: no basis for cell " + std::to_string(cell));
  if (degree < 1 || degree + 1 > tlg::kBasisMaxN)
    return basis_fail(TLG_ERR_UNSUPPORTED, "tlg_basis_create: degree must be 1 .. 15");
  if (cell == tlg::kPyramid && degree > tlg::kPyramidMaxP)
    return basis_fail(TLG_ERR_UNSUPPORTED, "tlg_basis_create: pyramid degrees 1 .. 4");
  try {
    const int td = tlg::tdim(cell);
    const int64_t k = tlg::num_lagrange_nodes(cell, degree);
    if (k > tlg::kBasisMaxK) return basis_fail(TLG_ERR_UNSUPPORTED, "tlg_basis_create: too many nodes");
    const bool tensor = cell == tlg::kInterval || cell == tlg::kQuadrilateral || cell == tlg::kHexahedron;
    const bool simplex = cell == tlg::kTriangle || cell == tlg::kTetrahedron;
    if (!tensor && family != TLG_EQUISPACED)
      return basis_fail(TLG_ERR_UNSUPPORTED, "tlg_basis_create: simplices and prisms have equispaced nodes only");
    std::vector<double> lp = tlg::lagrange_points(cell, degree, family);
    std::vector<double> s1 = tlg::lagrange_points(tlg::kInterval, degree, family);
    std::sort(s1.begin(), s1.end());
    tlg::BasisData h;
    std::memset(&h, 0, sizeof(h));
    h.cell = cell;
    h.p = degree;
    h.k = (int)k;
    h.n = degree + 1;
    for (int i = 0; i < h.n; ++i) h.s[i] = s1[i];
    auto index_1d = [&](double x) {
      for (int i = 0; i < h.n; ++i)
        if (std::fabs(x - s1[i]) < 1e-12) return i;
      throw std::invalid_argument("tlg_basis_create: a node off the 1D lattice");
    };
    auto bary = [&](double x) {
      const double r = x * degree;
      const double m = std::round(r);
      if (std::fabs(r - m) > 1e-9 || m < 0 || m > degree)
        throw std::invalid_argument("tlg_basis_create: a node off the barycentric lattice");
      return (int)m;
    };
    const bool pyramid = cell == tlg::kPyramid;
    for (int64_t kk = 0; kk < k && !pyramid; ++kk) {
      const double* x = &lp[kk * td];
      if (tensor) {
        for (int d = 0; d < td; ++d) h.idx[kk][d] = (uint8_t)index_1d(x[d]);
      } else {
        const int nl = simplex ? td : 2;
        double l0 = 1.0;
        for (int d = 0; d < nl; ++d) l0 -= x[d];
        int sum = h.idx[kk][0] = (uint8_t)bary(l0);
        for (int d = 0; d < nl; ++d) sum += h.idx[kk][d + 1] = (uint8_t)bary(x[d]);
        if (sum != degree) throw std::invalid_argument("tlg_basis_create: barycentric indices");
        if (!simplex) h.idx[kk][3] = (uint8_t)index_1d(x[2]);
      }
    }
    auto b = new tlg_basis();
    b->cell = cell;
    b->degree = degree;
    b->family = family;
    b->td = td;
    b->k = k;
    // Pyramids: the expansion coefficients follow the header.
    const std::vector<double> coef =
        pyramid ? tlg::expansion_coefficients(cell, degree, family) : std::vector<double>();
    static_assert(sizeof(tlg::BasisData) % 16 == 0, "the coefficients start 16-byte aligned");
    cudaError_t e = cudaMalloc(&b->dev, sizeof(tlg::BasisData) + coef.size() * sizeof(double));
    if (e == cudaSuccess && pyramid) h.coef = reinterpret_cast<const double*>(b->dev + sizeof(tlg::BasisData));
    if (e == cudaSuccess) e = cudaMemcpy(b->dev, &h, sizeof(h), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && pyramid)
      e = cudaMemcpy(b->dev + sizeof(tlg::BasisData), coef.data(), coef.size() * sizeof(double),
                     cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      if (b->dev) cudaFree(b->dev);
      delete b;
      return tlg::cuda_fail(e, "tlg_basis_create");
    }
    *out = b;
    return tlg::ok();
  } catch (const std::exception& ex) {
    return basis_fail(TLG_ERR_INVALID_ARGUMENT, ex.what());
  }
}

tlg_status tlg_basis_destroy(tlg_basis* b) {
  if (!b) return tlg::ok();
  cudaError_t e = cudaFree(b->dev);
  delete b;
  if (e != cudaSuccess) return tlg::cuda_fail(e, "tlg_basis_destroy");
  return tlg::ok();
}

tlg_status tlg_pull_back_block(const tlg_basis* basis, const tlg_block* b, const void* x, int64_t x_first_cell,
                               int64_t first_cell, int64_t num_cells, int64_t out_first_cell, int num_points,
                               int tile, double tolerance, int max_iterations, int refinements, void* xi,
                               void* step, void* stream) {
  if (!basis || !b) return basis_fail(TLG_ERR_INVALID_ARGUMENT, "tlg_pull_back_block: NULL argument");
  if (b->dtype != TLG_F32 && b->dtype != TLG_F64)
    return basis_fail(TLG_ERR_INVALID_ARGUMENT, "tlg_pull_back_block: dtype must be 4 or 8");
  if (b->gdim < basis->td || b->gdim > 3)
    return basis_fail(TLG_ERR_INVALID_ARGUMENT, "tlg_pull_back_block: gdim below the cell's dimension");
  int shift = -1;
  for (int s = 0; s <= 4; ++s)
    if (tile == (1 << s)) shift = s;
  if (shift < 0) return basis_fail(TLG_ERR_INVALID_ARGUMENT, "tlg_pull_back_block: tile is not 1, 2, 4, 8 or 16");
  if (first_cell < 0 || num_cells < 0 || first_cell + num_cells > b->num_cells || x_first_cell < 0 ||
      out_first_cell < 0 || x_first_cell % tile || out_first_cell % tile || num_points < 0 || max_iterations < 0 ||
      refinements < 0)
    return basis_fail(TLG_ERR_INVALID_ARGUMENT, "tlg_pull_back_block: bad range, points or iterations");
  if (refinements > 0 && b->dtype != TLG_F64)
    return basis_fail(TLG_ERR_INVALID_ARGUMENT, "tlg_pull_back_block: mixed precision refines f64 meshes");
  if (num_cells == 0 || num_points == 0) return tlg::ok();
  if (!tlg::check_strategy(TLG_FAMILY_PULL_BACK)) return TLG_ERR_INVALID_ARGUMENT;
  if (!x || !xi || !step || !b->nodes || !b->dofmap)
    return basis_fail(TLG_ERR_INVALID_ARGUMENT, "tlg_pull_back_block: NULL points, outputs, nodes or dofmap");
  if (b->num_nodes < 1) return basis_fail(TLG_ERR_LENGTH_MISMATCH, "tlg_pull_back_block: cells but no nodes");
  tlg::PullBackArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nodes = b->nodes;
  a.dofmap = b->dofmap;
  a.basis = reinterpret_cast<const tlg::BasisData*>(basis->dev);
  a.x = x;
  a.xi = xi;
  a.step = step;
  a.first_cell = first_cell;
  a.padded = (num_cells + tile - 1) / tile * tile;
  a.out_first_cell = out_first_cell;
  a.x_first_cell = x_first_cell;
  a.last_cell = b->num_cells - 1;
  for (int g = 0; g < 3; ++g) a.origin[g] = b->origin[g];
  a.tolerance = tolerance > 0 ? tolerance : (b->dtype == TLG_F64 ? 1e-13 : 1e-5);
  a.last_node = (uint32_t)(b->num_nodes - 1);
  a.num_points = num_points;
  a.max_iterations = max_iterations;
  a.tile_shift = shift;
  a.refinements = refinements;
  // Threads per CTA: the node slots of 128 threads, or fewer, within 96 KiB (mixed precision
  // keeps f64 and f32 copies); the basis description adds a static 4 KiB. The dynamic size is
  // always declared, as static and dynamic shared memory together may pass the default 48 KiB.
  const size_t per_thread = (size_t)basis->k * b->gdim * (refinements > 0 ? 12 : (size_t)b->dtype);
  int threads = 128;
  while (threads > 32 && per_thread * threads > (size_t)96 * 1024) threads /= 2;
  const size_t smem = per_thread * threads;
  if (smem > (size_t)200 * 1024)
    return basis_fail(TLG_ERR_ALLOCATION_TOO_LARGE, "tlg_pull_back_block: too many nodes per cell");
  a.threads = threads;
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t need = (a.padded + threads - 1) / threads;
  const int64_t cap = (int64_t)sms * (2048 / threads);
  const unsigned grid = (unsigned)std::max<int64_t>(1, std::min(need, cap));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaSuccess;
#define TLG_PB(F, TD, GD) \
  if (basis->td == TD && b->gdim == GD) { \
    auto kern = tlg::pull_back_kernel<F, TD, GD>; \
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
    if (e == cudaSuccess) { \
      kern<<<grid, threads, smem, s>>>(a); \
      e = cudaGetLastError(); \
    } \
  }
#define TLG_PBS(TD, GD) \
  if (basis->td == TD && b->gdim == GD) { \
    auto kern = tlg::pull_back_split_kernel<TD, GD>; \
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
    if (e == cudaSuccess) { \
      kern<<<grid, threads, smem, s>>>(a); \
      e = cudaGetLastError(); \
    } \
  }
  if (refinements > 0) {
    TLG_PBS(1, 1) TLG_PBS(1, 2) TLG_PBS(1, 3) TLG_PBS(2, 2) TLG_PBS(2, 3) TLG_PBS(3, 3)
  } else if (b->dtype == TLG_F64) {
    TLG_PB(double, 1, 1) TLG_PB(double, 1, 2) TLG_PB(double, 1, 3) TLG_PB(double, 2, 2) TLG_PB(double, 2, 3)
    TLG_PB(double, 3, 3)
  } else {
    TLG_PB(float, 1, 1) TLG_PB(float, 1, 2) TLG_PB(float, 1, 3) TLG_PB(float, 2, 2) TLG_PB(float, 2, 3)
    TLG_PB(float, 3, 3)
  }
#undef TLG_PB
#undef TLG_PBS
  if (e != cudaSuccess) return tlg::cuda_fail(e, "tlg_pull_back_block launch");
  tlg::record_launch(TLG_FAMILY_PULL_BACK, TLG_STRATEGY_LOOPS);
  return tlg::ok();
}
