/*
 * Oracle, test infrastructure only: a plain-C restatement of the reference's host f64
 * evaluation of the geometric factors, used as the checker of the CUDA path and as the timed
 * CPU baseline. Only the tests, __graft_entry__.smoke() and the CPU-baseline leg of bench.py
 * load it; nothing in the product links it.
 *
 * Restated from (paths inside the reference project):
 *   - tetraloma-testing/src/reference.rs:48-73   BlockNodes::of_grid: node coordinates are the
 *     stored L-vector widened to f64 plus the grid's origin, gathered through the dofmap;
 *   - reference.rs:117-150   X and J: sums over the nodes of x(k, g) times the tabulated
 *     value or derivative, J(g, d) at component d * GD + g (column-major GD x TD);
 *   - reference.rs:170-193   det J (TD = GD; first-row cofactor expansion in 3D) or the
 *     pseudo-determinant sqrt(det(J^T J));
 *   - reference.rs:197-235   K = (J^T J)^-1 J^T through G = J^T J and its adjugate, K(t, g) at
 *     g * TD + t;
 *   - reference.rs:306-327   unit normals of codimension-1 blocks, sign flipped where bit 0 of
 *     the cell's flags is set;
 *   - reference.rs:335-354   facet normals K^T n_ref / |K^T n_ref|;
 *   - tetraloma-geometry/src/evector.rs:195-236  the E-vector gather: cells past the block
 *     repeat the last cell, node indices clamp to the last node (bit-exact copy);
 *   - tetraloma-geometry/src/measure.rs:15-41,141-185  per-cell sums of det J * w, then a sum
 *     over the cells finished in f64.
 *
 * Cell-major outputs [cell][point][component], the order of QuadField::to_host_cell_major
 * (tetraloma-geometry/src/field.rs:380-408). Loops are parallel over cells with OpenMP; each
 * cell's arithmetic is sequential and in the reference's order.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>

/* Nodes per cell the oracle accepts (a degree-7 hexahedron has 512). */
#define ORC_MAX_K 512
#endif

#define ORC_OK 0
#define ORC_BAD_ARGS 1

static double detj_of(const double* j, int td, int gd) {
  if (td == gd) {
    if (td == 1) return j[0];
    if (td == 2) return j[0] * j[3] - j[2] * j[1];
    /* m(g, d) = j[d * 3 + g] */
#define M(g, d) j[(d) * 3 + (g)]
    return M(0, 0) * (M(1, 1) * M(2, 2) - M(1, 2) * M(2, 1)) -
           M(0, 1) * (M(1, 0) * M(2, 2) - M(1, 2) * M(2, 0)) +
           M(0, 2) * (M(1, 0) * M(2, 1) - M(1, 1) * M(2, 0));
#undef M
  }
  if (td == 1) {
    double s = 0.0;
    for (int g = 0; g < gd; ++g) s += j[g] * j[g];
    return sqrt(s);
  }
  /* td == 2, gd == 3 */
  double a = 0.0, b = 0.0, c = 0.0;
  for (int g = 0; g < gd; ++g) {
    a += j[g] * j[g];
    b += j[g] * j[gd + g];
    c += j[gd + g] * j[gd + g];
  }
  return sqrt(a * c - b * b);
}

static void pinv_of(const double* j, int td, int gd, double* k) {
  double m[9], ginv[9];
  for (int a = 0; a < td; ++a)
    for (int b = 0; b < td; ++b) {
      double s = 0.0;
      for (int g = 0; g < gd; ++g) s += j[a * gd + g] * j[b * gd + g];
      m[a * td + b] = s;
    }
  if (td == 1) {
    ginv[0] = 1.0 / m[0];
  } else if (td == 2) {
    double inv = 1.0 / (m[0] * m[3] - m[1] * m[1]);
    ginv[0] = m[3] * inv;
    ginv[1] = -m[1] * inv;
    ginv[2] = -m[1] * inv;
    ginv[3] = m[0] * inv;
  } else {
#define COF(r0, r1, c0, c1) (m[(r0) * 3 + (c0)] * m[(r1) * 3 + (c1)] - m[(r0) * 3 + (c1)] * m[(r1) * 3 + (c0)])
    double adj[9] = {COF(1, 2, 1, 2), -COF(0, 2, 1, 2), COF(0, 1, 1, 2),
                     -COF(1, 2, 0, 2), COF(0, 2, 0, 2), -COF(0, 1, 0, 2),
                     COF(1, 2, 0, 1), -COF(0, 2, 0, 1), COF(0, 1, 0, 1)};
#undef COF
    double det = m[0] * adj[0] + m[1] * adj[3] + m[2] * adj[6];
    for (int i = 0; i < 9; ++i) ginv[i] = adj[i] / det;
  }
  for (int g = 0; g < gd; ++g)
    for (int t = 0; t < td; ++t) {
      double s = 0.0;
      for (int u = 0; u < td; ++u) s += ginv[t * td + u] * j[u * gd + g];
      k[g * td + t] = s;
    }
}

/*
 * One block. nodes [n][gd] are absolute f64 coordinates; tab is [1 + td][nq][k] (row 0 the
 * values, rows 1 + d the derivatives), ref_normals [nq][td]. Any output may be NULL.
 */
int orc_eval(int td, int gd, int k, int nq, int64_t ncells, const double* nodes, int64_t nnodes,
             const uint32_t* dofmap, const double* tab, const uint32_t* flags,
             const double* ref_normals, double* x, double* jac, double* detj, double* kinv,
             double* normals, double* facet_normals, int nthreads) {
  if (td < 1 || td > 3 || gd < td || gd > 3 || k < 1 || k > ORC_MAX_K || nq < 0 || ncells < 0 || nnodes < 1)
    return ORC_BAD_ARGS;
  if (normals && td + 1 != gd) return ORC_BAD_ARGS;
  if (facet_normals && (td != gd || !ref_normals)) return ORC_BAD_ARGS;
  const int need_j = jac || detj || kinv || normals || facet_normals;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(static)
#endif
  for (int64_t c = 0; c < ncells; ++c) {
    double xc[ORC_MAX_K * 3];
    double jq[9], kq[9];
    const double* cx = xc;
    for (int i = 0; i < k; ++i) {
      uint32_t n = dofmap[c * k + i];
      if ((int64_t)n >= nnodes) n = (uint32_t)(nnodes - 1);
      for (int g = 0; g < gd; ++g) xc[i * gd + g] = nodes[(int64_t)n * gd + g];
    }
    for (int q = 0; q < nq; ++q) {
      const int64_t cq = c * nq + q;
      if (x) {
        for (int g = 0; g < gd; ++g) {
          double s = 0.0;
          for (int i = 0; i < k; ++i) s += cx[i * gd + g] * tab[(int64_t)q * k + i];
          x[cq * gd + g] = s;
        }
      }
      if (!need_j) continue;
      for (int d = 0; d < td; ++d)
        for (int g = 0; g < gd; ++g) {
          double s = 0.0;
          for (int i = 0; i < k; ++i)
            s += cx[i * gd + g] * tab[((int64_t)(1 + d) * nq + q) * k + i];
          jq[d * gd + g] = s;
        }
      if (jac)
        for (int i = 0; i < td * gd; ++i) jac[cq * td * gd + i] = jq[i];
      if (detj) detj[cq] = detj_of(jq, td, gd);
      if (kinv || facet_normals) pinv_of(jq, td, gd, kq);
      if (kinv)
        for (int i = 0; i < td * gd; ++i) kinv[cq * td * gd + i] = kq[i];
      if (normals) {
        double v[3];
        if (gd == 2) {
          v[0] = jq[1];
          v[1] = -jq[0];
        } else {
          v[0] = jq[1] * jq[5] - jq[2] * jq[4];
          v[1] = jq[2] * jq[3] - jq[0] * jq[5];
          v[2] = jq[0] * jq[4] - jq[1] * jq[3];
        }
        double s = (flags && (flags[c] & 1u)) ? -1.0 : 1.0;
        double len = 0.0;
        for (int g = 0; g < gd; ++g) len += v[g] * v[g];
        len = sqrt(len);
        for (int g = 0; g < gd; ++g) normals[cq * gd + g] = s * v[g] / len;
      }
      if (facet_normals) {
        double m[3], len = 0.0;
        for (int g = 0; g < gd; ++g) {
          double s = 0.0;
          for (int t = 0; t < td; ++t) s += kq[g * td + t] * ref_normals[q * td + t];
          m[g] = s;
          len += s * s;
        }
        len = sqrt(len);
        for (int g = 0; g < gd; ++g) facet_normals[cq * gd + g] = m[g] / len;
      }
    }
  }
  return ORC_OK;
}

/*
 * The E-vector chunk of cells [first_cell, first_cell + padded) of a block: out[(k * gd + g) *
 * stride + c] = nodes[min(dofmap[min(first_cell + c, num_cells - 1) * K + k], last_node) * gd
 * + g], copied byte for byte (elem_size 4 or 8).
 */
int orc_evector(const void* nodes, int64_t nnodes, int elem_size, const uint32_t* dofmap,
                int64_t num_cells, int k, int gd, int64_t first_cell, int64_t padded,
                int64_t stride, void* out) {
  if ((elem_size != 4 && elem_size != 8) || num_cells < 1 || padded > stride) return ORC_BAD_ARGS;
  const uint32_t last_node = nnodes > 0 ? (uint32_t)(nnodes - 1) : 0;
  const char* src = (const char*)nodes;
  char* dst = (char*)out;
  for (int64_t c = 0; c < padded; ++c) {
    int64_t cell = first_cell + c;
    if (cell > num_cells - 1) cell = num_cells - 1;
    for (int i = 0; i < k; ++i) {
      uint32_t n = dofmap[cell * k + i];
      if (n > last_node) n = last_node;
      for (int g = 0; g < gd; ++g)
        memcpy(dst + (((int64_t)i * gd + g) * stride + c) * elem_size,
               src + ((int64_t)n * gd + g) * elem_size, (size_t)elem_size);
    }
  }
  return ORC_OK;
}

/* Per-cell sums of det J * w over the points, then the f64 total. */
double orc_measure(const double* detj, const double* weights, int64_t ncells, int nq) {
  double total = 0.0;
  for (int64_t c = 0; c < ncells; ++c) {
    double s = 0.0;
    for (int q = 0; q < nq; ++q) s += detj[c * nq + q] * weights[q];
    total += s;
  }
  return total;
}

/*
 * Adjoint restated in f64 (no reference counterpart: the reference has no adjoint): for
 * codimension 0 (td == gd), the node cotangents of L = sum_c sum_q [xbar . x + dbar det J +
 * Kbar : K], accumulated cell by cell into grad [node][gd] (sequential, deterministic). K by the
 * adjugate of J over det J. xbar [cell][q][gd], dbar [cell][q], kbar [cell][q][td * gd] (K(t, g)
 * at g * td + t) may be NULL.
 */
int orc_vjp(int d, int k, int nq, int64_t ncells, const double* nodes, int64_t nnodes,
            const uint32_t* dofmap, const double* tab, const double* xbar, const double* dbar,
            const double* kbar, double* grad) {
  if (d < 1 || d > 3 || k < 1 || k > ORC_MAX_K || nq < 0 || ncells < 0 || nnodes < 1) return ORC_BAD_ARGS;
  for (int64_t i = 0; i < nnodes * d; ++i) grad[i] = 0.0;
  double xc[ORC_MAX_K * 3], gl[ORC_MAX_K * 3];
  for (int64_t c = 0; c < ncells; ++c) {
    uint32_t idx[ORC_MAX_K];
    for (int i = 0; i < k; ++i) {
      uint32_t n = dofmap[c * k + i];
      if ((int64_t)n >= nnodes) n = (uint32_t)(nnodes - 1);
      idx[i] = n;
      for (int g = 0; g < d; ++g) xc[i * d + g] = nodes[(int64_t)n * d + g];
    }
    for (int i = 0; i < k * d; ++i) gl[i] = 0.0;
    for (int q = 0; q < nq; ++q) {
      const int64_t cq = c * nq + q;
      double j[9], kk[9], det;
      for (int dd = 0; dd < d; ++dd)
        for (int g = 0; g < d; ++g) {
          double s = 0.0;
          for (int i = 0; i < k; ++i) s += xc[i * d + g] * tab[((int64_t)(1 + dd) * nq + q) * k + i];
          j[dd * d + g] = s;
        }
      /* M(g, dd) = J(g, dd) = j[dd * d + g]; inverse by adjugate. */
      if (d == 1) {
        det = j[0];
        kk[0] = 1.0 / det;
      } else if (d == 2) {
        det = j[0] * j[3] - j[2] * j[1];
        kk[0] = j[3] / det;
        kk[1] = -j[1] / det;
        kk[2] = -j[2] / det;
        kk[3] = j[0] / det;
      } else {
        det = detj_of(j, 3, 3);
#define J_(g, dd) j[(dd) * 3 + (g)]
        /* K(t, g) = cof(J)(g, t) / det, stored at g * 3 + t */
        for (int g = 0; g < 3; ++g)
          for (int t = 0; t < 3; ++t) {
            const int r0 = (g + 1) % 3, r1 = (g + 2) % 3, c0 = (t + 1) % 3, c1 = (t + 2) % 3;
            const double cof = J_(r0, c0) * J_(r1, c1) - J_(r0, c1) * J_(r1, c0);
            kk[g * 3 + t] = cof / det;
          }
#undef J_
      }
      double jb[9];
      for (int i = 0; i < d * d; ++i) jb[i] = 0.0;
      /* Jbar(g, dd) = dbar det K(dd, g) - sum_{t,h} K(t, g) Kbar(t, h) K(dd, h) */
      for (int g = 0; g < d; ++g)
        for (int dd = 0; dd < d; ++dd) {
          double v = dbar ? dbar[cq] * det * kk[g * d + dd] : 0.0;
          if (kbar)
            for (int t = 0; t < d; ++t)
              for (int h = 0; h < d; ++h)
                v -= kk[g * d + t] * kbar[cq * d * d + h * d + t] * kk[h * d + dd];
          jb[dd * d + g] = v;
        }
      for (int i = 0; i < k; ++i)
        for (int g = 0; g < d; ++g) {
          double v = xbar ? tab[(int64_t)q * k + i] * xbar[cq * d + g] : 0.0;
          for (int dd = 0; dd < d; ++dd) v += jb[dd * d + g] * tab[((int64_t)(1 + dd) * nq + q) * k + i];
          gl[i * d + g] += v;
        }
    }
    for (int i = 0; i < k; ++i)
      for (int g = 0; g < d; ++g) grad[(int64_t)idx[i] * d + g] += gl[i * d + g];
  }
  return ORC_OK;
}

/*
 * Adjoint of a block of any codimension, restated in f64: the node cotangents of
 * L = sum_c sum_q [xbar . x + dbar a + Kbar : K + nbar . n] with a = det J (codimension 0) or the
 * area element sqrt(det(J^T J)), K the (pseudo-)inverse and n the unit normal of codimension-1
 * blocks (sign flipped where bit 0 of the cell's flag is set; flags may be NULL). Codimension 0
 * without normals is orc_vjp. For td < gd, with G = J^T J and P = I - J K:
 *   dL/dJ = dbar a K^T - K^T Kbar K^T + P Kbar^T G^-1 + (normal term),
 * the normal term from n = s v / |v|, v = J0 x J1 (gd 3) or (J0_y, -J0_x) (gd 2): with
 * w = s (nbar - (nbar . v^) v^) / |v|, dL/dJ0 += J1 x w, dL/dJ1 += w x J0 (gd 3), or
 * dL/dJ0 += (-w_y, w_x) (gd 2). nbar [cell][q][gd] may be NULL.
 */
int orc_vjp2(int td, int gd, int k, int nq, int64_t ncells, const double* nodes, int64_t nnodes,
             const uint32_t* dofmap, const double* tab, const uint32_t* flags, int64_t nflags,
             const double* xbar, const double* dbar, const double* kbar, const double* nbar, double* grad) {
  if (td < 1 || gd < td || gd > 3 || k < 1 || k > ORC_MAX_K || nq < 0 || ncells < 0 || nnodes < 1) return ORC_BAD_ARGS;
  if (nbar && td + 1 != gd) return ORC_BAD_ARGS;
  if (td == gd) return orc_vjp(td, k, nq, ncells, nodes, nnodes, dofmap, tab, xbar, dbar, kbar, grad);
  for (int64_t i = 0; i < nnodes * gd; ++i) grad[i] = 0.0;
  double xc[ORC_MAX_K * 3], gl[ORC_MAX_K * 3];
  for (int64_t c = 0; c < ncells; ++c) {
    uint32_t idx[ORC_MAX_K];
    for (int i = 0; i < k; ++i) {
      uint32_t n = dofmap[c * k + i];
      if ((int64_t)n >= nnodes) n = (uint32_t)(nnodes - 1);
      idx[i] = n;
      for (int g = 0; g < gd; ++g) xc[i * gd + g] = nodes[(int64_t)n * gd + g];
    }
    const double sgn = (flags && c < nflags && (flags[c] & 1u)) ? -1.0 : 1.0;
    for (int i = 0; i < k * gd; ++i) gl[i] = 0.0;
    for (int q = 0; q < nq; ++q) {
      const int64_t cq = c * nq + q;
      double j[6], kk[6], gm[4], gi[4];
      for (int dd = 0; dd < td; ++dd)
        for (int g = 0; g < gd; ++g) {
          double s = 0.0;
          for (int i = 0; i < k; ++i) s += xc[i * gd + g] * tab[((int64_t)(1 + dd) * nq + q) * k + i];
          j[dd * gd + g] = s;
        }
#define J_(g, dd) j[(dd) * gd + (g)]
#define K_(t, g) kk[(g) * td + (t)]
      for (int a = 0; a < td; ++a)
        for (int b = 0; b < td; ++b) {
          double s = 0.0;
          for (int g = 0; g < gd; ++g) s += J_(g, a) * J_(g, b);
          gm[a * td + b] = s;
        }
      if (td == 1) {
        gi[0] = 1.0 / gm[0];
      } else {
        const double det = gm[0] * gm[3] - gm[1] * gm[2];
        gi[0] = gm[3] / det;
        gi[1] = -gm[1] / det;
        gi[2] = -gm[2] / det;
        gi[3] = gm[0] / det;
      }
      for (int t = 0; t < td; ++t)
        for (int g = 0; g < gd; ++g) {
          double s = 0.0;
          for (int u = 0; u < td; ++u) s += gi[t * td + u] * J_(g, u);
          K_(t, g) = s;
        }
      const double area = detj_of(j, td, gd);
      double jb[6] = {0, 0, 0, 0, 0, 0};
#define JB(g, dd) jb[(dd) * gd + (g)]
      if (dbar)
        for (int g = 0; g < gd; ++g)
          for (int dd = 0; dd < td; ++dd) JB(g, dd) += dbar[cq] * area * K_(dd, g);
      if (kbar) {
        const double* kb = kbar + cq * td * gd;  /* Kbar(t, g) at g * td + t */
        double pm[9];
        for (int g = 0; g < gd; ++g)
          for (int h = 0; h < gd; ++h) {
            double s = g == h ? 1.0 : 0.0;
            for (int t = 0; t < td; ++t) s -= J_(g, t) * K_(t, h);
            pm[g * gd + h] = s;
          }
        for (int g = 0; g < gd; ++g)
          for (int dd = 0; dd < td; ++dd) {
            double v = 0.0;
            for (int t = 0; t < td; ++t)
              for (int h = 0; h < gd; ++h) v -= K_(t, g) * kb[h * td + t] * K_(dd, h);
            for (int h = 0; h < gd; ++h)
              for (int t = 0; t < td; ++t) v += pm[g * gd + h] * kb[h * td + t] * gi[t * td + dd];
            JB(g, dd) += v;
          }
      }
      if (nbar) {
        double v[3], w[3], len = 0.0, dot = 0.0;
        if (gd == 2) {
          v[0] = J_(1, 0);
          v[1] = -J_(0, 0);
        } else {
          v[0] = J_(1, 0) * J_(2, 1) - J_(2, 0) * J_(1, 1);
          v[1] = J_(2, 0) * J_(0, 1) - J_(0, 0) * J_(2, 1);
          v[2] = J_(0, 0) * J_(1, 1) - J_(1, 0) * J_(0, 1);
        }
        for (int g = 0; g < gd; ++g) len += v[g] * v[g];
        len = sqrt(len);
        const double* nb = nbar + cq * gd;
        for (int g = 0; g < gd; ++g) dot += nb[g] * v[g] / len;
        for (int g = 0; g < gd; ++g) w[g] = sgn * (nb[g] - dot * v[g] / len) / len;
        if (gd == 2) {
          JB(0, 0) += -w[1];
          JB(1, 0) += w[0];
        } else {
          /* J1 x w into column 0, w x J0 into column 1 */
          JB(0, 0) += J_(1, 1) * w[2] - J_(2, 1) * w[1];
          JB(1, 0) += J_(2, 1) * w[0] - J_(0, 1) * w[2];
          JB(2, 0) += J_(0, 1) * w[1] - J_(1, 1) * w[0];
          JB(0, 1) += w[1] * J_(2, 0) - w[2] * J_(1, 0);
          JB(1, 1) += w[2] * J_(0, 0) - w[0] * J_(2, 0);
          JB(2, 1) += w[0] * J_(1, 0) - w[1] * J_(0, 0);
        }
      }
      for (int i = 0; i < k; ++i)
        for (int g = 0; g < gd; ++g) {
          double v = xbar ? tab[(int64_t)q * k + i] * xbar[cq * gd + g] : 0.0;
          for (int dd = 0; dd < td; ++dd) v += JB(g, dd) * tab[((int64_t)(1 + dd) * nq + q) * k + i];
          gl[i * gd + g] += v;
        }
#undef JB
#undef K_
#undef J_
    }
    for (int i = 0; i < k; ++i)
      for (int g = 0; g < gd; ++g) grad[(int64_t)idx[i] * gd + g] += gl[i * gd + g];
  }
  return ORC_OK;
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
