// Host reference-cell tables (f64) for the device tabulation.
//
// Restates, in the product's own code (paths inside the reference project):
//  - the reference cells and the lexicographic sub-entity numbering of
//    tetraloma-refcell/src/cell.rs:23-190 (DefElement conventions);
//  - the Lagrange node order of tetraloma-refcell/src/lagrange.rs:163-266: vertices, edges,
//    faces, interior, each entity's nodes along its own vertex list;
//  - the collapsed Gauss rules of tetraloma-refcell/src/quadrature.rs:77-159, first direction
//    fastest, with Gauss-Jacobi nodes by Newton's method on the Jacobi polynomial with
//    deflation of the roots found so far (tetraloma-refcell/src/jacobi.rs);
//  - the Lagrange basis (tetraloma-refcell/src/tabulation.rs:1-5): the reference expands it in
//    an orthonormal set; here the expansion set is orthogonal but not normalised: products of
//    shifted Legendre polynomials on intervals, quadrilaterals and hexahedra, Dubiner's
//    collapsed-coordinate polynomials on triangles and tetrahedra (and triangle x Legendre on
//    prisms), and the generalised Vandermonde matrix is inverted by LU with partial pivoting.
//    Both span the same space, so the Lagrange functions agree to rounding; orthogonality keeps
//    the Vandermonde matrix well conditioned at high degree.
//  - pyramids: the space of tetraloma-refcell/src/polynomials/pyramid.rs:1-17 (rational:
//    x^a y^b z^c / (1 - z)^min(a,b), a + c <= p, b + c <= p), expanded in the orthogonal
//    rationomials Q_i(2x - s, s) Q_j(2y - s, s) / s^min(i,j) * P_k^(2 max(i,j) + 2, 0)(2z - 1),
//    s = 1 - z, max(i, j) + k <= p, with Q_i the scaled Legendre polynomials (not normalised).
//    At the apex (s = 0) the functions with min(i, j) >= 1 are 0 with a zero gradient, the limit
//    along the pyramid's axis, as the reference returns there.
#include "refcell.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <stdexcept>

namespace tlg {

namespace {

const double kPi = 3.14159265358979323846;

struct CellTables {
  int td;
  std::vector<std::vector<double>> verts;
  std::vector<std::vector<int>> edges, faces;
};

std::vector<std::vector<int>> sorted(std::vector<std::vector<int>> v) {
  for (auto& e : v) std::sort(e.begin(), e.end());
  std::sort(v.begin(), v.end());
  return v;
}

const CellTables& tables(int cell) {
  static const CellTables t[8] = {
      {0, {{}}, {}, {}},
      {1, {{0.0}, {1.0}}, {{0, 1}}, {}},
      {2, {{0, 0}, {1, 0}, {0, 1}}, sorted({{0, 1}, {1, 2}, {0, 2}}), sorted({{0, 1, 2}})},
      {2, {{0, 0}, {1, 0}, {0, 1}, {1, 1}}, sorted({{0, 1}, {2, 3}, {0, 2}, {1, 3}}),
       sorted({{0, 1, 2, 3}})},
      {3, {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}},
       sorted({{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}}),
       sorted({{1, 2, 3}, {0, 2, 3}, {0, 1, 3}, {0, 1, 2}})},
      {3,
       {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0}, {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}},
       // Edges join vertices differing in one coordinate bit; faces fix one bit.
       sorted({{0, 1}, {2, 3}, {4, 5}, {6, 7}, {0, 2}, {1, 3}, {4, 6}, {5, 7}, {0, 4}, {1, 5},
               {2, 6}, {3, 7}}),
       sorted({{0, 2, 4, 6}, {1, 3, 5, 7}, {0, 1, 4, 5}, {2, 3, 6, 7}, {0, 1, 2, 3}, {4, 5, 6, 7}})},
      {3, {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {0, 1, 1}},
       sorted({{0, 1}, {1, 2}, {0, 2}, {3, 4}, {4, 5}, {3, 5}, {0, 3}, {1, 4}, {2, 5}}),
       sorted({{0, 1, 2}, {3, 4, 5}, {0, 1, 3, 4}, {1, 2, 4, 5}, {0, 2, 3, 5}})},
      {3, {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {1, 1, 0}, {0, 0, 1}},
       sorted({{0, 1}, {0, 2}, {1, 3}, {2, 3}, {0, 4}, {1, 4}, {2, 4}, {3, 4}}),
       sorted({{0, 1, 2, 3}, {0, 1, 4}, {0, 2, 4}, {1, 3, 4}, {2, 3, 4}})},
  };
  if (!valid_cell(cell)) throw std::invalid_argument("unknown cell type " + std::to_string(cell));
  return t[cell];
}

// Jacobi polynomial P_n^(a, b)(x) on [-1, 1] and its derivative, by the three-term recurrence.
void jacobi(int n, double a, double b, double x, double& p, double& dp) {
  if (n == 0) {
    p = 1.0;
    dp = 0.0;
    return;
  }
  double p0 = 1.0, dp0 = 0.0;
  double p1 = 0.5 * (a - b) + 0.5 * (a + b + 2.0) * x, dp1 = 0.5 * (a + b + 2.0);
  for (int k = 2; k <= n; ++k) {
    const double s = 2.0 * k + a + b;
    const double c1 = 2.0 * k * (k + a + b) * (s - 2.0);
    const double c2 = (s - 1.0) * (a * a - b * b);
    const double c3 = (s - 1.0) * s * (s - 2.0);
    const double c4 = 2.0 * (k + a - 1.0) * (k + b - 1.0) * s;
    const double p2 = ((c2 + c3 * x) * p1 - c4 * p0) / c1;
    const double dp2 = ((c2 + c3 * x) * dp1 + c3 * p1 - c4 * dp0) / c1;
    p0 = p1;
    dp0 = dp1;
    p1 = p2;
    dp1 = dp2;
  }
  p = p1;
  dp = dp1;
}

// Roots of P_m^(a, b) on (-1, 1), ascending, by Newton's method with deflation.
std::vector<double> jacobi_roots(int m, double a, double b) {
  std::vector<double> r;
  r.reserve(m);
  for (int i = 0; i < m; ++i) {
    double x = -std::cos(kPi * (2.0 * i + 1.0) / (2.0 * m));
    if (!r.empty()) x = 0.5 * (x + r.back());
    bool done = false;
    for (int it = 0; it < 200 && !done; ++it) {
      double p, dp;
      jacobi(m, a, b, x, p, dp);
      double defl = 0.0;
      for (double y : r) defl += 1.0 / (x - y);
      const double dx = p / (dp - defl * p);
      x -= dx;
      done = std::fabs(dx) <= 4.0 * 2.220446049250313e-16 * std::max(1.0, std::fabs(x));
    }
    if (!done) throw std::domain_error("Jacobi root iteration did not converge");
    r.push_back(x);
  }
  return r;
}

// Shifted Legendre L_i(x) = P_i(2x - 1), i = 0..n, and derivatives.
void legendre01(int n, double x, double* val, double* der) {
  const double t = 2.0 * x - 1.0;
  val[0] = 1.0;
  der[0] = 0.0;
  if (n >= 1) {
    val[1] = t;
    der[1] = 1.0;
  }
  for (int i = 1; i < n; ++i) {
    val[i + 1] = ((2.0 * i + 1.0) * t * val[i] - i * val[i - 1]) / (i + 1.0);
    der[i + 1] = der[i - 1] + (2.0 * i + 1.0) * val[i];
  }
  for (int i = 0; i <= n; ++i) der[i] *= 2.0;
}

// Scaled Jacobi polynomials R_n = P_n^(alpha,0)(f / g) g^n, n = 0..m, with gradients dr[n * td + d]:
// the three-term recurrence of P_n^(alpha,0) multiplied through by g^n, so that nothing is
// divided by g (which vanishes at the collapsed vertex). With g = 1 these are the Jacobi
// polynomials of f.
//   R_0 = 1,  R_1 = ((alpha + 2) f + alpha g) / 2,
//   R_n = (A_n f + B_n g) R_{n-1} - C_n g^2 R_{n-2}, with D = 2n (n + alpha) (2n + alpha - 2),
//   A_n = (2n + alpha - 1)(2n + alpha)(2n + alpha - 2) / D, B_n = (2n + alpha - 1) alpha^2 / D,
//   C_n = 2 (n + alpha - 1)(n - 1)(2n + alpha) / D.
void scaled_jacobi(int m, double alpha, double f, const double* df, double g, const double* dg, int td,
                   double* r, double* dr) {
  r[0] = 1.0;
  for (int d = 0; d < td; ++d) dr[d] = 0.0;
  if (m < 1) return;
  r[1] = 0.5 * ((alpha + 2.0) * f + alpha * g);
  for (int d = 0; d < td; ++d) dr[td + d] = 0.5 * ((alpha + 2.0) * df[d] + alpha * dg[d]);
  for (int n = 2; n <= m; ++n) {
    const double D = 2.0 * n * (n + alpha) * (2.0 * n + alpha - 2.0);
    const double A = (2.0 * n + alpha - 1.0) * (2.0 * n + alpha) * (2.0 * n + alpha - 2.0) / D;
    const double B = (2.0 * n + alpha - 1.0) * alpha * alpha / D;
    const double C = 2.0 * (n + alpha - 1.0) * (n - 1.0) * (2.0 * n + alpha) / D;
    const double lin = A * f + B * g;
    r[n] = lin * r[n - 1] - C * g * g * r[n - 2];
    for (int d = 0; d < td; ++d)
      dr[n * td + d] = (A * df[d] + B * dg[d]) * r[n - 1] + lin * dr[(n - 1) * td + d] -
                       C * (2.0 * g * dg[d] * r[n - 2] + g * g * dr[(n - 2) * td + d]);
  }
}

// Dubiner's orthogonal polynomials at one point of the reference triangle (td = 2), tetrahedron
// (td = 3) or prism (triangle x Legendre, td = 3), for the exponent triples of `sp`:
//   triangle:    Q_a(x, y) T_ab(y),        Q_a = P_a(f/g) g^a, f = 2x + y - 1, g = 1 - y,
//                                          T_ab = P_b^(2a+1,0)(2y - 1);
//   tetrahedron: Q_a(x, y, z) R_ab(y, z) S_abc(z), f = 2x + y + z - 1, g = 1 - y - z;
//                R_ab = P_b^(2a+1,0)(f2/g2) g2^b, f2 = 2y + z - 1, g2 = 1 - z;
//                S_abc = P_c^(2a+2b+2,0)(2z - 1);
//   prism:       Q_a(x, y) T_ab(y) L_c(z), L_c = P_c(2z - 1).
void dubiner_point(int cell, int p, const double* x, const std::vector<std::array<int, 3>>& sp, double* val,
                   double* grad /* [j][td] */) {
  const int td = cell == kTriangle ? 2 : 3;
  const bool tet = cell == kTetrahedron;
  const double X = x[0], Y = x[1], Z = td == 3 ? x[2] : 0.0;
  const double zero[3] = {0.0, 0.0, 0.0};
  // Q_a: the scaled Legendre polynomials of the first collapsed direction.
  const double f1 = 2.0 * X + Y + (tet ? Z : 0.0) - 1.0, g1 = 1.0 - Y - (tet ? Z : 0.0);
  const double df1[3] = {2.0, 1.0, tet ? 1.0 : 0.0}, dg1[3] = {0.0, -1.0, tet ? -1.0 : 0.0};
  std::vector<double> q(p + 1), dq((p + 1) * 3);
  scaled_jacobi(p, 0.0, f1, df1, g1, dg1, 3, q.data(), dq.data());
  // Line factor of the prism.
  std::vector<double> l(p + 1), dl((p + 1) * 3);
  if (cell == kPrism) {
    const double dfz[3] = {0.0, 0.0, 2.0};
    scaled_jacobi(p, 0.0, 2.0 * Z - 1.0, dfz, 1.0, zero, 3, l.data(), dl.data());
  }
  std::vector<double> r(p + 1), dr((p + 1) * 3), t(p + 1), dt((p + 1) * 3);
  for (size_t j = 0; j < sp.size(); ++j) {
    const int a = sp[j][0], b = sp[j][1], c = sp[j][2];
    double v = q[a], gv[3] = {dq[a * 3], dq[a * 3 + 1], dq[a * 3 + 2]};
    auto times = [&](double w, const double* dw) {
      for (int d = 0; d < 3; ++d) gv[d] = gv[d] * w + v * dw[d];
      v *= w;
    };
    if (tet) {
      const double f2 = 2.0 * Y + Z - 1.0, g2 = 1.0 - Z;
      const double df2[3] = {0.0, 2.0, 1.0}, dg2[3] = {0.0, 0.0, -1.0};
      scaled_jacobi(b, 2.0 * a + 1.0, f2, df2, g2, dg2, 3, r.data(), dr.data());
      times(r[b], &dr[b * 3]);
      const double dfz[3] = {0.0, 0.0, 2.0};
      scaled_jacobi(c, 2.0 * a + 2.0 * b + 2.0, 2.0 * Z - 1.0, dfz, 1.0, zero, 3, t.data(), dt.data());
      times(t[c], &dt[c * 3]);
    } else {
      const double dfy[3] = {0.0, 2.0, 0.0};
      scaled_jacobi(b, 2.0 * a + 1.0, 2.0 * Y - 1.0, dfy, 1.0, zero, 3, t.data(), dt.data());
      times(t[b], &dt[b * 3]);
      if (cell == kPrism) times(l[c], &dl[c * 3]);
    }
    val[j] = v;
    for (int d = 0; d < td; ++d) grad[j * td + d] = gv[d];
  }
}

// The pyramid's orthogonal rationomials (i, j, k) of `sp` at one point, values and gradients.
void pyramid_point(int p, const double* x, const std::vector<std::array<int, 3>>& sp, double* val,
                   double* grad /* [j][3] */) {
  const double s = 1.0 - x[2];
  const double zero[3] = {0.0, 0.0, 0.0};
  // Q_i(2x - s, s) and Q_j(2y - s, s): d(2x - s) = (2, 0, 1), d(2y - s) = (0, 2, 1), ds = (0, 0, -1).
  const double dfx[3] = {2.0, 0.0, 1.0}, dfy[3] = {0.0, 2.0, 1.0}, ds[3] = {0.0, 0.0, -1.0};
  std::vector<double> qx(p + 1), dqx((p + 1) * 3), qy(p + 1), dqy((p + 1) * 3);
  scaled_jacobi(p, 0.0, 2.0 * x[0] - s, dfx, s, ds, 3, qx.data(), dqx.data());
  scaled_jacobi(p, 0.0, 2.0 * x[1] - s, dfy, s, ds, 3, qy.data(), dqy.data());
  std::vector<double> t(p + 1), dt((p + 1) * 3);
  const double dfz[3] = {0.0, 0.0, 2.0};
  for (size_t m = 0; m < sp.size(); ++m) {
    const int i = sp[m][0], j = sp[m][1], k = sp[m][2];
    const int n = std::min(i, j);
    double f = 0.0, gf[3] = {0.0, 0.0, 0.0};
    if (n == 0 || s != 0.0) {
      const double r = n ? std::pow(s, -n) : 1.0;
      const double rz = n ? n * r / s : 0.0;  // d(s^-n)/dz
      f = qx[i] * qy[j] * r;
      for (int d = 0; d < 3; ++d) gf[d] = (dqx[i * 3 + d] * qy[j] + qx[i] * dqy[j * 3 + d]) * r;
      gf[2] += qx[i] * qy[j] * rz;
    }
    scaled_jacobi(k, 2.0 * std::max(i, j) + 2.0, 2.0 * x[2] - 1.0, dfz, 1.0, zero, 3, t.data(), dt.data());
    val[m] = f * t[k];
    for (int d = 0; d < 3; ++d) grad[m * 3 + d] = gf[d] * t[k] + f * dt[k * 3 + d];
  }
}

// Exponent triples of the expansion set of (cell, p); on pyramids the (i, j, k) above.
std::vector<std::array<int, 3>> space(int cell, int p) {
  std::vector<std::array<int, 3>> s;
  if (cell == kPyramid) {
    for (int i = 0; i <= p; ++i)
      for (int j = 0; j <= p; ++j)
        for (int k = 0; k + std::max(i, j) <= p; ++k) s.push_back({i, j, k});
    return s;
  }
  for (int c = 0; c <= p; ++c)
    for (int b = 0; b <= p; ++b)
      for (int a = 0; a <= p; ++a) {
        bool keep = false;
        switch (cell) {
          case kInterval: keep = b == 0 && c == 0; break;
          case kTriangle: keep = c == 0 && a + b <= p; break;
          case kQuadrilateral: keep = c == 0; break;
          case kTetrahedron: keep = a + b + c <= p; break;
          case kHexahedron: keep = true; break;
          case kPrism: keep = a + b <= p; break;
          default: throw std::domain_error("no polynomial space for this cell in this build");
        }
        if (keep) s.push_back({a, b, c});
      }
  return s;
}

// [1 + nderivs * td][npts][nbasis]
std::vector<double> basis(int cell, int p, const double* pts, long npts, int nderivs) {
  const int td = tdim(cell);
  const auto sp = space(cell, p);
  const long nb = (long)sp.size();
  const int rows = 1 + (nderivs ? td : 0);
  std::vector<double> out((size_t)rows * npts * nb);
  std::vector<double> val(3 * (p + 1)), der(3 * (p + 1));
  const bool collapsed = cell == kTriangle || cell == kTetrahedron || cell == kPrism;
  std::vector<double> v1(nb), g1((size_t)nb * 3);
  for (long q = 0; q < npts; ++q) {
    if (collapsed || cell == kPyramid) {
      if (cell == kPyramid)
        pyramid_point(p, pts + q * td, sp, v1.data(), g1.data());
      else
        dubiner_point(cell, p, pts + q * td, sp, v1.data(), g1.data());
      for (long j = 0; j < nb; ++j) {
        out[q * nb + j] = v1[j];
        if (nderivs)
          for (int dd = 0; dd < td; ++dd) out[((size_t)(1 + dd) * npts + q) * nb + j] = g1[j * td + dd];
      }
      continue;
    }
    for (int d = 0; d < td; ++d) legendre01(p, pts[q * td + d], &val[d * (p + 1)], &der[d * (p + 1)]);
    for (long j = 0; j < nb; ++j) {
      double v = 1.0;
      for (int d = 0; d < td; ++d) v *= val[d * (p + 1) + sp[j][d]];
      out[q * nb + j] = v;
      if (nderivs)
        for (int dd = 0; dd < td; ++dd) {
          double f = 1.0;
          for (int d = 0; d < td; ++d)
            f *= (d == dd ? der : val)[d * (p + 1) + sp[j][d]];
          out[((size_t)(1 + dd) * npts + q) * nb + j] = f;
        }
    }
  }
  return out;
}

// Solves A X = B in place (A n x n row-major, B n x m), LU with partial pivoting.
void lu_solve(std::vector<double> a, int n, std::vector<double>& b, int m) {
  for (int col = 0; col < n; ++col) {
    int piv = col;
    for (int r = col + 1; r < n; ++r)
      if (std::fabs(a[(size_t)r * n + col]) > std::fabs(a[(size_t)piv * n + col])) piv = r;
    if (a[(size_t)piv * n + col] == 0.0) throw std::domain_error("singular Vandermonde matrix");
    if (piv != col) {
      for (int j = 0; j < n; ++j) std::swap(a[(size_t)col * n + j], a[(size_t)piv * n + j]);
      for (int j = 0; j < m; ++j) std::swap(b[(size_t)col * m + j], b[(size_t)piv * m + j]);
    }
    for (int r = col + 1; r < n; ++r) {
      const double f = a[(size_t)r * n + col] / a[(size_t)col * n + col];
      if (f == 0.0) continue;
      for (int j = col; j < n; ++j) a[(size_t)r * n + j] -= f * a[(size_t)col * n + j];
      for (int j = 0; j < m; ++j) b[(size_t)r * m + j] -= f * b[(size_t)col * m + j];
    }
  }
  for (int r = n - 1; r >= 0; --r) {
    for (int j = 0; j < m; ++j) {
      double s = b[(size_t)r * m + j];
      for (int c = r + 1; c < n; ++c) s -= a[(size_t)r * n + c] * b[(size_t)c * m + j];
      b[(size_t)r * m + j] = s / a[(size_t)r * n + r];
    }
  }
}

}  // namespace

bool valid_cell(int cell) { return cell >= kPoint && cell <= kPyramid; }

int tdim(int cell) { return tables(cell).td; }

const std::vector<std::vector<double>>& cell_vertices(int cell) { return tables(cell).verts; }

const std::vector<std::vector<int>>& sub_entities(int cell, int dim) {
  static std::vector<std::vector<int>> vert_lists[8], whole[8], none;
  const CellTables& t = tables(cell);
  if (dim == 0) {
    auto& v = vert_lists[cell];
    if (v.empty())
      for (int i = 0; i < (int)t.verts.size(); ++i) v.push_back({i});
    return v;
  }
  if (dim > t.td) return none;
  if (dim == t.td) {
    auto& w = whole[cell];
    if (w.empty()) {
      std::vector<int> all;
      for (int i = 0; i < (int)t.verts.size(); ++i) all.push_back(i);
      w.push_back(all);
    }
    return w;
  }
  return dim == 1 ? t.edges : t.faces;
}

int entity_type(int cell, int dim, int index) {
  if (dim == 0) return kPoint;
  if (dim == 1) return kInterval;
  if (dim == tdim(cell)) return cell;
  return sub_entities(cell, dim)[index].size() == 3 ? kTriangle : kQuadrilateral;
}

long num_lagrange_nodes(int cell, int p) {
  const long a = p + 1, b = p + 2;
  switch (cell) {
    case kPoint: return 1;
    case kInterval: return a;
    case kTriangle: return a * b / 2;
    case kQuadrilateral: return a * a;
    case kTetrahedron: return a * b * (p + 3) / 6;
    case kHexahedron: return a * a * a;
    case kPrism: return a * a * b / 2;
    case kPyramid: return a * b * (2 * p + 3) / 6;
  }
  return -1;
}

void gauss_jacobi(int m, double alpha, std::vector<double>& x, std::vector<double>& w) {
  if (m < 1) throw std::invalid_argument("a Gauss rule needs at least one point");
  const std::vector<double> t = jacobi_roots(m, alpha, 0.0);
  x.resize(m);
  w.resize(m);
  double sum = 0.0;
  for (int i = 0; i < m; ++i) {
    double p, dp;
    jacobi(m, alpha, 0.0, t[i], p, dp);
    w[i] = 1.0 / ((1.0 - t[i] * t[i]) * dp * dp);
    sum += w[i];
    x[i] = 0.5 * (1.0 + t[i]);
  }
  const double scale = 1.0 / ((alpha + 1.0) * sum);
  for (double& wi : w) wi *= scale;
}

std::vector<double> gll_points(int m) {
  if (m < 2) throw std::invalid_argument("GLL points need both ends");
  std::vector<double> pts(m, 0.0);
  pts[m - 1] = 1.0;
  if (m > 2) {
    // Interior points: the zeros of P'_{m-1}, i.e. of P_{m-2}^(1, 1); symmetrised.
    const std::vector<double> t = jacobi_roots(m - 2, 1.0, 1.0);
    for (int i = 1; i <= m - 2; ++i) {
      const double lo = 0.5 * (1.0 + t[i - 1]);
      const double hi = 0.5 * (1.0 + t[m - 2 - i]);
      pts[i] = 0.5 * (lo + (1.0 - hi));
    }
    if (m % 2 == 1) pts[m / 2] = 0.5;
  }
  return pts;
}

std::vector<double> lagrange_points(int cell, int p, int family) {
  if (p < 1) throw std::invalid_argument("Lagrange nodes need degree >= 1");
  const int td = tdim(cell);
  std::vector<double> line;
  if (family == 0) {
    for (int i = 1; i < p; ++i) line.push_back((double)i / p);
  } else if (family == 1) {
    if (cell != kInterval && cell != kQuadrilateral && cell != kHexahedron)
      throw std::invalid_argument("GLL nodes exist on intervals, quadrilaterals, hexahedra only");
    const auto g = gll_points(p + 1);
    line.assign(g.begin() + 1, g.begin() + p);
  } else {
    throw std::invalid_argument("unknown node family");
  }
  const auto& verts = cell_vertices(cell);
  std::vector<double> out;
  out.reserve((size_t)num_lagrange_nodes(cell, p) * td);
  auto frac = [p](int i) { return (double)i / p; };
  for (int dim = 0; dim <= td; ++dim) {
    const auto& ents = sub_entities(cell, dim);
    for (int e = 0; e < (int)ents.size(); ++e) {
      const auto& ent = ents[e];
      auto push = [&](std::initializer_list<double> t, std::initializer_list<int> axes) {
        for (int j = 0; j < td; ++j) {
          const double v0 = verts[ent[0]][j];
          double x = v0;
          auto a = axes.begin();
          for (double tk : t) {
            x += tk * (verts[ent[*a]][j] - v0);
            ++a;
          }
          out.push_back(x);
        }
      };
      switch (entity_type(cell, dim, e)) {
        case kPoint: push({}, {}); break;
        case kInterval:
          for (double t : line) push({t}, {1});
          break;
        case kTriangle:
          for (int i1 = 1; i1 < p; ++i1)
            for (int i0 = 1; i0 < p - i1; ++i0) push({frac(i0), frac(i1)}, {1, 2});
          break;
        case kQuadrilateral:
          for (double t1 : line)
            for (double t0 : line) push({t0, t1}, {1, 2});
          break;
        case kTetrahedron:
          for (int i2 = 1; i2 < p; ++i2)
            for (int i1 = 1; i1 < p - i2; ++i1)
              for (int i0 = 1; i0 < p - i2 - i1; ++i0) push({frac(i0), frac(i1), frac(i2)}, {1, 2, 3});
          break;
        case kHexahedron:
          for (double t2 : line)
            for (double t1 : line)
              for (double t0 : line) push({t0, t1, t2}, {1, 2, 4});
          break;
        case kPrism:
          for (int i2 = 1; i2 < p; ++i2)
            for (int i1 = 1; i1 < p; ++i1)
              for (int i0 = 1; i0 < p - i1; ++i0) push({frac(i0), frac(i1), frac(i2)}, {1, 2, 3});
          break;
        case kPyramid:
          for (int i2 = 1; i2 < p - 1; ++i2)
            for (int i1 = 1; i1 < p - i2; ++i1)
              for (int i0 = 1; i0 < p - i2; ++i0) {
                out.push_back(frac(i0));
                out.push_back(frac(i1));
                out.push_back(frac(i2));
              }
          break;
      }
    }
  }
  return out;
}

void collapsed_rule(int cell, const int* counts, std::vector<double>& points,
                    std::vector<double>& weights) {
  const int td = tdim(cell);
  points.clear();
  weights.clear();
  if (td == 0) {
    weights.push_back(1.0);
    return;
  }
  // Weight exponent alpha of each direction and the map to the reference cell.
  double alpha[3] = {0, 0, 0};
  switch (cell) {
    case kTriangle: alpha[1] = 1; break;
    case kTetrahedron: alpha[1] = 1; alpha[2] = 2; break;
    case kPrism: alpha[1] = 1; break;
    case kPyramid: alpha[2] = 2; break;
    default: break;
  }
  std::vector<double> x[3], w[3];
  long total = 1;
  for (int d = 0; d < td; ++d) {
    gauss_jacobi(counts[d], alpha[d], x[d], w[d]);
    total *= counts[d];
  }
  int idx[3] = {0, 0, 0};
  for (long n = 0; n < total; ++n) {
    double p[3] = {0, 0, 0}, wt = 1.0;
    for (int d = 0; d < td; ++d) {
      p[d] = x[d][idx[d]];
      wt *= w[d][idx[d]];
    }
    double m[3] = {p[0], p[1], p[2]};
    switch (cell) {
      case kTriangle: m[0] = p[0] * (1.0 - p[1]); break;
      case kTetrahedron: {
        const double s = 1.0 - p[2];
        m[0] = p[0] * (1.0 - p[1]) * s;
        m[1] = p[1] * s;
        break;
      }
      case kPrism: m[0] = p[0] * (1.0 - p[1]); break;
      case kPyramid: {
        const double s = 1.0 - p[2];
        m[0] = p[0] * s;
        m[1] = p[1] * s;
        break;
      }
      default: break;
    }
    for (int d = 0; d < td; ++d) points.push_back(m[d]);
    weights.push_back(wt);
    for (int d = 0; d < td; ++d) {  // first direction fastest
      if (++idx[d] < counts[d]) break;
      idx[d] = 0;
    }
  }
}

std::vector<double> expansion_coefficients(int cell, int degree, int family) {
  const std::vector<double> nodes = lagrange_points(cell, degree, family);
  const int n = (int)num_lagrange_nodes(cell, degree);
  // V[i][m] = basis_m(node_i); coefficients C = V^-1 (V C = I).
  const std::vector<double> v = basis(cell, degree, nodes.data(), n, 0);
  std::vector<double> c((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) c[(size_t)i * n + i] = 1.0;
  lu_solve(v, n, c, n);
  return c;
}

std::vector<double> tabulate(int cell, int degree, int family, const double* points, long npoints,
                             int nderivs) {
  if (nderivs < 0 || nderivs > 1) throw std::invalid_argument("derivative order must be 0 or 1");
  const int td = tdim(cell);
  const int n = (int)num_lagrange_nodes(cell, degree);
  const std::vector<double> c = expansion_coefficients(cell, degree, family);
  const std::vector<double> phi = basis(cell, degree, points, npoints, nderivs);
  const int rows = 1 + (nderivs ? td : 0);
  std::vector<double> out((size_t)rows * npoints * n, 0.0);
  for (long r = 0; r < (long)rows * npoints; ++r)
    for (int m = 0; m < n; ++m) {
      const double f = phi[(size_t)r * n + m];
      if (f == 0.0) continue;
      for (int j = 0; j < n; ++j) out[(size_t)r * n + j] += f * c[(size_t)m * n + j];
    }
  return out;
}

std::vector<double> reference_facet_normals(int cell) {
  const int td = tdim(cell);
  if (td < 1) throw std::invalid_argument("the point cell has no facets");
  const auto& verts = cell_vertices(cell);
  std::vector<double> mid(td, 0.0);
  for (const auto& v : verts)
    for (int j = 0; j < td; ++j) mid[j] += v[j] / verts.size();
  std::vector<double> out;
  for (const auto& f : sub_entities(cell, td - 1)) {
    double n[3] = {1.0, 0.0, 0.0};
    if (td == 2) {
      n[0] = verts[f[1]][1] - verts[f[0]][1];
      n[1] = -(verts[f[1]][0] - verts[f[0]][0]);
    } else if (td == 3) {
      double a[3], b[3];
      for (int j = 0; j < 3; ++j) {
        a[j] = verts[f[1]][j] - verts[f[0]][j];
        b[j] = verts[f[2]][j] - verts[f[0]][j];
      }
      n[0] = a[1] * b[2] - a[2] * b[1];
      n[1] = a[2] * b[0] - a[0] * b[2];
      n[2] = a[0] * b[1] - a[1] * b[0];
    }
    double dir = 0.0, len = 0.0;
    for (int j = 0; j < td; ++j) {
      double fc = 0.0;
      for (int v : f) fc += verts[v][j] / f.size();
      dir += n[j] * (fc - mid[j]);
      len += n[j] * n[j];
    }
    const double s = (dir > 0 ? 1.0 : -1.0) / std::sqrt(len);
    for (int j = 0; j < td; ++j) out.push_back(n[j] * s);
  }
  return out;
}

}  // namespace tlg
