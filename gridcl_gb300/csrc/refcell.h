// Host reference-cell tables of the product (f64): Lagrange node layouts, collapsed Gauss
// rules and the Lagrange tabulation that the device tables are built from. C++ restatement of
// the parts of tetraloma-refcell the geometry path reads (tetraloma-refcell/src/lib.rs:58-69).
#pragma once

#include <string>
#include <vector>

namespace tlg {

enum Cell { kPoint = 0, kInterval, kTriangle, kQuadrilateral, kTetrahedron, kHexahedron, kPrism, kPyramid };

int tdim(int cell);
bool valid_cell(int cell);
const std::vector<std::vector<double>>& cell_vertices(int cell);
// Sub-entities of dimension `dim`, each by its sorted vertex list, in lexicographic order.
const std::vector<std::vector<int>>& sub_entities(int cell, int dim);
int entity_type(int cell, int dim, int index);
long num_lagrange_nodes(int cell, int degree);

// Throws std::invalid_argument / std::domain_error with a message on bad input.
std::vector<double> lagrange_points(int cell, int degree, int family);
void gauss_jacobi(int m, double alpha, std::vector<double>& x, std::vector<double>& w);
std::vector<double> gll_points(int m);
void collapsed_rule(int cell, const int* counts, std::vector<double>& points,
                    std::vector<double>& weights);
// C [m][k] (m-major): Lagrange function k = sum_m C[m][k] e_m, e_m the expansion set (on
// pyramids the orthogonal rationomials (i, j, k), i outer, j, then k, max(i, j) + k <= degree).
std::vector<double> expansion_coefficients(int cell, int degree, int family);
// [deriv][q][k]
std::vector<double> tabulate(int cell, int degree, int family, const double* points, long npoints,
                             int nderivs);
std::vector<double> reference_facet_normals(int cell);

}  // namespace tlg
