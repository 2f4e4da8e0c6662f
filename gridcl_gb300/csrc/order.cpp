// Cell orderings of a mesh block before upload, and node numbering by first use
// (tetraloma/src/pipeline/order.rs:24-192, tetraloma/src/builder.rs:95-113): the order in which
// the kernels visit cells, which sets the locality of the node gathers.
//
//  - input: the given order;
//  - Hilbert: by the Hilbert key of the cell's vertex centroid, each coordinate quantised to
//    2^21 steps in the node bounding box (floor, clamped; 0 on an axis of zero extent), then by
//    input position. The key follows J. Skilling, "Programming the Hilbert curve" (AIP Conf.
//    Proc. 707, 2004): the transpose of the key by the inverse-undo and Gray-encode passes, then
//    its bits interleaved from the most significant, axis 0 first; the curve starts at the origin;
//  - reverse Cuthill-McKee on the facet graph (cells sharing a facet, facets keyed by their
//    sorted vertex numbers): each connected component starts at its cell of least (degree,
//    input position), neighbours are queued by (degree, input position), and the whole order is
//    reversed.
// Nodes are then numbered in the order of the first cell that uses them (each cell's nodes in
// Lagrange order), unused nodes last in their old order.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/tlgeom.h"
#include "refcell.h"
#include "status.h"

namespace {

constexpr int kHilbertBits = 21;

uint64_t hilbert_key(const uint32_t* in, int d, int bits) {
  uint32_t x[3] = {0, 0, 0};
  for (int i = 0; i < d; ++i) x[i] = in[i];
  const uint32_t m = 1u << (bits - 1);
  for (uint32_t q = m; q > 1; q >>= 1) {  // inverse undo
    const uint32_t p = q - 1;
    for (int i = 0; i < d; ++i) {
      if (x[i] & q) {
        x[0] ^= p;
      } else {
        const uint32_t t = (x[0] ^ x[i]) & p;
        x[0] ^= t;
        x[i] ^= t;
      }
    }
  }
  for (int i = 1; i < d; ++i) x[i] ^= x[i - 1];  // Gray encode
  uint32_t t = 0;
  for (uint32_t q = m; q > 1; q >>= 1)
    if (x[d - 1] & q) t ^= q - 1;
  for (int i = 0; i < d; ++i) x[i] ^= t;
  uint64_t key = 0;
  for (int b = bits - 1; b >= 0; --b)
    for (int i = 0; i < d; ++i) key = (key << 1) | ((x[i] >> b) & 1u);
  return key;
}

uint32_t quantise(double x, double lo, double hi) {
  const double cells = (double)(1u << kHilbertBits);
  if (!(hi > lo)) return 0;
  double v = std::floor((x - lo) / (hi - lo) * cells);
  v = std::min(std::max(v, 0.0), cells - 1.0);
  return (uint32_t)v;
}

int num_vertices(int cell) {
  switch (cell) {
    case tlg::kInterval: return 2;
    case tlg::kTriangle: return 3;
    case tlg::kQuadrilateral: return 4;
    case tlg::kTetrahedron: return 4;
    case tlg::kHexahedron: return 8;
    case tlg::kPrism: return 6;
    default: return 0;
  }
}

std::vector<int64_t> hilbert_order(int cell, const uint32_t* cells, int64_t n, int k, const double* nodes,
                                   int64_t nnodes, int gd) {
  const int nv = num_vertices(cell);
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  for (int g = 0; g < gd; ++g) {
    lo[g] = INFINITY;
    hi[g] = -INFINITY;
  }
  for (int64_t i = 0; i < nnodes; ++i)
    for (int g = 0; g < gd; ++g) {
      lo[g] = std::min(lo[g], nodes[i * gd + g]);
      hi[g] = std::max(hi[g], nodes[i * gd + g]);
    }
  std::vector<std::pair<uint64_t, int64_t>> keys((size_t)n);
  for (int64_t c = 0; c < n; ++c) {
    uint32_t q[3] = {0, 0, 0};
    for (int g = 0; g < gd; ++g) {
      double sum = 0.0;
      for (int v = 0; v < nv; ++v) sum += nodes[(int64_t)std::min<int64_t>(cells[c * k + v], nnodes - 1) * gd + g];
      q[g] = quantise(sum / nv, lo[g], hi[g]);
    }
    keys[(size_t)c] = {hilbert_key(q, gd, kHilbertBits), c};
  }
  std::sort(keys.begin(), keys.end());
  std::vector<int64_t> order((size_t)n);
  for (int64_t i = 0; i < n; ++i) order[(size_t)i] = keys[(size_t)i].second;
  return order;
}

// The facet graph in compressed rows of sorted, distinct neighbours: every (facet key, cell) pair
// sorted by key, the cells of each run of equal keys joined pairwise. A facet key is its sorted
// vertex numbers, 32 bits each, packed into two 64-bit words (absent vertices all ones).
struct FacetGraph {
  std::vector<int64_t> start, len, nbr;  // row c: nbr[start[c] .. start[c] + len[c])
};

FacetGraph facet_graph(int cell, const uint32_t* cells, int64_t n, int k) {
  const int td = tlg::tdim(cell);
  const auto& facets = tlg::sub_entities(cell, td - 1);
  struct Entry {
    uint64_t hi, lo;
    int64_t cell;
    bool operator<(const Entry& o) const {
      return hi != o.hi ? hi < o.hi : lo != o.lo ? lo < o.lo : cell < o.cell;
    }
  };
  std::vector<Entry> entries;
  entries.reserve((size_t)n * facets.size());
  for (int64_t c = 0; c < n; ++c)
    for (const auto& f : facets) {
      uint32_t v[4] = {UINT32_MAX, UINT32_MAX, UINT32_MAX, UINT32_MAX};
      for (size_t j = 0; j < f.size(); ++j) v[j] = cells[c * k + f[j]];
      std::sort(v, v + f.size());
      entries.push_back({(uint64_t)v[0] << 32 | v[1], (uint64_t)v[2] << 32 | v[3], c});
    }
  std::sort(entries.begin(), entries.end());
  // Runs of equal keys; two passes over them: count each cell's pairs, then write them.
  std::vector<std::pair<size_t, size_t>> runs;
  for (size_t i = 0; i < entries.size();) {
    size_t j = i + 1;
    while (j < entries.size() && entries[j].hi == entries[i].hi && entries[j].lo == entries[i].lo) ++j;
    if (j - i > 1) runs.push_back({i, j});
    i = j;
  }
  FacetGraph g;
  g.start.assign((size_t)n + 1, 0);
  g.len.assign((size_t)n, 0);
  // A cell's neighbours across a facet are the other cells of the facet's run (a degenerate cell
  // with two facets on the same vertices does not neighbour itself, as in order.rs:147).
  for (const auto& r : runs)
    for (size_t a = r.first; a < r.second; ++a)
      for (size_t b = r.first; b < r.second; ++b)
        if (entries[b].cell != entries[a].cell) ++g.start[(size_t)entries[a].cell + 1];
  for (int64_t c = 0; c < n; ++c) g.start[(size_t)c + 1] += g.start[(size_t)c];
  g.nbr.resize((size_t)g.start[(size_t)n]);
  std::vector<int64_t> fill(g.start.begin(), g.start.end() - 1);
  for (const auto& r : runs)
    for (size_t a = r.first; a < r.second; ++a)
      for (size_t b = r.first; b < r.second; ++b)
        if (entries[b].cell != entries[a].cell) g.nbr[(size_t)fill[(size_t)entries[a].cell]++] = entries[b].cell;
  for (int64_t c = 0; c < n; ++c) {
    auto first = g.nbr.begin() + g.start[(size_t)c], last = g.nbr.begin() + g.start[(size_t)c + 1];
    std::sort(first, last);
    g.len[(size_t)c] = std::unique(first, last) - first;
  }
  return g;
}

std::vector<int64_t> rcm_order(int cell, const uint32_t* cells, int64_t n, int k) {
  const FacetGraph adj = facet_graph(cell, cells, n, k);
  auto rank_less = [&](int64_t a, int64_t b) {
    const int64_t da = adj.len[(size_t)a], db = adj.len[(size_t)b];
    return da != db ? da < db : a < b;
  };
  std::vector<int64_t> starts((size_t)n);
  for (int64_t i = 0; i < n; ++i) starts[(size_t)i] = i;
  std::sort(starts.begin(), starts.end(), rank_less);
  std::vector<char> visited((size_t)n, 0);
  std::vector<int64_t> order, next;
  order.reserve((size_t)n);
  for (int64_t s : starts) {
    if (visited[(size_t)s]) continue;
    visited[(size_t)s] = 1;
    size_t head = order.size();
    order.push_back(s);
    while (head < order.size()) {
      const int64_t a = order[head++];
      next.clear();
      for (int64_t e = adj.start[(size_t)a]; e < adj.start[(size_t)a] + adj.len[(size_t)a]; ++e)
        if (!visited[(size_t)adj.nbr[(size_t)e]]) next.push_back(adj.nbr[(size_t)e]);
      std::sort(next.begin(), next.end(), rank_less);
      for (int64_t b : next) {
        visited[(size_t)b] = 1;
        order.push_back(b);
      }
    }
  }
  std::reverse(order.begin(), order.end());
  return order;
}

}  // namespace

uint64_t tlg_hilbert_key(const uint32_t* x, int d, int bits) {
  if (!x || d < 1 || d > 3 || bits < 1 || bits > 32 || d * bits > 64) return 0;
  return hilbert_key(x, d, bits);
}

uint32_t tlg_quantise(double x, double lo, double hi) { return quantise(x, lo, hi); }

tlg_status tlg_order_cells(int ordering, int cell, const uint32_t* cells, int64_t num_cells, int nodes_per_cell,
                           const double* nodes, int64_t num_nodes, int gdim, int64_t* order) {
  if (!order || num_cells < 0 || nodes_per_cell < 1 || (num_cells > 0 && !cells))
    return tlg::fail(TLG_ERR_INVALID_ARGUMENT, "tlg_order_cells: bad arguments");
  if (num_vertices(cell) == 0 || num_vertices(cell) > nodes_per_cell)
    return tlg::fail(TLG_ERR_UNSUPPORTED, "tlg_order_cells: no ordering for this cell type");
  if (ordering < TLG_ORDER_INPUT || ordering > TLG_ORDER_RCM)
    return tlg::fail(TLG_ERR_INVALID_ARGUMENT, "tlg_order_cells: ordering must be 0, 1 or 2");
  try {
    std::vector<int64_t> o;
    if (ordering == TLG_ORDER_INPUT) {
      o.resize((size_t)num_cells);
      for (int64_t i = 0; i < num_cells; ++i) o[(size_t)i] = i;
    } else if (ordering == TLG_ORDER_HILBERT) {
      if (gdim < 1 || gdim > 3 || num_nodes < 1 || !nodes)
        return tlg::fail(TLG_ERR_INVALID_ARGUMENT, "tlg_order_cells: the Hilbert order needs the nodes");
      o = hilbert_order(cell, cells, num_cells, nodes_per_cell, nodes, num_nodes, gdim);
    } else {
      o = rcm_order(cell, cells, num_cells, nodes_per_cell);
    }
    std::copy(o.begin(), o.end(), order);
    return tlg::ok();
  } catch (const std::exception& e) {
    return tlg::fail(TLG_ERR_INVALID_ARGUMENT, std::string("tlg_order_cells: ") + e.what());
  }
}

tlg_status tlg_number_nodes(const uint32_t* cells, int64_t num_cells, int nodes_per_cell, int64_t num_nodes,
                            uint32_t* new_cells, int64_t* node_order) {
  if (num_cells < 0 || nodes_per_cell < 1 || num_nodes < 0 || !node_order || (num_cells > 0 && (!cells || !new_cells)))
    return tlg::fail(TLG_ERR_INVALID_ARGUMENT, "tlg_number_nodes: bad arguments");
  std::vector<int64_t> new_id((size_t)num_nodes, -1);
  int64_t next = 0;
  for (int64_t i = 0; i < num_cells * nodes_per_cell; ++i) {
    const uint32_t n = cells[i];
    if ((int64_t)n >= num_nodes) return tlg::fail(TLG_ERR_INVALID_ARGUMENT, "tlg_number_nodes: node index out of range");
    if (new_id[n] < 0) {
      new_id[n] = next;
      node_order[next++] = n;
    }
    new_cells[i] = (uint32_t)new_id[n];
  }
  for (int64_t n = 0; n < num_nodes; ++n)
    if (new_id[(size_t)n] < 0) node_order[next++] = n;
  return tlg::ok();
}
