// The C ABI of include/tlgeom.h: argument checks with the reference's error kinds, the device
// tables (tabulations, point pairs, the adjoint's node rows, sum-factorisation blocks), the
// strategy settings and policy, and the launches of the evaluation, E-vector and adjoint kernels,
// singly and as CUDA-graph batches.
#include <algorithm>
#include <array>
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/tlgeom.h"
#include "eval_launch.cuh"
#include "refcell.h"
#include "status.h"
#include "coop.cuh"
#include "tc.cuh"
#include "umma.cuh"
#include "sumfact.cuh"
#include "eval_df.cuh"
#include "sumfact_df.cuh"
#include "vjp.cuh"

struct tlg_batch {
  std::vector<const tlg_tables*> tables;
  std::vector<tlg_block> blocks;
  std::vector<tlg_outputs> outputs;
  std::vector<int> grid;  // launch grid per block (0: the kernel's persistent default)
  std::vector<int> strategy;  // per block: TLG_STRATEGY_* forced on every family, -1 the caller's
  bool serial = false;    // the blocks one after another instead of parallel graph branches
  float tuned_ms = 0.0f;  // the tuner's median time of the chosen graph (0: not tuned here)
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> events;  // fork, then one join per block
  cudaStream_t capture = nullptr;
  cudaGraphExec_t exec = nullptr;
};

struct tlg_tables {
  int cell, degree, family, td, gd, dtype;
  // Double-float tables (TLG_DF64): dtype is TLG_F64 (every f64 section, so that the f64 kernels
  // run on them), plus the double-float sections below.
  bool df = false;
  int64_t k, q;
  bool has_refn;
  unsigned char* dev = nullptr;  // phi [Q][K] | dphi [Q][K][TD] | refn [Q][TD] | error word
  uint32_t bytes = 0;            // table bytes (multiple of 16), error word excluded
  bool staged = true;            // the tables fit the kernels' shared-memory budget
  uint32_t off_dphi = 0, off_refn = 0, off_rows2 = 0, off_dphi64 = 0;
  // Double-float rows of the paired f64 kernels, inside the staged prefix (0 bytes beyond 27
  // nodes per cell): per point pair p and node k, 1 + TD float4 (phi, dphi_0 .. dphi_{TD-1}), each
  // (head of point 2p, head of point 2p + 1, tail of 2p, tail of 2p + 1); an odd last point pairs
  // with itself.
  uint32_t off_dfrows = 0, dfrows_bytes = 0;
  // The double-float monomial form (tetrahedra P1-P3): dfrows hold the monomials' rows, off_dfmono
  // the expansion C [k][m] (f32 head, tail) and the monomials' direction masks.
  uint32_t off_dfmono = 0;
  bool df_mono = false;
  // The adjoint's table after the error word (codimension 0, f64 or split tables; 0 bytes when
  // absent or too large to stage): per node of each point (f64) or point pair (split) the 32
  // bytes phi, dphi_0 .. dphi_{TD-1}, zero padding, as f64 values or f32 pairs.
  uint32_t off_vjp = 0, vjp_bytes = 0;
  // Sum-factorisation section (quadrilaterals and hexahedra at a tensor-product point set), after
  // the adjoint's: per direction d, B_d [m_d][N] = l_i(u_d[a]) and D_d [m_d][N] = l_i'(u_d[a]) in the
  // arithmetic's type, then perm [K] u32 (lexicographic node index -> Lagrange node); offsets
  // relative to the section.
  // The section holds the block headers (tlg::SfBlock each), the blocks' tables, the permutation
  // and, for facet rules, the reference normals [Q][TD] in the arithmetic's type; offsets are
  // relative to the section. Prisms: per block psi, d_x psi, d_y psi [m_t][NT] in B_0, D_0, D_1,
  // the interval's l, l' [m_z][N] in B_2, D_2, perm [N * NT] (index c NT + t -> Lagrange node).
  bool sf_ok = false, sf_prism = false;
  int sf_n = 0, sf_nblocks = 0;
  tlg::SfBlock sf_block0{};  // the first block (the adjoint's single-block rule)
  uint32_t off_sf = 0, sf_bytes = 0, sf_offperm = 0, sf_offrefn = 0;
  // Double-float tables: the sum-factorisation section again after it, with headers of its own:
  // B_d and D_d as (head, tail) f32 pairs [m_d][cols], except the direction whose points the
  // kernels take two at a time (direction 0; the z points of prisms), stored per point pair as
  // float4 (head of a, head of a + 1, tail of a, tail of a + 1) [ceil(m_d / 2)][cols], a + 1 clamped
  // to the last point; then perm and the f64 reference normals.
  uint32_t off_sfdf = 0, sfdf_bytes = 0, sfdf_offperm = 0, sfdf_offrefn = 0;
  // Tensor-core section (f32 and split tables, TD >= 2), after the sum-factorisation section, read
  // from global memory: the basis in mma fragment order, [col tile][k-step][lane] x 4 f32
  // (b0 head, b1 head, b0 tail, b1 tail) of B[k][4 q + r] (r = 0 phi, 1 + d dphi_d).
  uint64_t off_tc = 0;
  int tc_ksteps = 0, tc_col_tiles = 0;
  // Section of the tcgen05 kernel (f32 and split tables of volume cells in 3D, 20 < K <= 88): per
  // chunk of 8 points the TF32 heads, then the tails, of B[32 x kpad] (column 4 p + r of point
  // 8 chunk + p, r = 0 phi, 1 + d dphi_d; node k) in the canonical K-major layout of the MMA
  // operands (8-row x 16-byte core matrices, 128 bytes apart along K, kpad * 32 bytes apart along
  // the columns), copied into shared memory chunk by chunk.
  uint64_t off_umma = 0;
  int umma_kpad = 0, umma_chunks = 0;
  int* err = nullptr;
  std::vector<unsigned char> host;  // host copy of the device bytes
};

namespace {
thread_local std::string g_error;
}  // namespace

namespace tlg {

tlg_status fail(tlg_status s, const std::string& msg) {
  g_error = msg;
  return s;
}

tlg_status ok() {
  g_error.clear();
  return TLG_OK;
}

tlg_status cuda_fail(cudaError_t e, const char* what) {
  return fail(TLG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace tlg

namespace {

using tlg::cuda_fail;
using tlg::fail;
using tlg::ok;

// Runs `f`, turning the refcell's exceptions into status codes.
template <typename Fn>
tlg_status guarded(Fn f) {
  try {
    return f();
  } catch (const std::invalid_argument& e) {
    return fail(TLG_ERR_INVALID_ARGUMENT, e.what());
  } catch (const std::domain_error& e) {
    return fail(TLG_ERR_UNSUPPORTED, e.what());
  } catch (const std::exception& e) {
    return fail(TLG_ERR_INVALID_ARGUMENT, e.what());
  }
}

uint32_t align16(size_t x) { return (uint32_t)((x + 15) / 16 * 16); }

int tile_shift(int tile) {
  switch (tile) {
    case 1: return 0;
    case 2: return 1;
    case 4: return 2;
    case 8: return 3;
    case 16: return 4;
  }
  return -1;
}

template <typename F>
void narrow_into(std::vector<unsigned char>& buf, size_t off, const double* src, size_t n) {
  F* dst = reinterpret_cast<F*>(buf.data() + off);
  for (size_t i = 0; i < n; ++i) dst[i] = (F)src[i];
}

// f64 values as double-floats: (nearest f32, f32 nearest to the remainder) pairs.
void split_into(std::vector<unsigned char>& buf, size_t off, const double* src, size_t n) {
  float* dst = reinterpret_cast<float*>(buf.data() + off);
  for (size_t i = 0; i < n; ++i) {
    dst[2 * i] = (float)src[i];
    dst[2 * i + 1] = (float)(src[i] - (double)(float)src[i]);
  }
}

// The paired-FP32 kernel: an f32 mesh (split = false) or split precision (split = true).
// `found` is false when no paired kernel exists for the element (nothing launched).
// Strategies per kernel family (tetraloma-geometry/src/strategy.rs:311-407): this thread's
// override (tlg_set_family_strategy, tlg_set_strategy), else TLG_GEOM_STRATEGY, else the policy
// (TLG_STRATEGY_AUTO). -1: no override.
constexpr int kFamilies = 6;
thread_local int g_override[kFamilies] = {-1, -1, -1, -1, -1, -1};
// The strategy that ran in this thread's last launch (TLG_STRATEGY_*, 0: none) and its family.
thread_local int g_last_family = 0;
thread_local bool g_measure_fused = false;  // the last eval launch summed cell_measure
thread_local int g_last_kind = -1;

const char* const kFamilyNames[kFamilies] = {"EVector", "Points", "Jacobian", "Normals", "FacetNormals", "PullBack"};

// A strategy name of the environment variable: policy (or auto), direct, loops, sumfact, shared,
// cooperative; -1 for anything else.
int strategy_named(std::string n) {
  while (!n.empty() && n.front() == ' ') n.erase(n.begin());
  while (!n.empty() && n.back() == ' ') n.pop_back();
  const char* names[] = {"policy", "direct", "loops", "sumfact", "shared", "cooperative", "tensor"};
  for (int i = 0; i < 7; ++i)
    if (n == names[i]) return i;
  if (n == "auto") return TLG_STRATEGY_AUTO;
  return -1;
}

struct EnvStrategies {
  int s[kFamilies] = {-1, -1, -1, -1, -1, -1};
  std::string error;  // non-empty: the variable is invalid (every launch then fails)
};

// TLG_GEOM_STRATEGY, read once: one strategy name for every family, or a comma list of
// <family>=<strategy> (families EVector, Points, Jacobian, Normals, FacetNormals, PullBack, in any
// case), each family at most once (strategy.rs:311-337).
const EnvStrategies& env_strategies() {
  static const EnvStrategies v = [] {
    EnvStrategies r;
    const char* e = std::getenv("TLG_GEOM_STRATEGY");
    if (!e || !*e) return r;
    const std::string val(e);
    const std::string invalid = "TLG_GEOM_STRATEGY=" + val +
                                ": expected policy, direct, loops, sumfact, shared, cooperative or tensor, or a comma "
                                "list of <family>=<strategy> with the families EVector, Points, Jacobian, "
                                "Normals, FacetNormals and PullBack";
    const int one = strategy_named(val);
    if (one >= 0) {
      for (int& x : r.s) x = one;
      return r;
    }
    size_t pos = 0;
    while (pos <= val.size()) {
      size_t comma = val.find(',', pos);
      if (comma == std::string::npos) comma = val.size();
      const std::string item = val.substr(pos, comma - pos);
      const size_t eq = item.find('=');
      int fam = -1;
      if (eq != std::string::npos) {
        std::string f = item.substr(0, eq);
        while (!f.empty() && f.front() == ' ') f.erase(f.begin());
        while (!f.empty() && f.back() == ' ') f.pop_back();
        for (int i = 0; i < kFamilies; ++i) {
          const std::string n = kFamilyNames[i];
          bool same = n.size() == f.size();
          for (size_t c = 0; same && c < n.size(); ++c) same = std::tolower((unsigned char)n[c]) == std::tolower((unsigned char)f[c]);
          if (same) fam = i;
        }
      }
      const int st = eq == std::string::npos ? -1 : strategy_named(item.substr(eq + 1));
      if (fam < 0 || st < 0) {
        r.error = invalid;
        return r;
      }
      if (r.s[fam] >= 0) {
        r.error = invalid + ": " + kFamilyNames[fam] + " given twice";
        return r;
      }
      r.s[fam] = st;
      pos = comma + 1;
    }
    return r;
  }();
  return v;
}

// The strategy wanted for a family (override, environment, policy); false with the error set when
// the environment variable is invalid.
bool wanted_strategy(int family, int* out) {
  const EnvStrategies& env = env_strategies();
  if (!env.error.empty()) {
    fail(TLG_ERR_INVALID_ARGUMENT, env.error);
    return false;
  }
  if (g_override[family] >= 0) *out = g_override[family];
  else if (env.s[family] >= 0) *out = env.s[family];
  else *out = TLG_STRATEGY_AUTO;
  return true;
}

// The family whose strategy decides a fused launch: J, det J and K are the Jacobian family; else
// normals, facet normals, points, in that order.
int principal_family(uint32_t mask) {
  if (mask & (tlg::kOutJacobian | tlg::kOutDetJ | tlg::kOutPinv)) return TLG_FAMILY_JACOBIAN;
  if (mask & tlg::kOutNormals) return TLG_FAMILY_NORMALS;
  if (mask & tlg::kOutFacetNormals) return TLG_FAMILY_FACET_NORMALS;
  return TLG_FAMILY_POINTS;
}

// The policy of TLG_STRATEGY_AUTO for tables with sum-factorisation data, from GB300 timings of
// curved hexahedra (ms per launch, 128^3 Q1/Q2, 64^3 Q3; paired-or-unrolled / loops / sumfact):
// f64 Q1 4.19 / 5.00 / 3.14, Q2 34.6 / 45.3 / 13.1 (the FP64 pipe bounds, and sum factorisation
// does a third of the multiply-adds); split Q1 0.33 / 1.21 / 0.35, Q2 1.37 / 21.9 / 1.53,
// Q3 - / 11.5 / 0.62; f32 Q2 1.15 / 17.6 / 1.39, Q3 - / 16.7 / 0.55. So: sum factorisation
// always in f64, and in f32 and split precision above the degrees with paired kernels
// (quadrilaterals and hexahedra Q1-Q2).
bool sumfact_preferred(const tlg_tables* t) { return t->sf_ok && (t->dtype == TLG_F64 || t->sf_n >= 4); }

// The policy of TLG_STRATEGY_AUTO beyond the compiled unrolled kernels (more than 27 nodes per
// cell): the cooperative kernel instead of the loops kernel.
bool coop_preferred(const tlg_tables* t) { return t->k > 27; }

// The mma.sync kernel is not in the policy: on GB300 it measured level with the cooperative
// kernel at P4/P5 tetrahedra and slower at P6 (f32 1.42 ms cooperative, 2.03 ms mma.sync), with
// up to 5x the cooperative kernel's error (3xTF32 rounds the tails at 2^-22).
bool tc_preferred(const tlg_tables*) { return false; }

// The tcgen05 kernel replaces the cooperative kernel where it applies (f32 and split tables of
// volume cells in 3D, 27 < K <= 88). GB300, curved tetrahedra 6 x 16^3 at Gauss rules of degree
// 2p, ms (tcgen05 / cooperative): f32 P4 0.180 / 0.197, P5 0.313 / 0.691, P6 0.629 / 1.436;
// split P4 0.201 / 0.215, P5 0.465 / 0.765, P6 0.897 / 2.750.
bool umma_preferred(const tlg_tables* t) { return t->umma_kpad > 0 && t->k > 27; }

// The sum-factorised kernel; `found` is false when it does not apply (no tensor structure, facet
// normals, split precision at a tile other than 16, or no instantiation): nothing is launched.
tlg_status eval_sumfact(const tlg_tables* t, const tlg_block* b, const tlg_outputs* o, uint32_t mask,
                        cudaStream_t stream, bool* found) {
  *found = false;
  if (!t->sf_ok || ((t->dtype == TLG_SPLIT32 || t->df) && o->tile != 16))
    return TLG_ERR_UNSUPPORTED;
  tlg::SfArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nodes = b->nodes;
  a.dofmap = b->dofmap;
  a.flags = b->flags;
  a.tab = t->dev + t->off_sf;
  a.tab_bytes = t->sf_bytes;
  a.dphi64 = t->dtype == TLG_SPLIT32 ? reinterpret_cast<const double*>(t->dev + t->off_dphi64) : nullptr;
  void* outs[6] = {o->points, o->jacobian, o->detj, o->pinv, o->normals, o->facet_normals};
  for (int i = 0; i < 6; ++i) a.out[i] = outs[i];
  a.err = t->err;
  a.recomputed = o->recomputed;
  a.first_cell = o->first_cell;
  a.padded = (o->num_cells + o->tile - 1) / o->tile * o->tile;
  a.range_cells = o->num_cells;
  a.out_first_cell = o->out_first_cell;
  a.tile_shift = tile_shift(o->tile);
  a.last_cell = b->num_cells - 1;
  const int64_t nflags = b->flags ? std::min<int64_t>(b->num_cells, b->num_flags) : 0;
  a.last_flag = nflags - 1;
  for (int g = 0; g < 3; ++g) a.origin[g] = b->origin[g];
  a.cond_limit = o->cond_limit > 0 ? (float)o->cond_limit : 256.0f;
  a.last_node = (uint32_t)(b->num_nodes - 1);
  a.nblocks = t->sf_nblocks;
  a.off_perm = t->sf_offperm;
  a.off_refn = t->sf_offrefn;
  a.prism = t->sf_prism;
  a.mask = mask;
  a.num_points = (int)t->q;
  const size_t fbytes = t->dtype == TLG_F64 ? 8 : 4;
  if (t->df) {  // the double-float section
    a.tab = t->dev + t->off_sfdf;
    a.tab_bytes = t->sfdf_bytes;
    a.off_perm = t->sfdf_offperm;
    a.off_refn = t->sfdf_offrefn;
  }
  // Double-float hexahedra without facet normals: three lanes per cell.
  const bool three = t->df && t->cell == tlg::kHexahedron && !(mask & tlg::kOutFacetNormals);
  const size_t slots = three    ? tlg::sumfact_df3_slot_bytes((int)t->k)
                       : t->df ? tlg::sumfact_df_slot_bytes((int)t->k, t->gd)
                               : tlg::sumfact_slot_bytes((int)t->k, t->gd, fbytes);
  const size_t smem = (a.tab_bytes + 15) / 16 * 16 + slots;
  if (smem > (size_t)227 * 1024) return TLG_ERR_UNSUPPORTED;
  cudaError_t e = three   ? tlg::launch_sumfact_df3(t->sf_n, a, smem, stream, found)
                  : t->df ? tlg::launch_sumfact_df(t->td, t->gd, t->sf_n, a, smem, stream, found)
                          : tlg::launch_sumfact(t->dtype, t->td, t->gd, t->sf_n, a, smem, stream, found);
  if (!*found) return TLG_ERR_UNSUPPORTED;
  if (e != cudaSuccess) return cuda_fail(e, "tlg_eval_block launch");
  g_last_family = TLG_STRATEGY_SUMFACT;
  return ok();
}

void fill_pair_args(const tlg_tables* t, const tlg_block* b, const tlg_outputs* o, uint32_t mask,
                    tlg::PairArgs* ap);

tlg_status eval_pair(const tlg_tables* t, const tlg_block* b, const tlg_outputs* o, uint32_t mask,
                     bool split, cudaStream_t stream, bool* found) {
  tlg::PairArgs a;
  std::memset(&a, 0, sizeof(a));
  fill_pair_args(t, b, o, mask, &a);
  if (!t->staged) {
    *found = false;
    return TLG_ERR_UNSUPPORTED;
  }
  if (o->cell_measure) {  // summed as the points are evaluated
    a.mask |= tlg::kOutCellMeasure;
    a.weights = static_cast<const float*>(o->weights);
    a.cell_measure = static_cast<float*>(o->cell_measure);
  }
  cudaError_t e = o->cell_measure
                      ? tlg::launch_eval_pair_meas(split, t->td, t->gd, (int)t->k, a, t->bytes, stream, found)
                      : tlg::launch_eval_pair(split, t->td, t->gd, (int)t->k, a, t->bytes, stream, found);
  if (!*found) return TLG_ERR_UNSUPPORTED;
  if (e != cudaSuccess) return cuda_fail(e, "tlg_eval_block launch");
  g_last_family = TLG_STRATEGY_DIRECT;
  g_measure_fused = o->cell_measure != nullptr;
  return ok();
}

// The arguments of the paired and split-loops kernels.
void fill_pair_args(const tlg_tables* t, const tlg_block* b, const tlg_outputs* o, uint32_t mask,
                    tlg::PairArgs* ap) {
  tlg::PairArgs& a = *ap;
  a.nodes = b->nodes;
  a.dofmap = b->dofmap;
  a.flags = b->flags;
  a.tab = t->dev;
  void* outs[6] = {o->points, o->jacobian, o->detj, o->pinv, o->normals, o->facet_normals};
  for (int i = 0; i < 6; ++i) a.out[i] = static_cast<float*>(outs[i]);
  a.err = t->err;
  a.recomputed = o->recomputed;
  a.first_cell = o->first_cell;
  a.padded = (o->num_cells + o->tile - 1) / o->tile * o->tile;
  a.range_cells = o->num_cells;
  a.out_first_cell = o->out_first_cell;
  a.last_cell = b->num_cells - 1;
  const int64_t nflags = b->flags ? std::min<int64_t>(b->num_cells, b->num_flags) : 0;
  a.last_flag = nflags - 1;
  for (int g = 0; g < 3; ++g) a.origin[g] = b->origin[g];
  a.cond_limit = o->cond_limit > 0 ? (float)o->cond_limit : 256.0f;
  a.last_node = (uint32_t)(b->num_nodes - 1);
  a.tab_bytes = t->bytes;
  a.off_refn = t->off_refn;
  a.off_rows2 = t->off_rows2;
  a.off_dphi64 = t->off_dphi64;
  a.off_dphi = t->off_dphi;
  a.k_runtime = (int)t->k;
  a.mask = mask;
  a.num_points = (int)t->q;
}

tlg_status eval_split(const tlg_tables* t, const tlg_block* b, const tlg_outputs* o, uint32_t mask,
                      cudaStream_t stream, bool allow_direct, bool global_tables) {
  if (o->tile != 16)
    return fail(TLG_ERR_UNSUPPORTED, "tlg_eval_block: split precision runs with tile 16, not " +
                                         std::to_string(o->tile));
  bool found = false;
  tlg_status st = allow_direct ? eval_pair(t, b, o, mask, true, stream, &found) : TLG_ERR_UNSUPPORTED;
  if (found) return st;
  // No paired kernel for this element, or tables beyond the shared-memory budget.
  tlg::PairArgs a;
  std::memset(&a, 0, sizeof(a));
  fill_pair_args(t, b, o, mask, &a);
  const bool global = global_tables || !t->staged;
  cudaError_t e = tlg::launch_split_loops(t->td, t->gd, global, a, t->bytes, stream);
  if (e != cudaSuccess) return cuda_fail(e, "tlg_eval_block launch");
  g_last_family = global ? TLG_STRATEGY_LOOPS : TLG_STRATEGY_SHARED;
  return ok();
}

// The double-float kernel (TLG_DF64 tables, tile 16); `found` is false where none is compiled or
// the tables lack its rows (nothing launched).
tlg_status eval_df(const tlg_tables* t, const tlg_block* b, const tlg_outputs* o, uint32_t mask,
                   cudaStream_t stream, bool* found) {
  *found = false;
  if (!t->df || t->dfrows_bytes == 0 || o->tile != 16 || !t->staged) return TLG_ERR_UNSUPPORTED;
  tlg::DfArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nodes = static_cast<const double*>(b->nodes);
  a.dofmap = b->dofmap;
  a.flags = b->flags;
  a.tab = t->dev;
  void* outs[6] = {o->points, o->jacobian, o->detj, o->pinv, o->normals, o->facet_normals};
  for (int i = 0; i < 6; ++i) a.out[i] = static_cast<double*>(outs[i]);
  a.err = t->err;
  a.first_cell = o->first_cell;
  a.padded = (o->num_cells + 15) / 16 * 16;
  a.out_first_cell = o->out_first_cell;
  a.last_cell = b->num_cells - 1;
  const int64_t nflags = b->flags ? std::min<int64_t>(b->num_cells, b->num_flags) : 0;
  a.last_flag = nflags - 1;
  for (int g = 0; g < 3; ++g) a.origin[g] = b->origin[g];
  a.last_node = (uint32_t)(b->num_nodes - 1);
  a.tab_bytes = t->bytes;
  a.off_rows = t->off_dfrows;
  a.off_refn = t->off_refn;
  a.mask = mask;
  a.num_points = (int)t->q;
  a.off_mono = t->off_dfmono;
  a.mono = t->df_mono ? 1 : 0;
  const size_t smem = (size_t)(t->bytes + 15) / 16 * 16 + tlg::df_slot_bytes((int)t->k, t->gd, t->df_mono);
  if (smem > (size_t)227 * 1024) return TLG_ERR_UNSUPPORTED;
  cudaError_t e = tlg::launch_eval_df(t->td, t->gd, (int)t->k, a, smem, stream, found);
  if (!*found) return TLG_ERR_UNSUPPORTED;
  if (e != cudaSuccess) return cuda_fail(e, "tlg_eval_block launch");
  g_last_family = TLG_STRATEGY_DIRECT;
  return ok();
}

template <typename F>
tlg_status eval_typed(const tlg_tables* t, const tlg_block* b, const tlg_outputs* o, uint32_t mask,
                      cudaStream_t stream, bool allow_direct, bool global_tables) {
  tlg::EvalArgs<F> a;
  std::memset(&a, 0, sizeof(a));
  a.nodes = static_cast<const F*>(b->nodes);
  a.dofmap = b->dofmap;
  a.flags = b->flags;
  a.tab = t->dev;
  void* outs[6] = {o->points, o->jacobian, o->detj, o->pinv, o->normals, o->facet_normals};
  for (int i = 0; i < 6; ++i) a.out[i] = static_cast<F*>(outs[i]);
  for (int g = 0; g < 3; ++g) a.origin[g] = (F)b->origin[g];
  a.err = t->err;
  const int shift = tile_shift(o->tile);
  a.first_cell = o->first_cell;
  a.padded = (o->num_cells + o->tile - 1) / o->tile * o->tile;
  a.out_first_cell = o->out_first_cell;
  a.last_cell = b->num_cells - 1;
  const int64_t nflags = b->flags ? std::min<int64_t>(b->num_cells, b->num_flags) : 0;
  a.last_flag = nflags - 1;
  a.last_node = (uint32_t)(b->num_nodes - 1);
  a.tab_bytes = t->bytes;
  a.off_dphi = t->off_dphi;
  a.off_refn = t->off_refn;
  a.mask = mask;
  a.num_points = (int)t->q;
  a.tile_shift = shift;
  a.k_runtime = (int)t->k;
  // The unrolled kernels read staged tables; the loops kernel reads them staged or from global
  // memory.
  a.tab_global = t->staged && !global_tables ? 0 : 1;
  a.loops_only = allow_direct && t->staged ? 0 : 1;
  bool direct = false;
  cudaError_t e;
  if constexpr (sizeof(F) == 4) {
    if (shift == 4 && allow_direct) {  // the GPU tile: the paired-FP32 kernel, when compiled
      tlg_status st = eval_pair(t, b, o, mask, false, stream, &direct);
      if (direct) return st;
    }
    e = tlg::launch_eval_f32(t->td, t->gd, (int)t->k, a, t->bytes, stream, &direct);
  } else {
    e = tlg::launch_eval_f64(t->td, t->gd, (int)t->k, a, t->bytes, stream, &direct);
  }
  if (e != cudaSuccess) return cuda_fail(e, "tlg_eval_block launch");
  g_last_family = direct ? TLG_STRATEGY_DIRECT : a.tab_global ? TLG_STRATEGY_LOOPS : TLG_STRATEGY_SHARED;
  return ok();
}

// The tensor-core kernel (f32 and split tables, TD >= 2, tile 16); `found` is false where it does
// not apply (nothing launched).
tlg_status eval_tc(const tlg_tables* t, const tlg_block* b, const tlg_outputs* o, uint32_t mask,
                   cudaStream_t stream, bool* found) {
  *found = false;
  if (t->tc_ksteps == 0 || o->tile != 16 || (t->dtype != TLG_F32 && t->dtype != TLG_SPLIT32))
    return TLG_ERR_UNSUPPORTED;
  const size_t smem = tlg::tc_smem_bytes(t->tc_ksteps, t->gd);
  if (smem > (size_t)227 * 1024) return TLG_ERR_UNSUPPORTED;
  const bool split = t->dtype == TLG_SPLIT32;
  tlg::TcArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nodes = b->nodes;
  a.dofmap = b->dofmap;
  a.flags = b->flags;
  a.bfrag = reinterpret_cast<const float4*>(t->dev + t->off_tc);
  a.refn = reinterpret_cast<const float*>(t->dev + t->off_refn);
  a.dphi64 = split ? reinterpret_cast<const double*>(t->dev + t->off_dphi64) : nullptr;
  void* outs[6] = {o->points, o->jacobian, o->detj, o->pinv, o->normals, o->facet_normals};
  for (int i = 0; i < 6; ++i) a.out[i] = outs[i];
  a.recomputed = split ? o->recomputed : nullptr;
  a.first_cell = o->first_cell;
  a.padded = (o->num_cells + 15) / 16 * 16;
  a.range_cells = o->num_cells;
  a.out_first_cell = o->out_first_cell;
  a.last_cell = b->num_cells - 1;
  const int64_t nflags = b->flags ? std::min<int64_t>(b->num_cells, b->num_flags) : 0;
  a.last_flag = nflags - 1;
  for (int g = 0; g < 3; ++g) a.origin[g] = b->origin[g];
  a.cond_limit = o->cond_limit > 0 ? (float)o->cond_limit : 256.0f;
  a.last_node = (uint32_t)(b->num_nodes - 1);
  a.mask = mask;
  a.k = (int)t->k;
  a.ksteps = t->tc_ksteps;
  a.num_points = (int)t->q;
  a.col_tiles = t->tc_col_tiles;
  cudaError_t e = tlg::launch_tc(split, t->td, t->gd, a, smem, stream, found);
  if (!*found) return TLG_ERR_UNSUPPORTED;
  if (e != cudaSuccess) return cuda_fail(e, "tlg_eval_block launch");
  g_last_family = TLG_STRATEGY_TENSOR;
  return ok();
}

// The tcgen05 kernel (f32 and split tables of volume cells in 3D with 20 < K <= 88, tile 16);
// `found` is false where it does not apply (nothing launched).
tlg_status eval_umma(const tlg_tables* t, const tlg_block* b, const tlg_outputs* o, uint32_t mask,
                     cudaStream_t stream, bool* found) {
  *found = false;
  if (t->umma_kpad == 0 || o->tile != 16 || (t->dtype != TLG_F32 && t->dtype != TLG_SPLIT32) ||
      (mask & tlg::kOutNormals))
    return TLG_ERR_UNSUPPORTED;
  // At least 80 KiB, so that at most two CTAs (2 x 256 tensor-memory columns) share an SM.
  const size_t smem = std::max<size_t>(tlg::umma_smem_bytes(t->umma_kpad), (size_t)80 * 1024);
  if (smem > (size_t)227 * 1024) return TLG_ERR_UNSUPPORTED;
  const bool split = t->dtype == TLG_SPLIT32;
  tlg::UmmaArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nodes = b->nodes;
  a.dofmap = b->dofmap;
  a.flags = b->flags;
  a.btab = t->dev + t->off_umma;
  a.refn = reinterpret_cast<const float*>(t->dev + t->off_refn);
  a.dphi64 = split ? reinterpret_cast<const double*>(t->dev + t->off_dphi64) : nullptr;
  void* outs[6] = {o->points, o->jacobian, o->detj, o->pinv, o->normals, o->facet_normals};
  for (int i = 0; i < 6; ++i) a.out[i] = outs[i];
  a.err = t->err;
  a.recomputed = split ? o->recomputed : nullptr;
  a.first_cell = o->first_cell;
  a.padded = (o->num_cells + 15) / 16 * 16;
  a.range_cells = o->num_cells;
  a.out_first_cell = o->out_first_cell;
  a.last_cell = b->num_cells - 1;
  for (int g = 0; g < 3; ++g) a.origin[g] = b->origin[g];
  a.cond_limit = o->cond_limit > 0 ? (float)o->cond_limit : 256.0f;
  a.last_node = (uint32_t)(b->num_nodes - 1);
  a.mask = mask;
  a.k = (int)t->k;
  a.kpad = t->umma_kpad;
  a.num_points = (int)t->q;
  a.chunks = t->umma_chunks;
  *found = true;
  cudaError_t e = tlg::launch_umma(split, a, smem, stream);
  if (e != cudaSuccess) return cuda_fail(e, "tlg_eval_block launch");
  g_last_family = TLG_STRATEGY_TENSOR;
  return ok();
}

// The cooperative kernel; `found` is false where it does not apply (nothing launched).
tlg_status eval_coop(const tlg_tables* t, const tlg_block* b, const tlg_outputs* o, uint32_t mask,
                     cudaStream_t stream, bool* found) {
  *found = false;
  if (t->td < 2 || t->k > 128 || (t->dtype == TLG_F64 && t->k > 64)) return TLG_ERR_UNSUPPORTED;
  tlg::CoopArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nodes = b->nodes;
  a.dofmap = b->dofmap;
  a.flags = b->flags;
  a.tab = t->dev;
  void* outs[6] = {o->points, o->jacobian, o->detj, o->pinv, o->normals, o->facet_normals};
  for (int i = 0; i < 6; ++i) a.out[i] = outs[i];
  a.err = t->err;
  a.recomputed = t->dtype == TLG_SPLIT32 ? o->recomputed : nullptr;
  a.first_cell = o->first_cell;
  a.padded = (o->num_cells + o->tile - 1) / o->tile * o->tile;
  a.range_cells = o->num_cells;
  a.out_first_cell = o->out_first_cell;
  a.last_cell = b->num_cells - 1;
  const int64_t nflags = b->flags ? std::min<int64_t>(b->num_cells, b->num_flags) : 0;
  a.last_flag = nflags - 1;
  for (int g = 0; g < 3; ++g) a.origin[g] = b->origin[g];
  a.cond_limit = o->cond_limit > 0 ? (float)o->cond_limit : 256.0f;
  a.last_node = (uint32_t)(b->num_nodes - 1);
  // Only phi, dphi and the reference normals are staged (the FP64 recompute's table stays in
  // global memory), and only up to a third of the shared memory, so that three CTAs fit an SM.
  const size_t es = t->dtype == TLG_F64 ? 8 : 4;
  const size_t prefix = (t->off_refn + (size_t)t->q * t->td * es + 15) / 16 * 16;
  const bool stage = prefix <= (size_t)75 * 1024;
  a.tab_bytes = stage ? (uint32_t)prefix : 0;
  a.off_dphi = t->off_dphi;
  a.off_refn = t->off_refn;
  a.off_dphi64 = t->off_dphi64;
  a.mask = mask;
  a.num_points = (int)t->q;
  a.k = (int)t->k;
  a.tile_shift = tile_shift(o->tile);
  a.tab_global = stage ? 0 : 1;
  cudaError_t e = tlg::launch_coop(t->dtype, t->td, t->gd, (int)t->k, a, stage ? prefix : 0, stream, found);
  if (!*found) return TLG_ERR_UNSUPPORTED;
  if (e != cudaSuccess) return cuda_fail(e, "tlg_eval_block launch");
  g_last_family = TLG_STRATEGY_COOPERATIVE;
  return ok();
}

}  // namespace

namespace tlg {

bool check_strategy(int family) {
  int s = 0;
  return wanted_strategy(family, &s);
}

void record_launch(int family, int strategy) {
  g_last_kind = family;
  g_last_family = strategy;
}

}  // namespace tlg

// The double-float monomial form of a tetrahedron's tables (P1-P3): the monomials x^a, |a| <= p,
// the expansion C = V^-1 of the Lagrange functions in them (V[j][m] = x_j^(a_m) at the Lagrange
// points, Gauss-Jordan with partial pivoting), checked against the tabulation at every point
// (values and derivatives within 1e-11); on success the double-float rows are overwritten with the
// monomials' (the same layout: per point pair and monomial, x^a and its derivatives as heads and
// tails of both points) and the expansion and direction masks written at off_dfmono.
void df_monomial_form(tlg_tables* t, const double* points, int64_t npoints, const std::vector<double>& phi,
                      const std::vector<double>& dphi) {
  const int k = (int)t->k, td = t->td, p = t->degree;
  std::vector<std::array<int, 3>> al;
  for (int s = 0; s <= p; ++s)
    for (int a = s; a >= 0; --a)
      for (int b = s - a; b >= 0; --b) al.push_back({a, b, s - a - b});
  if ((int)al.size() != k || td != 3) return;
  auto mono = [&](const double* x, int m) {
    double v = 1.0;
    for (int d = 0; d < 3; ++d)
      for (int e = 0; e < al[m][d]; ++e) v *= x[d];
    return v;
  };
  auto dmono = [&](const double* x, int m, int d) {
    if (al[m][d] == 0) return 0.0;
    double v = (double)al[m][d];
    for (int e = 0; e < 3; ++e)
      for (int i = 0; i < al[m][e] - (e == d ? 1 : 0); ++i) v *= x[e];
    return v;
  };
  const std::vector<double> lp = tlg::lagrange_points(t->cell, p, t->family);
  // [V | I] -> [I | V^-1]
  std::vector<double> a((size_t)k * 2 * k, 0.0);
  for (int j = 0; j < k; ++j) {
    for (int m = 0; m < k; ++m) a[(size_t)j * 2 * k + m] = mono(&lp[(size_t)j * 3], m);
    a[(size_t)j * 2 * k + k + j] = 1.0;
  }
  for (int c = 0; c < k; ++c) {
    int piv = c;
    for (int r = c + 1; r < k; ++r)
      if (std::fabs(a[(size_t)r * 2 * k + c]) > std::fabs(a[(size_t)piv * 2 * k + c])) piv = r;
    if (std::fabs(a[(size_t)piv * 2 * k + c]) < 1e-12) return;
    if (piv != c)
      for (int e = 0; e < 2 * k; ++e) std::swap(a[(size_t)piv * 2 * k + e], a[(size_t)c * 2 * k + e]);
    const double inv = 1.0 / a[(size_t)c * 2 * k + c];
    for (int e = 0; e < 2 * k; ++e) a[(size_t)c * 2 * k + e] *= inv;
    for (int r = 0; r < k; ++r) {
      if (r == c) continue;
      const double f = a[(size_t)r * 2 * k + c];
      if (f != 0.0)
        for (int e = 0; e < 2 * k; ++e) a[(size_t)r * 2 * k + e] -= f * a[(size_t)c * 2 * k + e];
    }
  }
  // V C = I: C[m][kk] = (V^-1)[m][kk].
  std::vector<double> C((size_t)k * k);
  for (int m = 0; m < k; ++m)
    for (int kk = 0; kk < k; ++kk) {
      double v = a[(size_t)m * 2 * k + k + kk];
      if (std::fabs(v) < 1e-13) v = 0.0;
      C[(size_t)m * k + kk] = v;
    }
  double err = 0.0;
  for (int64_t q = 0; q < npoints; ++q)
    for (int kk = 0; kk < k; ++kk) {
      double v = 0.0, dv[3] = {0.0, 0.0, 0.0};
      for (int m = 0; m < k; ++m) {
        const double cm = C[(size_t)m * k + kk];
        v += cm * mono(points + q * 3, m);
        for (int d = 0; d < 3; ++d) dv[d] += cm * dmono(points + q * 3, m, d);
      }
      err = std::max(err, std::fabs(v - phi[(size_t)q * k + kk]));
      for (int d = 0; d < 3; ++d) err = std::max(err, std::fabs(dv[d] - dphi[((size_t)q * k + kk) * 3 + d]));
    }
  if (!(err <= 1e-11)) return;
  const int64_t qp = (npoints + 1) / 2;
  float* rows = reinterpret_cast<float*>(t->host.data() + t->off_dfrows);
  for (int64_t pp = 0; pp < qp; ++pp)
    for (int m = 0; m < k; ++m)
      for (int r = 0; r <= td; ++r)
        for (int h = 0; h < 2; ++h) {
          const int64_t q = std::min<int64_t>(2 * pp + h, npoints - 1);
          const double v = r == 0 ? mono(points + q * 3, m) : dmono(points + q * 3, m, r - 1);
          float* e = rows + ((pp * k + m) * (1 + td) + r) * 4;
          e[h] = (float)v;
          e[2 + h] = (float)(v - (double)(float)v);
        }
  float* coef = reinterpret_cast<float*>(t->host.data() + t->off_dfmono);
  for (int kk = 0; kk < k; ++kk)
    for (int m = 0; m < k; ++m) {
      const double v = C[(size_t)m * k + kk];
      coef[((size_t)kk * k + m) * 2] = (float)v;
      coef[((size_t)kk * k + m) * 2 + 1] = (float)(v - (double)(float)v);
    }
  uint32_t* mask = reinterpret_cast<uint32_t*>(t->host.data() + t->off_dfmono + (size_t)k * k * 8);
  for (int m = 0; m < k; ++m) {
    uint32_t bits = 0;
    for (int d = 0; d < 3; ++d)
      if (al[m][d] > 0) bits |= 1u << d;
    mask[m] = bits;
  }
  t->df_mono = true;
}

extern "C" {

const char* tlg_last_error(void) { return g_error.c_str(); }

int tlg_abi_version(void) { return TLG_ABI_VERSION; }

int64_t tlg_num_lagrange_nodes(int cell, int degree) {
  if (!tlg::valid_cell(cell) || degree < 0) return -1;
  return tlg::num_lagrange_nodes(cell, degree);
}

tlg_status tlg_lagrange_points(int cell, int degree, int family, double* out, int64_t cap) {
  return guarded([&] {
    if (!out) return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_lagrange_points: out is NULL");
    const std::vector<double> p = tlg::lagrange_points(cell, degree, family);
    if ((int64_t)p.size() > cap)
      return fail(TLG_ERR_LENGTH_MISMATCH, "tlg_lagrange_points: capacity " + std::to_string(cap) +
                                               " below " + std::to_string(p.size()));
    std::memcpy(out, p.data(), p.size() * sizeof(double));
    return ok();
  });
}

tlg_status tlg_collapsed_rule(int cell, const int* counts, double* points, double* weights,
                              int64_t cap_points, int64_t* num_points) {
  return guarded([&] {
    if (!counts || !points || !weights || !num_points)
      return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_collapsed_rule: NULL argument");
    const int td = tlg::tdim(cell);
    for (int d = 0; d < td; ++d)
      if (counts[d] < 1 || counts[d] > 64)
        return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_collapsed_rule: point counts must be 1..64");
    std::vector<double> p, w;
    tlg::collapsed_rule(cell, counts, p, w);
    if ((int64_t)w.size() > cap_points)
      return fail(TLG_ERR_LENGTH_MISMATCH, "tlg_collapsed_rule: capacity below the point count");
    std::memcpy(points, p.data(), p.size() * sizeof(double));
    std::memcpy(weights, w.data(), w.size() * sizeof(double));
    *num_points = (int64_t)w.size();
    return ok();
  });
}

tlg_status tlg_tabulate(int cell, int degree, int family, const double* points, int64_t npoints,
                        int nderivs, double* out, int64_t cap) {
  return guarded([&] {
    if ((!points && npoints > 0) || !out || npoints < 0)
      return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_tabulate: bad points or output");
    const std::vector<double> t = tlg::tabulate(cell, degree, family, points, (long)npoints, nderivs);
    if ((int64_t)t.size() > cap) return fail(TLG_ERR_LENGTH_MISMATCH, "tlg_tabulate: capacity too small");
    std::memcpy(out, t.data(), t.size() * sizeof(double));
    return ok();
  });
}

tlg_status tlg_reference_facet_normals(int cell, double* out, int64_t cap) {
  return guarded([&] {
    if (!out) return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_reference_facet_normals: out is NULL");
    const std::vector<double> n = tlg::reference_facet_normals(cell);
    if ((int64_t)n.size() > cap) return fail(TLG_ERR_LENGTH_MISMATCH, "capacity too small");
    std::memcpy(out, n.data(), n.size() * sizeof(double));
    return ok();
  });
}

namespace {

// 1D Lagrange basis at the sorted nodes s: l_i(x) and l_i'(x).
void lagrange_1d(const std::vector<double>& s, double x, double* val, double* der) {
  const int n = (int)s.size();
  for (int i = 0; i < n; ++i) {
    double v = 1.0, d = 0.0;
    for (int r = 0; r < n; ++r) {
      if (r == i) continue;
      const double w = 1.0 / (s[i] - s[r]);
      d = d * (x - s[r]) * w + v * w;
      v *= (x - s[r]) * w;
    }
    val[i] = v;
    der[i] = d;
  }
}

// Sum factorisation over tensor blocks. A point set is cut, in order, into maximal blocks whose
// points are a tensor product: on quadrilaterals and hexahedra up to one 1D point set per
// direction (point q = o + a s_0 + b s_1 + c s_2, a direction of one point keeps its coordinate),
// on prisms a set of (x, y) points times a set of z points. A Gauss rule is one block; a facet
// rule one block per facet (or fewer, where facets line up). Per block the tables B_d = l(u_d),
// D_d = l'(u_d) (prisms: the triangle's psi, d_x psi, d_y psi and the interval's l, l'), checked
// against the element's full tabulation before use.
struct SfBlockHost {
  int64_t o = 0;
  int m[3] = {1, 1, 1};
  int64_t s[3] = {0, 0, 0};
  std::vector<double> B[3], D[3];
};

// Point sets of more blocks than this, or of fewer than two points per block on average, are not
// taken as tensor point sets.
constexpr int kMaxSfBlocks = 16;

// The largest tensor block of a quadrilateral or hexahedron point set starting at q0: directions
// are added fastest first, each while the points repeat the block so far with one more coordinate
// varying. Sets o, m, s and the 1D coordinates u; returns the block's point count.
int64_t next_tensor_block(const double* pts, int64_t nq, int td, int64_t q0, SfBlockHost& b,
                          std::vector<double>* u) {
  auto P = [&](int64_t q, int d) { return pts[q * td + d]; };
  b.o = q0;
  for (int d = 0; d < 3; ++d) {
    b.m[d] = 1;
    b.s[d] = 0;
    u[d].assign(1, d < td ? P(q0, d) : 0.0);
  }
  bool used[3] = {false, false, false};
  int64_t size = 1;
  for (int level = 0; level < td; ++level) {
    const int64_t q1 = q0 + size;
    if (q1 >= nq) break;
    int dir = -1, ndiff = 0;
    for (int e = 0; e < td; ++e)
      if (P(q1, e) != P(q0, e)) {
        dir = e;
        ++ndiff;
      }
    if (ndiff != 1 || used[dir]) break;
    // Copies j = 1, 2, ... of the block so far, each with its own value of `dir`.
    std::vector<double> vals(1, P(q0, dir));
    int64_t m = 1;
    while (q0 + (m + 1) * size <= nq) {
      const int64_t base = q0 + m * size;
      const double v = P(base, dir);
      bool ok = std::find(vals.begin(), vals.end(), v) == vals.end();
      for (int64_t r = 0; ok && r < size; ++r)
        for (int e = 0; ok && e < td; ++e)
          ok = e == dir ? P(base + r, e) == v : P(base + r, e) == P(q0 + r, e);
      if (!ok) break;
      vals.push_back(v);
      ++m;
    }
    if (m < 2) break;
    used[dir] = true;
    b.m[dir] = (int)m;
    b.s[dir] = size;
    u[dir] = vals;
    size *= m;
  }
  return size;
}

// The largest prism block starting at q0: (x, y) points times z points, z the slowest or the
// fastest index (the larger block of the two).
int64_t next_prism_block(const double* pts, int64_t nq, int64_t q0, SfBlockHost& b, std::vector<double>& tri,
                         std::vector<double>& zs) {
  auto X = [&](int64_t q) { return pts[q * 3]; };
  auto Y = [&](int64_t q) { return pts[q * 3 + 1]; };
  auto Z = [&](int64_t q) { return pts[q * 3 + 2]; };
  // z slowest: groups of mt points with one z each, repeating the (x, y) of the first group.
  int64_t mt = 1;
  while (q0 + mt < nq && Z(q0 + mt) == Z(q0)) ++mt;
  int64_t mz = 1;
  std::vector<double> zsl(1, Z(q0));
  while (q0 + (mz + 1) * mt <= nq) {
    const int64_t base = q0 + mz * mt;
    const double z = Z(base);
    bool ok = std::find(zsl.begin(), zsl.end(), z) == zsl.end();
    for (int64_t i = 0; ok && i < mt; ++i)
      ok = Z(base + i) == z && X(base + i) == X(q0 + i) && Y(base + i) == Y(q0 + i);
    if (!ok) break;
    zsl.push_back(z);
    ++mz;
  }
  // z fastest: groups of mz2 points with one (x, y) each, repeating the z of the first group.
  int64_t mz2 = 1;
  while (q0 + mz2 < nq && X(q0 + mz2) == X(q0) && Y(q0 + mz2) == Y(q0)) ++mz2;
  int64_t mt2 = 1;
  while (q0 + (mt2 + 1) * mz2 <= nq) {
    const int64_t base = q0 + mt2 * mz2;
    bool ok = true;
    for (int64_t j = 0; ok && j < mz2; ++j)
      ok = X(base + j) == X(base) && Y(base + j) == Y(base) && Z(base + j) == Z(q0 + j);
    for (int64_t i = 0; ok && i < mt2; ++i)  // a new (x, y)
      ok = !(X(q0 + i * mz2) == X(base) && Y(q0 + i * mz2) == Y(base));
    if (!ok) break;
    ++mt2;
  }
  b.o = q0;
  b.m[1] = 1;
  b.s[1] = 0;
  if (mt * mz >= mt2 * mz2) {
    b.m[0] = (int)mt;
    b.m[2] = (int)mz;
    b.s[0] = 1;
    b.s[2] = mt;
    tri.resize((size_t)mt * 2);
    for (int64_t i = 0; i < mt; ++i) {
      tri[(size_t)(2 * i)] = X(q0 + i);
      tri[(size_t)(2 * i + 1)] = Y(q0 + i);
    }
    zs = zsl;
    return mt * mz;
  }
  b.m[0] = (int)mt2;
  b.m[2] = (int)mz2;
  b.s[0] = mz2;
  b.s[2] = 1;
  tri.resize((size_t)mt2 * 2);
  for (int64_t i = 0; i < mt2; ++i) {
    tri[(size_t)(2 * i)] = X(q0 + i * mz2);
    tri[(size_t)(2 * i + 1)] = Y(q0 + i * mz2);
  }
  zs.resize((size_t)mz2);
  for (int64_t j = 0; j < mz2; ++j) zs[(size_t)j] = Z(q0 + j);
  return mt2 * mz2;
}

// The node permutation of a quadrilateral or hexahedron (lexicographic index over the sorted 1D
// nodes -> Lagrange node) or of a prism (index c NT + t over the interval's sorted nodes and the
// triangle's nodes -> Lagrange node); false when the nodes are not such a lattice.
bool sf_permutation(int cell, int degree, int family, std::vector<double>& s1, std::vector<double>& lt,
                    std::vector<uint32_t>& perm) {
  const int td = tlg::tdim(cell);
  const int n = degree + 1;
  std::vector<double> lp;
  try {
    s1 = tlg::lagrange_points(tlg::kInterval, degree, family);
    lp = tlg::lagrange_points(cell, degree, family);
    if (cell == tlg::kPrism) lt = tlg::lagrange_points(tlg::kTriangle, degree, family);
  } catch (const std::exception&) {
    return false;
  }
  std::sort(s1.begin(), s1.end());
  if ((int)s1.size() != n) return false;
  const int64_t k = tlg::num_lagrange_nodes(cell, degree);
  if ((int64_t)lp.size() != k * td) return false;
  perm.assign((size_t)k, 0xFFFFFFFFu);
  auto find1 = [&](double v) {
    int found = -1;
    for (int i = 0; i < n; ++i)
      if (std::fabs(v - s1[i]) < 1e-12) found = i;
    return found;
  };
  for (int64_t kk = 0; kk < k; ++kk) {
    int64_t l = 0;
    if (cell == tlg::kPrism) {
      const int nt = n * (n + 1) / 2;
      if ((int)lt.size() != nt * 2 || k != (int64_t)nt * n) return false;
      int ft = -1;
      for (int t = 0; t < nt; ++t)
        if (std::fabs(lp[kk * 3] - lt[t * 2]) < 1e-12 && std::fabs(lp[kk * 3 + 1] - lt[t * 2 + 1]) < 1e-12) ft = t;
      const int fc = find1(lp[kk * 3 + 2]);
      if (ft < 0 || fc < 0) return false;
      l = (int64_t)fc * nt + ft;
    } else {
      int64_t scale = 1;
      for (int d = 0; d < td; ++d) {
        const int f = find1(lp[kk * td + d]);
        if (f < 0) return false;
        l += f * scale;
        scale *= n;
      }
    }
    if (perm[(size_t)l] != 0xFFFFFFFFu) return false;
    perm[(size_t)l] = (uint32_t)kk;
  }
  return true;
}

// The tensor blocks of `points` for a quadrilateral, hexahedron or prism, with their tables and
// the permutation; false when the point set is not a tensor point set or a table product misses
// the full tabulation `tab` ([deriv][q][k]) by more than 1e-10.
bool sf_blocks(int cell, int degree, int family, const double* pts, int64_t nq, const std::vector<double>& tab,
               std::vector<SfBlockHost>& blocks, std::vector<uint32_t>& perm) {
  const int td = tlg::tdim(cell);
  const int n = degree + 1;
  const int64_t k = tlg::num_lagrange_nodes(cell, degree);
  std::vector<double> s1, lt;
  if (nq < 1 || !sf_permutation(cell, degree, family, s1, lt, perm)) return false;
  blocks.clear();
  for (int64_t q0 = 0; q0 < nq;) {
    if ((int)blocks.size() >= kMaxSfBlocks) return false;
    SfBlockHost b;
    int64_t size = 0;
    if (cell == tlg::kPrism) {
      std::vector<double> tri, zs;
      size = next_prism_block(pts, nq, q0, b, tri, zs);
      const int nt = n * (n + 1) / 2;
      std::vector<double> tt;
      try {
        tt = tlg::tabulate(tlg::kTriangle, degree, family, tri.data(), (long)b.m[0], 1);
      } catch (const std::exception&) {
        return false;
      }
      const int mt = b.m[0];
      b.B[0].assign((size_t)mt * nt, 0.0);
      b.D[0].assign((size_t)mt * nt, 0.0);
      b.D[1].assign((size_t)mt * nt, 0.0);
      for (int i = 0; i < mt; ++i)
        for (int t = 0; t < nt; ++t) {
          b.B[0][(size_t)(i * nt + t)] = tt[(size_t)(i * nt + t)];
          b.D[0][(size_t)(i * nt + t)] = tt[(size_t)((mt + i) * nt + t)];
          b.D[1][(size_t)(i * nt + t)] = tt[(size_t)((2 * mt + i) * nt + t)];
        }
      b.B[2].assign((size_t)b.m[2] * n, 0.0);
      b.D[2].assign((size_t)b.m[2] * n, 0.0);
      for (int j = 0; j < b.m[2]; ++j)
        lagrange_1d(s1, zs[(size_t)j], &b.B[2][(size_t)(j * n)], &b.D[2][(size_t)(j * n)]);
      // Identity: psi_t(i) l_c(z_j) and its derivatives against the prism's tabulation.
      for (int i = 0; i < mt; ++i)
        for (int j = 0; j < b.m[2]; ++j) {
          const int64_t q = b.o + i * b.s[0] + j * b.s[2];
          for (int c = 0; c < n; ++c)
            for (int t = 0; t < nt; ++t) {
              const int64_t kk = perm[(size_t)(c * nt + t)];
              const double l = b.B[2][(size_t)(j * n + c)], ld = b.D[2][(size_t)(j * n + c)];
              const double want[4] = {b.B[0][(size_t)(i * nt + t)] * l, b.D[0][(size_t)(i * nt + t)] * l,
                                      b.D[1][(size_t)(i * nt + t)] * l, b.B[0][(size_t)(i * nt + t)] * ld};
              for (int r = 0; r < 4; ++r) {
                const double got = tab[(size_t)((r * nq + q) * k + kk)];
                if (!(std::fabs(got - want[r]) <= 1e-10 * std::max(1.0, std::fabs(got)))) return false;
              }
            }
        }
    } else {
      std::vector<double> u[3];
      size = next_tensor_block(pts, nq, td, q0, b, u);
      for (int d = 0; d < td; ++d) {
        b.B[d].assign((size_t)b.m[d] * n, 0.0);
        b.D[d].assign((size_t)b.m[d] * n, 0.0);
        for (int a = 0; a < b.m[d]; ++a)
          lagrange_1d(s1, u[d][(size_t)a], &b.B[d][(size_t)(a * n)], &b.D[d][(size_t)(a * n)]);
      }
      // Identity: prod_d l_{i_d}(u_d) and its derivatives against the tabulation.
      const int m2 = td == 3 ? b.m[2] : 1;
      for (int c2 = 0; c2 < m2; ++c2)
        for (int b1 = 0; b1 < b.m[1]; ++b1)
          for (int a0 = 0; a0 < b.m[0]; ++a0) {
            const int64_t q = b.o + a0 * b.s[0] + b1 * b.s[1] + c2 * b.s[2];
            const int pt[3] = {a0, b1, c2};
            for (int64_t l = 0; l < k; ++l) {
              int64_t rest = l;
              int idx[3] = {0, 0, 0};
              for (int d = 0; d < td; ++d) {
                idx[d] = (int)(rest % n);
                rest /= n;
              }
              const int64_t kk = perm[(size_t)l];
              for (int r = 0; r <= td; ++r) {
                double want = 1.0;
                for (int d = 0; d < td; ++d) {
                  const std::vector<double>& T = (r == d + 1) ? b.D[d] : b.B[d];
                  want *= T[(size_t)(pt[d] * n + idx[d])];
                }
                const double got = tab[(size_t)((r * nq + q) * k + kk)];
                if (!(std::fabs(got - want) <= 1e-10 * std::max(1.0, std::fabs(got)))) return false;
              }
            }
          }
    }
    blocks.push_back(std::move(b));
    q0 += size;
  }
  return nq >= 2 * (int64_t)blocks.size();
}

}  // namespace

tlg_status tlg_tables_create(int cell, int degree, int family, int gdim, int dtype,
                             const double* points, int64_t npoints, const double* ref_normals,
                             tlg_tables** out) {
  return guarded([&]() -> tlg_status {
    if (!out) return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_tables_create: out is NULL");
    *out = nullptr;
    if (!tlg::valid_cell(cell) || cell == tlg::kPoint)
      return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_tables_create: no cell type " + std::to_string(cell));
    const int td = tlg::tdim(cell);
    if (gdim < td || gdim > 3)
      return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_tables_create: gdim " + std::to_string(gdim) +
                                                " with tdim " + std::to_string(td));
    if (dtype != TLG_F32 && dtype != TLG_F64 && dtype != TLG_SPLIT32 && dtype != TLG_DF64)
      return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_tables_create: dtype must be 4, 8, 12 or 16");
    const bool df = dtype == TLG_DF64;
    if (df) dtype = TLG_F64;  // every f64 section, then the double-float ones
    if (degree < 1) return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_tables_create: degree must be >= 1");
    if (npoints < 0 || (npoints > 0 && !points))
      return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_tables_create: bad points");
    const int64_t k = tlg::num_lagrange_nodes(cell, degree);
    if (k > 1024) return fail(TLG_ERR_UNSUPPORTED, "tlg_tables_create: more than 1024 nodes per cell");
    std::vector<double> tab = tlg::tabulate(cell, degree, family, points, (long)npoints, 1);
    auto t = new tlg_tables();
    t->cell = cell;
    t->degree = degree;
    t->family = family;
    t->td = td;
    t->gd = gdim;
    t->dtype = dtype;
    t->df = df;
    t->k = k;
    t->q = npoints;
    t->has_refn = ref_normals != nullptr;
    const size_t es = dtype == TLG_SPLIT32 ? 4 : (size_t)dtype;
    const size_t n_phi = (size_t)npoints * k, n_dphi = n_phi * td, n_refn = (size_t)npoints * td;
    t->off_dphi = align16(n_phi * es);
    t->off_refn = align16(t->off_dphi + n_dphi * es);
    size_t total = align16(t->off_refn + std::max<size_t>(n_refn, 1) * es);
    // Point pairs for the paired-FP32 kernels: rows2 [QP][K][RW] f32, per node of a point pair
    // phi, dphi_0 .. dphi_{TD-1} as (point 2p, point 2p + 1) pairs, zero padded to RW = 8 (TD > 1)
    // or 4 (TD = 1) floats, so that a node's row is one or two 16-byte shared loads; an odd last
    // point is paired with itself.
    const int64_t qp = (npoints + 1) / 2;
    const int rw = td == 1 ? 4 : 8;
    if (dtype != TLG_F64) {
      t->off_rows2 = (uint32_t)total;
      total = align16(total + std::max<size_t>((size_t)qp * k * rw, 1) * 4);
    }
    if (dtype == TLG_SPLIT32) {  // the f64 derivative table of the FP64 recompute follows
      t->off_dphi64 = (uint32_t)total;
      total = align16(total + std::max<size_t>(n_dphi, 1) * 8);
    }
    if (df && k <= 30 && npoints > 0) {  // the double-float rows of the paired f64 kernels
      t->off_dfrows = (uint32_t)total;
      t->dfrows_bytes = (uint32_t)((size_t)qp * k * (1 + td) * 16);
      total = align16(total + t->dfrows_bytes);
      if (cell == tlg::kTetrahedron && gdim == 3 && (k == 4 || k == 10 || k == 20)) {
        t->off_dfmono = (uint32_t)total;
        total = align16(total + (size_t)k * k * 8 + (size_t)k * 4);
      }
    }
    // Tables beyond the shared-memory budget stay in global memory: the loops kernels read them
    // there (L1/L2-cached) instead of staging them.
    if (total > ((size_t)1 << 31)) {
      delete t;
      return fail(TLG_ERR_ALLOCATION_TOO_LARGE,
                  "tlg_tables_create: the tabulation (" + std::to_string(total) + " bytes) exceeds 2 GiB");
    }
    t->staged = total + 16 <= (size_t)200 * 1024;
    t->bytes = (uint32_t)total;
    t->off_vjp = (uint32_t)(total + 16);
    if (td == gdim && dtype != TLG_F32) {
      const size_t vb = (size_t)(dtype == TLG_SPLIT32 ? qp : npoints) * k * 32;
      if (vb > 0 && vb <= (size_t)160 * 1024) t->vjp_bytes = (uint32_t)vb;
    }
    std::vector<SfBlockHost> sf;
    std::vector<uint32_t> sf_perm;
    if (((cell == tlg::kQuadrilateral || cell == tlg::kHexahedron) && degree + 1 <= 6) ||
        (cell == tlg::kPrism && degree <= 3 && gdim == 3)) {
      t->sf_ok = sf_blocks(cell, degree, family, points, npoints, tab, sf, sf_perm);
      t->sf_prism = t->sf_ok && cell == tlg::kPrism;
    }
    t->off_sf = (uint32_t)align16(t->off_vjp + t->vjp_bytes);
    std::vector<tlg::SfBlock> heads, dfheads;
    if (t->sf_ok) {
      t->sf_n = degree + 1;
      t->sf_nblocks = (int)sf.size();
      size_t off = align16(sf.size() * sizeof(tlg::SfBlock));
      heads.resize(sf.size());
      for (size_t bi = 0; bi < sf.size(); ++bi) {
        tlg::SfBlock& h = heads[bi];
        std::memset(&h, 0, sizeof(h));
        h.o = (int)sf[bi].o;
        for (int d = 0; d < 3; ++d) {
          h.m[d] = sf[bi].m[d];
          h.s[d] = (int)sf[bi].s[d];
          h.off_b[d] = (uint32_t)off;
          off = align16(off + sf[bi].B[d].size() * es);
          h.off_d[d] = (uint32_t)off;
          off = align16(off + sf[bi].D[d].size() * es);
        }
      }
      t->sf_block0 = heads[0];
      t->sf_offperm = (uint32_t)off;
      off = align16(off + sf_perm.size() * 4);
      t->sf_offrefn = (uint32_t)off;
      if (ref_normals) off = align16(off + (size_t)npoints * td * es);
      t->sf_bytes = (uint32_t)off;
      if (df) {
        dfheads = heads;
        size_t doff = align16(sf.size() * sizeof(tlg::SfBlock));
        const int pd = t->sf_prism ? 2 : 0;
        for (size_t bi = 0; bi < sf.size(); ++bi)
          for (int d = 0; d < 3; ++d) {
            const int m = sf[bi].m[d];
            auto bytes = [&](const std::vector<double>& v) {
              const size_t cols = m > 0 ? v.size() / m : 0;
              return d == pd ? (size_t)((m + 1) / 2) * cols * 16 : v.size() * 8;
            };
            dfheads[bi].off_b[d] = (uint32_t)doff;
            doff = align16(doff + bytes(sf[bi].B[d]));
            dfheads[bi].off_d[d] = (uint32_t)doff;
            doff = align16(doff + bytes(sf[bi].D[d]));
          }
        t->sfdf_offperm = (uint32_t)doff;
        doff = align16(doff + sf_perm.size() * 4);
        t->sfdf_offrefn = (uint32_t)doff;
        if (ref_normals) doff = align16(doff + (size_t)npoints * td * 8);
        t->sfdf_bytes = (uint32_t)doff;
        t->off_sfdf = (uint32_t)align16((size_t)t->off_sf + t->sf_bytes);
      }
    }
    // The tensor-core section.
    size_t host_bytes = t->off_sfdf ? (size_t)t->off_sfdf + t->sfdf_bytes : (size_t)t->off_sf + t->sf_bytes;
    if (dtype != TLG_F64 && td >= 2 && k > 10 && npoints > 0) {
      t->tc_ksteps = (int)((k + 7) / 8);
      t->tc_col_tiles = (int)((npoints + 1) / 2);
      t->off_tc = align16(host_bytes);
      host_bytes = t->off_tc + (size_t)t->tc_col_tiles * t->tc_ksteps * 32 * 16;
    }
    if (dtype != TLG_F64 && td == 3 && gdim == 3 && k > 20 && (k + 7) / 8 * 8 <= tlg::kUmmaMaxKpad &&
        npoints > 0) {
      t->umma_kpad = (int)((k + 7) / 8 * 8);
      t->umma_chunks = (int)((npoints + tlg::kUmmaPoints - 1) / tlg::kUmmaPoints);
      t->off_umma = align16(host_bytes);
      // Zero chunks after the last, for work items whose last group runs past it.
      host_bytes = t->off_umma + (size_t)(t->umma_chunks + tlg::kUmmaMaxGroups - 1) * 2 * tlg::kUmmaN * t->umma_kpad * 4;
    }
    t->host.assign(host_bytes, 0);
    if (t->sf_ok) {
      std::memcpy(t->host.data() + t->off_sf, heads.data(), heads.size() * sizeof(tlg::SfBlock));
      for (size_t bi = 0; bi < sf.size(); ++bi)
        for (int d = 0; d < 3; ++d) {
          const size_t ob = t->off_sf + heads[bi].off_b[d], od = t->off_sf + heads[bi].off_d[d];
          if (dtype == TLG_F64) {
            narrow_into<double>(t->host, ob, sf[bi].B[d].data(), sf[bi].B[d].size());
            narrow_into<double>(t->host, od, sf[bi].D[d].data(), sf[bi].D[d].size());
          } else {
            narrow_into<float>(t->host, ob, sf[bi].B[d].data(), sf[bi].B[d].size());
            narrow_into<float>(t->host, od, sf[bi].D[d].data(), sf[bi].D[d].size());
          }
        }
      std::memcpy(t->host.data() + t->off_sf + t->sf_offperm, sf_perm.data(), sf_perm.size() * 4);
      if (ref_normals) {
        if (dtype == TLG_F64) narrow_into<double>(t->host, t->off_sf + t->sf_offrefn, ref_normals, (size_t)npoints * td);
        else narrow_into<float>(t->host, t->off_sf + t->sf_offrefn, ref_normals, (size_t)npoints * td);
      }
      if (t->off_sfdf) {  // the double-float section
        unsigned char* base = t->host.data() + t->off_sfdf;
        std::memcpy(base, dfheads.data(), dfheads.size() * sizeof(tlg::SfBlock));
        const int pd = t->sf_prism ? 2 : 0;
        for (size_t bi = 0; bi < sf.size(); ++bi)
          for (int d = 0; d < 3; ++d) {
            const int m = sf[bi].m[d];
            auto write = [&](uint32_t off, const std::vector<double>& v) {
              if (d != pd) {
                split_into(t->host, t->off_sfdf + off, v.data(), v.size());
                return;
              }
              const int cols = m > 0 ? (int)(v.size() / m) : 0;
              float* dst = reinterpret_cast<float*>(base + off);
              for (int pp = 0; pp < (m + 1) / 2; ++pp)
                for (int c = 0; c < cols; ++c)
                  for (int hh = 0; hh < 2; ++hh) {
                    const double x = v[(size_t)std::min(2 * pp + hh, m - 1) * cols + c];
                    float* e = dst + ((size_t)pp * cols + c) * 4;
                    e[hh] = (float)x;
                    e[2 + hh] = (float)(x - (double)(float)x);
                  }
            };
            write(dfheads[bi].off_b[d], sf[bi].B[d]);
            write(dfheads[bi].off_d[d], sf[bi].D[d]);
          }
        std::memcpy(base + t->sfdf_offperm, sf_perm.data(), sf_perm.size() * 4);
        if (ref_normals) narrow_into<double>(t->host, t->off_sfdf + t->sfdf_offrefn, ref_normals, (size_t)npoints * td);
      }
    }
    // Reorder [deriv][q][k] into phi [q][k] and dphi [q][k][d].
    std::vector<double> phi(n_phi), dphi(n_dphi), refn(n_refn, 0.0);
    for (int64_t q = 0; q < npoints; ++q)
      for (int64_t i = 0; i < k; ++i) {
        phi[q * k + i] = tab[q * k + i];
        for (int d = 0; d < td; ++d) dphi[(q * k + i) * td + d] = tab[((1 + d) * npoints + q) * k + i];
      }
    if (ref_normals) std::memcpy(refn.data(), ref_normals, n_refn * sizeof(double));
    if (dtype == TLG_SPLIT32) narrow_into<double>(t->host, t->off_dphi64, dphi.data(), n_dphi);
    if (t->dfrows_bytes > 0) {
      float* dst = reinterpret_cast<float*>(t->host.data() + t->off_dfrows);
      for (int64_t p = 0; p < qp; ++p)
        for (int64_t i = 0; i < k; ++i)
          for (int r = 0; r <= td; ++r)
            for (int h = 0; h < 2; ++h) {
              const int64_t q = std::min<int64_t>(2 * p + h, npoints - 1);
              const double v = r == 0 ? phi[q * k + i] : dphi[(q * k + i) * td + (r - 1)];
              float* e = dst + ((p * k + i) * (1 + td) + r) * 4;
              e[h] = (float)v;
              e[2 + h] = (float)(v - (double)(float)v);
            }
    }
    if (t->off_dfmono) df_monomial_form(t, points, npoints, phi, dphi);
    if (dtype != TLG_F64) {
      std::vector<double> rows2((size_t)qp * k * rw, 0.0);
      for (int64_t p = 0; p < qp; ++p)
        for (int h = 0; h < 2; ++h) {
          const int64_t q = std::min<int64_t>(2 * p + h, npoints - 1);
          for (int64_t i = 0; i < k; ++i) {
            double* r = &rows2[(size_t)((p * k + i) * rw)];
            r[h] = phi[q * k + i];
            for (int d = 0; d < td; ++d) r[2 * (d + 1) + h] = dphi[(q * k + i) * td + d];
          }
        }
      narrow_into<float>(t->host, t->off_rows2, rows2.data(), rows2.size());
      if (t->tc_ksteps > 0) {
        // B[k][4 q + r] narrowed to f32, split into TF32 head (round to nearest, ties away) and
        // tail; lane = 4 grp + tig holds B[8 ks + tig][8 j + grp] and B[8 ks + tig + 4][8 j + grp].
        auto bval = [&](int64_t kk, int64_t col) -> float {
          const int64_t q = col / 4, r = col % 4;
          if (kk >= k || q >= npoints || r > td) return 0.0f;
          return (float)(r == 0 ? phi[q * k + kk] : dphi[(q * k + kk) * td + (r - 1)]);
        };
        auto head = [](float x) {
          uint32_t u;
          std::memcpy(&u, &x, 4);
          if ((u & 0x7F800000u) != 0x7F800000u) u = (u + 0x1000u) & 0xFFFFE000u;
          float h;
          std::memcpy(&h, &u, 4);
          return h;
        };
        if (t->umma_kpad > 0) {
          const int kp = t->umma_kpad;
          const size_t half = (size_t)tlg::kUmmaN * kp;  // floats
          float* ub = reinterpret_cast<float*>(t->host.data() + t->off_umma);
          for (int ch = 0; ch < t->umma_chunks; ++ch)
            for (int n = 0; n < tlg::kUmmaN; ++n)
              for (int kk = 0; kk < kp; ++kk) {
                const float v = bval(kk, (int64_t)ch * tlg::kUmmaN + n);
                const float h = head(v);
                const size_t off = (size_t)(n >> 3) * (kp * 8) + (size_t)(kk >> 2) * 32 + (n & 7) * 4 + (kk & 3);
                ub[ch * 2 * half + off] = h;
                ub[ch * 2 * half + half + off] = head(v - h);
              }
        }
        float* dst = reinterpret_cast<float*>(t->host.data() + t->off_tc);
        for (int j = 0; j < t->tc_col_tiles; ++j)
          for (int ks = 0; ks < t->tc_ksteps; ++ks)
            for (int lane = 0; lane < 32; ++lane) {
              const int grp = lane >> 2, tig = lane & 3;
              const float v0 = bval(8 * ks + tig, 8 * j + grp), v1 = bval(8 * ks + tig + 4, 8 * j + grp);
              const float h0 = head(v0), h1 = head(v1);
              float* e = dst + (((size_t)j * t->tc_ksteps + ks) * 32 + lane) * 4;
              e[0] = h0;
              e[1] = h1;
              e[2] = head(v0 - h0);
              e[3] = head(v1 - h1);
            }
      }
    }
    if (t->vjp_bytes > 0) {
      const int pn = dtype == TLG_SPLIT32 ? 2 : 1;  // points per table row
      const int64_t rows = dtype == TLG_SPLIT32 ? qp : npoints;
      std::vector<double> v((size_t)rows * k * 4 * pn, 0.0);
      for (int64_t r = 0; r < rows; ++r)
        for (int h = 0; h < pn; ++h) {
          const int64_t q = std::min<int64_t>(r * pn + h, npoints - 1);
          for (int64_t i = 0; i < k; ++i) {
            double* row = v.data() + (r * k + i) * 4 * pn;
            row[h] = phi[q * k + i];
            for (int d = 0; d < td; ++d) row[(1 + d) * pn + h] = dphi[(q * k + i) * td + d];
          }
        }
      if (dtype == TLG_SPLIT32) narrow_into<float>(t->host, t->off_vjp, v.data(), v.size());
      else narrow_into<double>(t->host, t->off_vjp, v.data(), v.size());
    }
    if (dtype != TLG_F64) {
      narrow_into<float>(t->host, 0, phi.data(), n_phi);
      narrow_into<float>(t->host, t->off_dphi, dphi.data(), n_dphi);
      narrow_into<float>(t->host, t->off_refn, refn.data(), n_refn);
    } else {
      narrow_into<double>(t->host, 0, phi.data(), n_phi);
      narrow_into<double>(t->host, t->off_dphi, dphi.data(), n_dphi);
      narrow_into<double>(t->host, t->off_refn, refn.data(), n_refn);
    }
    cudaError_t e = cudaMalloc(&t->dev, t->host.size());
    if (e != cudaSuccess) {
      delete t;
      return cuda_fail(e, "tlg_tables_create: cudaMalloc");
    }
    t->err = reinterpret_cast<int*>(t->dev + total);
    e = cudaMemcpy(t->dev, t->host.data(), t->host.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      cudaFree(t->dev);
      delete t;
      return cuda_fail(e, "tlg_tables_create: upload");
    }
    *out = t;
    return ok();
  });
}

tlg_status tlg_tables_destroy(tlg_tables* t) {
  if (!t) return ok();
  cudaError_t e = cudaFree(t->dev);
  delete t;
  if (e != cudaSuccess) return cuda_fail(e, "tlg_tables_destroy");
  return ok();
}

tlg_status tlg_tables_set_wait(tlg_tables* t, int64_t polls, int issue_copy) {
  if (!t || polls < 0 || polls > INT32_MAX || (issue_copy != 0 && issue_copy != 1))
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_tables_set_wait: NULL tables, polls outside 0 .. 2^31 - 1 or "
                                          "issue_copy not 0 or 1");
  const int words[2] = {(int)polls, issue_copy ? 0 : 1};
  cudaError_t e = cudaMemcpy(t->err + 1, words, sizeof(words), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "tlg_tables_set_wait");
  return ok();
}

int64_t tlg_tables_num_points(const tlg_tables* t) { return t ? t->q : -1; }

int64_t tlg_tables_nodes_per_cell(const tlg_tables* t) { return t ? t->k : -1; }

tlg_status tlg_tables_device_status(const tlg_tables* t, void* stream) {
  if (!t) return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_tables_device_status: NULL tables");
  int flag = 0;
  cudaError_t e = cudaMemcpyAsync(&flag, t->err, sizeof(int), cudaMemcpyDeviceToHost,
                                  static_cast<cudaStream_t>(stream));
  if (e == cudaSuccess) e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "tlg_tables_device_status");
  if (flag != 0) {
    cudaMemsetAsync(t->err, 0, sizeof(int), static_cast<cudaStream_t>(stream));
    return fail(TLG_ERR_DEVICE_TIMEOUT, "a bounded device wait expired in an evaluation kernel");
  }
  return ok();
}

}  // extern "C"

namespace {

// The strategy's kernel for one range (the reference's dispatch, strategy.rs:311-407).
tlg_status eval_dispatch(const tlg_tables* t, const tlg_block* b, const tlg_outputs* o, uint32_t mask,
                         cudaStream_t s) {
  const int family = principal_family(mask);
  int strategy = TLG_STRATEGY_AUTO;
  if (!wanted_strategy(family, &strategy)) return TLG_ERR_INVALID_ARGUMENT;
  g_last_kind = family;
  // A forced strategy that does not apply runs the loops kernel (strategy.rs:400-404); AUTO
  // falls through to the unrolled kernels, then the loops kernel over staged tables.
  const bool is_auto = strategy == TLG_STRATEGY_AUTO;
  if (strategy == TLG_STRATEGY_SUMFACT || (is_auto && sumfact_preferred(t))) {
    bool found = false;
    tlg_status st = eval_sumfact(t, b, o, mask, s, &found);
    if (found) return st;
  }
  if (strategy == TLG_STRATEGY_TENSOR || (is_auto && umma_preferred(t))) {
    bool found = false;
    tlg_status st = eval_umma(t, b, o, mask, s, &found);
    if (found) return st;
  }
  if (strategy == TLG_STRATEGY_TENSOR || (is_auto && tc_preferred(t))) {
    bool found = false;
    tlg_status st = eval_tc(t, b, o, mask, s, &found);
    if (found) return st;
  }
  if (strategy == TLG_STRATEGY_COOPERATIVE || (is_auto && coop_preferred(t))) {
    bool found = false;
    tlg_status st = eval_coop(t, b, o, mask, s, &found);
    if (found) return st;
  }
  const bool allow_direct = is_auto || strategy == TLG_STRATEGY_DIRECT;
  const bool global_tables = !(is_auto || strategy == TLG_STRATEGY_SHARED);
  if (t->df && allow_direct) {
    bool found = false;
    tlg_status st = eval_df(t, b, o, mask, s, &found);
    if (found) return st;
  }
  if (t->dtype == TLG_SPLIT32) return eval_split(t, b, o, mask, s, allow_direct, global_tables);
  if (t->dtype == TLG_F32) return eval_typed<float>(t, b, o, mask, s, allow_direct, global_tables);
  return eval_typed<double>(t, b, o, mask, s, allow_direct, global_tables);
}

}  // namespace

extern "C" {

tlg_status tlg_eval_block(const tlg_tables* t, const tlg_block* b, const tlg_outputs* o,
                          void* stream) {
  if (!t || !b || !o) return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_eval_block: NULL argument");
  if (b->dtype != (t->dtype == TLG_SPLIT32 ? TLG_F64 : t->dtype))
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_eval_block: block and tables differ in dtype");
  if (b->gdim != t->gd)
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_eval_block: block gdim " + std::to_string(b->gdim) +
                                              " but tables for gdim " + std::to_string(t->gd));
  if (tile_shift(o->tile) < 0)
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_eval_block: tile " + std::to_string(o->tile) +
                                              " is not 1, 2, 4, 8 or 16");
  if (o->first_cell < 0 || o->num_cells < 0 || o->out_first_cell < 0 ||
      o->first_cell + o->num_cells > b->num_cells)
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_eval_block: cell range outside the block");
  if (o->out_first_cell % o->tile != 0)
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_eval_block: out_first_cell is not a multiple of the tile");
  uint32_t mask = 0;
  if (o->points) mask |= tlg::kOutPoints;
  if (o->jacobian) mask |= tlg::kOutJacobian;
  if (o->detj) mask |= tlg::kOutDetJ;
  if (o->pinv) mask |= tlg::kOutPinv;
  if (o->normals) mask |= tlg::kOutNormals;
  if (o->facet_normals) mask |= tlg::kOutFacetNormals;
  if (o->normals && t->td + 1 != t->gd)
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_eval_block: normals need a block of codimension 1");
  if (o->facet_normals && (t->td != t->gd || !t->has_refn))
    return fail(TLG_ERR_INVALID_ARGUMENT,
                "tlg_eval_block: facet normals need codimension 0 and tables with reference normals");
  if (o->cell_measure && (!o->detj || !o->weights))
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_eval_block: cell_measure needs the det J output and weights");
  if (o->num_cells == 0 || t->q == 0 || mask == 0) return ok();  // layout.rs:509-511
  if (!b->nodes || !b->dofmap) return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_eval_block: NULL nodes or dofmap");
  if (b->num_nodes < 1)  // Geometry::new rejects cells without nodes (geometry.rs:268-275)
    return fail(TLG_ERR_LENGTH_MISMATCH, "tlg_eval_block: cells but no nodes");
  if (b->num_nodes > (int64_t)UINT32_MAX + 1 || b->num_cells > (int64_t)UINT32_MAX)
    return fail(TLG_ERR_TOO_LARGE, "tlg_eval_block: node or cell count does not fit u32");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  g_measure_fused = false;
  tlg_status st = eval_dispatch(t, b, o, mask, s);
  if (st != TLG_OK || !o->cell_measure || g_measure_fused) return st;
  // The kernel that ran does not sum the measure: per-cell sums over the det J it wrote (the
  // range starts at a tile boundary of the output, so its cells start a tile there).
  const int es = t->dtype == TLG_F64 ? 8 : 4;
  const unsigned char* detj = static_cast<const unsigned char*>(o->detj) + o->out_first_cell * t->q * es;
  return tlg_measure_cell_sums(detj, es, o->num_cells, t->q, o->tile, o->weights, o->cell_measure, stream);
}

tlg_status tlg_set_strategy(int strategy) {
  if (strategy < -1 || strategy > TLG_STRATEGY_TENSOR)
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_set_strategy: strategy must be -1 .. 6");
  for (int& x : g_override) x = strategy;
  return ok();
}

tlg_status tlg_set_family_strategy(int family, int strategy) {
  if (family < 0 || family >= kFamilies)
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_set_family_strategy: family must be 0 .. 5");
  if (strategy < -1 || strategy > TLG_STRATEGY_TENSOR)
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_set_family_strategy: strategy must be -1 .. 6");
  g_override[family] = strategy;
  return ok();
}

int tlg_get_family_override(int family) { return family >= 0 && family < kFamilies ? g_override[family] : -1; }

tlg_status tlg_get_family_strategy(int family, int* strategy) {
  if (family < 0 || family >= kFamilies || !strategy)
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_get_family_strategy: family must be 0 .. 5");
  if (!wanted_strategy(family, strategy)) return TLG_ERR_INVALID_ARGUMENT;
  return ok();
}

int tlg_get_strategy(void) {
  int s = TLG_STRATEGY_AUTO;
  return wanted_strategy(TLG_FAMILY_JACOBIAN, &s) ? s : -1;
}

int tlg_last_kernel_family(void) { return g_last_family; }

int tlg_last_launch_family(void) { return g_last_kind; }

tlg_status tlg_evector(const tlg_block* b, int nodes_per_cell, int64_t first_cell, int64_t chunk_cells,
                       int64_t stride, void* out, void* stream) {
  if (!b || !out) return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_evector: NULL argument");
  if (b->dtype != TLG_F32 && b->dtype != TLG_F64)
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_evector: dtype must be 4 or 8");
  if (nodes_per_cell < 1 || b->gdim < 1 || b->gdim > 3)
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_evector: bad nodes_per_cell or gdim");
  if (first_cell < 0 || chunk_cells < 0 || first_cell + chunk_cells > b->num_cells)
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_evector: chunk outside the block");
  const int64_t padded = (chunk_cells + 15) / 16 * 16;  // VECTOR_PAD
  if (stride < padded) return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_evector: stride below the padded chunk");
  if (chunk_cells == 0) return ok();
  if (!tlg::check_strategy(TLG_FAMILY_EVECTOR)) return TLG_ERR_INVALID_ARGUMENT;
  if (!b->nodes || !b->dofmap) return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_evector: NULL nodes or dofmap");
  if (b->num_nodes < 1) return fail(TLG_ERR_LENGTH_MISMATCH, "tlg_evector: cells but no nodes");
  if (b->num_nodes > (int64_t)UINT32_MAX + 1)
    return fail(TLG_ERR_TOO_LARGE, "tlg_evector: node count does not fit u32");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int threads = 256;
  int64_t blocks = (padded + threads - 1) / threads;
  if (blocks > 65535LL * 16) blocks = 65535LL * 16;
  const uint32_t last_node = (uint32_t)(b->num_nodes - 1);
  if (b->dtype == TLG_F32)
    tlg::evector_kernel<uint32_t><<<(unsigned)blocks, threads, 0, s>>>(
        static_cast<const uint32_t*>(b->nodes), b->dofmap, static_cast<uint32_t*>(out), first_cell,
        b->num_cells - 1, last_node, nodes_per_cell, b->gdim, padded, stride);
  else
    tlg::evector_kernel<uint64_t><<<(unsigned)blocks, threads, 0, s>>>(
        static_cast<const uint64_t*>(b->nodes), b->dofmap, static_cast<uint64_t*>(out), first_cell,
        b->num_cells - 1, last_node, nodes_per_cell, b->gdim, padded, stride);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "tlg_evector launch");
  tlg::record_launch(TLG_FAMILY_EVECTOR, TLG_STRATEGY_LOOPS);
  return ok();
}

namespace {

// Hexahedra with a tensor-product rule and 2 or 3 nodes per direction have the sum-factorised
// adjoint.
bool vjp_sumfact_preferred(const tlg_tables* t) {
  // One block in rule order (direction 0 fastest): the kernel walks the points in that order and
  // loads the cotangents of the points ahead of the current one.
  const tlg::SfBlock& h = t->sf_block0;
  return t->sf_ok && t->cell == tlg::kHexahedron && (t->sf_n == 2 || t->sf_n == 3) && t->sf_nblocks == 1 &&
         h.o == 0 && h.s[0] == 1 && h.s[1] == h.m[0] && h.s[2] == h.m[0] * h.m[1];
}

// The sum-factorised adjoint from the arguments of the node-row kernel; `found` is false when
// the element has none (then the node-row kernel runs).
tlg_status vjp_sumfact(const tlg_tables* t, const tlg::VjpArgs& v, cudaStream_t s, bool* found) {
  *found = false;
  if (!vjp_sumfact_preferred(t)) return TLG_ERR_UNSUPPORTED;
  const bool split = t->dtype == TLG_SPLIT32;
  const size_t fbytes = split ? 4 : 8;
  const int threads = tlg::kEvalThreads;
  const size_t smem = (t->sf_bytes + 15) / 16 * 16 + tlg::vjp_sumfact_extra_bytes(t->sf_n, threads, fbytes);
  if (smem > (size_t)227 * 1024) return TLG_ERR_UNSUPPORTED;
  tlg::VjpSfArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nodes = v.nodes;
  a.dofmap = v.dofmap;
  a.tab = t->dev + t->off_sf;
  for (int i = 0; i < 3; ++i) a.ct[i] = v.ct[i];
  for (int i = 0; i < 4; ++i) a.out[i] = v.out[i];
  a.local = v.local;
  a.err = v.err;
  a.first_cell = v.first_cell;
  a.padded = v.padded;
  a.out_first_cell = v.out_first_cell;
  a.last_cell = v.last_cell;
  a.range_end = v.range_end;
  for (int g = 0; g < 3; ++g) a.origin[g] = v.origin[g];
  a.last_node = v.last_node;
  a.tab_bytes = t->sf_bytes;
  for (int d = 0; d < 3; ++d) {
    a.off_b[d] = t->sf_block0.off_b[d];
    a.off_d[d] = t->sf_block0.off_d[d];
    a.m[d] = t->sf_block0.m[d];
  }
  a.off_perm = t->sf_offperm;
  a.num_points = v.num_points;
  cudaError_t e = tlg::launch_vjp_sumfact(split, t->sf_n, a, smem, threads, s, found);
  if (!*found) return TLG_ERR_UNSUPPORTED;
  if (e != cudaSuccess) return cuda_fail(e, "tlg_vjp_block launch");
  g_last_family = TLG_STRATEGY_SUMFACT;
  return ok();
}

// The sum-factorised adjoint from forward fields already written (det J and K in o->detj and
// o->pinv, read); `found` is false where it does not apply.
tlg_status vjp_sumfact_from_fields(const tlg_tables* t, const tlg_block* b, const tlg_outputs* o,
                                   const tlg_cotangents* ct, void* local, cudaStream_t s, bool* found) {
  *found = false;
  if (!vjp_sumfact_preferred(t) || !o->detj || !o->pinv) return TLG_ERR_UNSUPPORTED;
  const bool split = t->dtype == TLG_SPLIT32;
  const size_t fbytes = split ? 4 : 8;
  const int threads = tlg::kEvalThreads;
  // The tile kernel where a tile's points and plane sums fit, else one thread per cell.
  const size_t stab = (t->sf_bytes + 15) / 16 * 16;
  const size_t smem_tile = stab + tlg::vjp_sumfact_tile_extra_bytes(t->sf_n, (int)t->q, t->sf_block0.m[2], fbytes);
  const bool tiled = smem_tile <= (size_t)227 * 1024;
  const size_t smem = tiled ? smem_tile : stab + tlg::vjp_sumfact_bwd_extra_bytes(t->sf_n, threads, fbytes);
  if (smem > (size_t)227 * 1024) return TLG_ERR_UNSUPPORTED;
  tlg::VjpSfArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nodes = b->nodes;
  a.dofmap = b->dofmap;
  a.tab = t->dev + t->off_sf;
  a.ct[0] = ct->points;
  a.ct[1] = ct->detj;
  a.ct[2] = ct->pinv;
  a.out[2] = o->detj;
  a.out[3] = o->pinv;
  a.local = local;
  a.err = t->err;
  a.first_cell = o->first_cell;
  a.padded = (o->num_cells + 15) / 16 * 16;
  a.out_first_cell = o->out_first_cell;
  a.last_cell = b->num_cells - 1;
  a.range_end = o->first_cell + o->num_cells;
  a.last_node = (uint32_t)(b->num_nodes - 1);
  a.tab_bytes = t->sf_bytes;
  for (int d = 0; d < 3; ++d) {
    a.off_b[d] = t->sf_block0.off_b[d];
    a.off_d[d] = t->sf_block0.off_d[d];
    a.m[d] = t->sf_block0.m[d];
  }
  a.off_perm = t->sf_offperm;
  a.num_points = (int)t->q;
  cudaError_t e = tiled ? tlg::launch_vjp_sumfact_tile(split, t->sf_n, a, smem, s, found)
                        : tlg::launch_vjp_sumfact_bwd(split, t->sf_n, a, smem, threads, s, found);
  if (!*found) return TLG_ERR_UNSUPPORTED;
  if (e != cudaSuccess) return cuda_fail(e, "tlg_vjp_block_from_fields launch");
  g_last_family = TLG_STRATEGY_SUMFACT;
  return ok();
}

// The adjoint of volume cells of any kind from forward fields already written (vjp_tile_kernel):
// the node rows staged, then 12 * 16 values of F per point; `found` is false where it does not
// apply (no node-row table, or more than the shared memory holds).
size_t vjp_tile_smem(const tlg_tables* t) {
  const size_t fbytes = t->dtype == TLG_SPLIT32 ? 4 : 8;
  return (size_t)(t->vjp_bytes + 15) / 16 * 16 + (size_t)t->q * tlg::kVjpTileRec * 16 * fbytes;
}

bool vjp_tile_applies(const tlg_tables* t) {
  return t->td == 3 && t->gd == 3 && t->vjp_bytes > 0 && t->k <= 1024 && vjp_tile_smem(t) <= (size_t)227 * 1024;
}

tlg_status vjp_tile_from_fields(const tlg_tables* t, const tlg_block* b, const tlg_outputs* o, const tlg_cotangents* ct,
                                void* local, cudaStream_t s, bool* found) {
  *found = false;
  if (!vjp_tile_applies(t) || !o->detj || !o->pinv) return TLG_ERR_UNSUPPORTED;
  *found = true;
  tlg::VjpArgs a;
  std::memset(&a, 0, sizeof(a));
  a.tab = t->dev + t->off_vjp;
  a.ct[0] = ct->points;
  a.ct[1] = ct->detj;
  a.ct[2] = ct->pinv;
  a.out[2] = o->detj;
  a.out[3] = o->pinv;
  a.local = local;
  a.err = t->err;
  a.first_cell = o->first_cell;
  a.padded = (o->num_cells + 15) / 16 * 16;
  a.out_first_cell = o->out_first_cell;
  a.last_cell = b->num_cells - 1;
  a.range_end = o->first_cell + o->num_cells;
  a.tab_bytes = t->vjp_bytes;
  a.num_points = (int)t->q;
  a.k_runtime = (int)t->k;
  cudaError_t e = tlg::launch_vjp_tile(t->dtype == TLG_SPLIT32, a, vjp_tile_smem(t), s);
  if (e != cudaSuccess) return cuda_fail(e, "tlg_vjp_block_from_fields launch");
  g_last_family = TLG_STRATEGY_DIRECT;
  return ok();
}

// Whether tlg_vjp_block_from_fields serves the tables.
bool from_fields_applies(const tlg_tables* t) { return vjp_sumfact_preferred(t) || vjp_tile_applies(t); }

// The adjoint below codimension 0 (vjp_surface.cu) from the node-row kernel's arguments: phi and
// dphi staged when they and the thread slots (2 K GD values per thread) fit, else read from global
// memory; 32 to 128 threads per CTA.
tlg_status vjp_surface(const tlg_tables* t, const tlg_block* b, const tlg_outputs* o, const tlg_cotangents* ct,
                       const tlg::VjpArgs& v, cudaStream_t s) {
  const bool split = t->dtype == TLG_SPLIT32;
  const size_t fbytes = split ? 4 : 8;
  const size_t per_thread = 2 * (size_t)t->k * t->gd * fbytes;
  const size_t budget = (size_t)227 * 1024;
  const size_t prefix = (size_t)t->off_refn;  // phi and dphi
  bool global = !(prefix + 32 * per_thread <= budget);
  const size_t avail = budget - (global ? 0 : prefix);
  int threads = (int)std::min<size_t>(128, avail / per_thread / 32 * 32);
  if (threads < 32) return fail(TLG_ERR_ALLOCATION_TOO_LARGE, "tlg_vjp_block: too many nodes per cell");
  tlg::VjpSurfArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nodes = v.nodes;
  a.dofmap = v.dofmap;
  a.flags = b->flags;
  a.tab = t->dev;
  a.ct[0] = ct->points;
  a.ct[1] = ct->detj;
  a.ct[2] = ct->pinv;
  a.ct[3] = ct->normals;
  a.out[0] = o->points;
  a.out[1] = o->jacobian;
  a.out[2] = o->detj;
  a.out[3] = o->pinv;
  a.out[4] = o->normals;
  a.local = v.local;
  a.err = v.err;
  a.first_cell = v.first_cell;
  a.padded = v.padded;
  a.out_first_cell = v.out_first_cell;
  a.last_cell = v.last_cell;
  a.range_end = v.range_end;
  const int64_t nflags = b->flags ? std::min<int64_t>(b->num_cells, b->num_flags) : 0;
  a.last_flag = nflags - 1;
  for (int g = 0; g < 3; ++g) a.origin[g] = v.origin[g];
  a.last_node = v.last_node;
  a.tab_bytes = global ? 0 : (uint32_t)prefix;
  a.off_dphi = t->off_dphi;
  a.k = (int)t->k;
  a.num_points = v.num_points;
  a.tab_global = global ? 1 : 0;
  const size_t smem = (global ? 0 : (prefix + 15) / 16 * 16) + (size_t)threads * per_thread;
  bool found = false;
  cudaError_t e = tlg::launch_vjp_surface(split, t->td, t->gd, a, smem, threads, s, &found);
  if (!found) return fail(TLG_ERR_UNSUPPORTED, "tlg_vjp_block: no adjoint kernel for this element");
  if (e != cudaSuccess) return cuda_fail(e, "tlg_vjp_block launch");
  g_last_family = TLG_STRATEGY_LOOPS;
  return ok();
}

}  // namespace

tlg_status tlg_vjp_block(const tlg_tables* t, const tlg_block* b, const tlg_outputs* o,
                         const tlg_cotangents* ct, void* local, int64_t local_cells, void* stream) {
  if (!t || !b || !o || !ct) return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_vjp_block: NULL argument");
  if (t->dtype != TLG_F64 && t->dtype != TLG_SPLIT32)
    return fail(TLG_ERR_UNSUPPORTED, "tlg_vjp_block: the adjoint runs with f64 or split-precision tables");
  if (b->dtype != TLG_F64) return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_vjp_block: the adjoint reads f64 meshes");
  if (b->gdim != t->gd) return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_vjp_block: block and tables differ in gdim");
  if (o->tile != 16) return fail(TLG_ERR_UNSUPPORTED, "tlg_vjp_block: the adjoint runs with tile 16");
  if (o->facet_normals) return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_vjp_block: no facet normals in the fused forward");
  if (o->cell_measure)
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_vjp_block: cell_measure is summed by tlg_eval_block only");
  if ((o->normals || ct->normals) && t->td + 1 != t->gd)
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_vjp_block: normals exist for TD + 1 = GD only");
  if (o->first_cell < 0 || o->num_cells < 0 || o->first_cell + o->num_cells > b->num_cells ||
      o->out_first_cell < 0 || o->out_first_cell % 16 != 0)
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_vjp_block: bad cell range");
  if (local_cells < b->num_cells) return fail(TLG_ERR_LENGTH_MISMATCH, "tlg_vjp_block: local_cells below the block's cells");
  if (o->num_cells == 0) return ok();
  if (!b->nodes || !b->dofmap || !local) return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_vjp_block: NULL nodes, dofmap or local");
  if (b->num_nodes < 1) return fail(TLG_ERR_LENGTH_MISMATCH, "tlg_vjp_block: cells but no nodes");
  tlg::VjpArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nodes = b->nodes;
  a.dofmap = b->dofmap;
  a.tab = t->dev + t->off_vjp;
  a.ct[0] = ct->points;
  a.ct[1] = ct->detj;
  a.ct[2] = ct->pinv;
  a.out[0] = o->points;
  a.out[1] = o->jacobian;
  a.out[2] = o->detj;
  a.out[3] = o->pinv;
  a.local = local;
  a.err = t->err;
  a.first_cell = o->first_cell;
  a.padded = (o->num_cells + 15) / 16 * 16;
  a.out_first_cell = o->out_first_cell;
  a.last_cell = b->num_cells - 1;
  a.range_end = o->first_cell + o->num_cells;
  for (int g = 0; g < 3; ++g) a.origin[g] = b->origin[g];
  a.last_node = (uint32_t)(b->num_nodes - 1);
  a.tab_bytes = t->vjp_bytes;
  const bool split = t->dtype == TLG_SPLIT32;
  a.num_points = (int)t->q;
  if (t->q == 0) return ok();
  // The adjoint follows the Jacobian family's strategy: sum factorisation where wanted (or AUTO)
  // and it applies, else the node-row kernel (the kernel below codimension 0 has K at run time).
  int strategy = TLG_STRATEGY_AUTO;
  if (!wanted_strategy(TLG_FAMILY_JACOBIAN, &strategy)) return TLG_ERR_INVALID_ARGUMENT;
  g_last_kind = TLG_FAMILY_JACOBIAN;
  if (t->td < t->gd) return vjp_surface(t, b, o, ct, a, static_cast<cudaStream_t>(stream));
  const size_t smem = (t->vjp_bytes + 15) / 16 * 16 + tlg::vjp_stage_bytes(split, t->td, (int)t->k);
  bool found = false;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (strategy == TLG_STRATEGY_SUMFACT || (strategy == TLG_STRATEGY_AUTO && vjp_sumfact_preferred(t))) {
    tlg_status st = vjp_sumfact(t, a, s, &found);
    if (found) return st;
  }
  cudaError_t e = cudaSuccess;
  if (t->vjp_bytes > 0 && smem <= (size_t)227 * 1024)
    e = split ? tlg::launch_vjp_split(t->td, (int)t->k, a, smem, s, &found)
              : tlg::launch_vjp_f64(t->td, (int)t->k, a, smem, s, &found);
  // No node-row kernel for the element (or its table does not fit): K at run time.
  if (!found) return vjp_surface(t, b, o, ct, a, s);
  if (e != cudaSuccess) return cuda_fail(e, "tlg_vjp_block launch");
  g_last_family = TLG_STRATEGY_DIRECT;
  return ok();
}

tlg_status tlg_vjp_block_from_fields(const tlg_tables* t, const tlg_block* b, const tlg_outputs* o,
                                     const tlg_cotangents* ct, void* local, int64_t local_cells, void* stream) {
  if (!t || !b || !o || !ct) return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_vjp_block_from_fields: NULL argument");
  if (t->dtype != TLG_F64 && t->dtype != TLG_SPLIT32)
    return fail(TLG_ERR_UNSUPPORTED, "tlg_vjp_block_from_fields: f64 or split-precision tables");
  if (b->gdim != t->gd || t->td != t->gd)
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_vjp_block_from_fields: codimension 0, block and tables alike");
  if (o->tile != 16) return fail(TLG_ERR_UNSUPPORTED, "tlg_vjp_block_from_fields: tile 16");
  if (!o->detj || !o->pinv)
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_vjp_block_from_fields: the det J and K fields are the inputs");
  if (o->first_cell < 0 || o->num_cells < 0 || o->first_cell + o->num_cells > b->num_cells ||
      o->out_first_cell < 0 || o->out_first_cell % 16 != 0)
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_vjp_block_from_fields: bad cell range");
  if (local_cells < b->num_cells)
    return fail(TLG_ERR_LENGTH_MISMATCH, "tlg_vjp_block_from_fields: local_cells below the block's cells");
  if (o->num_cells == 0 || t->q == 0) return ok();
  if (!local) return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_vjp_block_from_fields: NULL local");
  bool found = false;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  tlg_status st = vjp_sumfact_from_fields(t, b, o, ct, local, s, &found);
  if (!found) st = vjp_tile_from_fields(t, b, o, ct, local, s, &found);
  if (!found)
    return fail(TLG_ERR_UNSUPPORTED, "tlg_vjp_block_from_fields: no kernel for the element and rule (volume cells "
                                     "whose node rows and point slots fit in shared memory)");
  return st;
}

tlg_status tlg_vjp_gather(const uint32_t* offsets, const uint32_t* entries, int64_t num_nodes, int gdim,
                          const void* local, int local_dtype, double* grad, void* stream) {
  if (!offsets || !grad || num_nodes < 0 || gdim < 1 || gdim > 3 || (local_dtype != 4 && local_dtype != 8))
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_vjp_gather: bad arguments");
  if (num_nodes == 0) return ok();
  cudaError_t e = tlg::launch_vjp_gather(offsets, entries, num_nodes, gdim, local, local_dtype, grad,
                                         static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "tlg_vjp_gather launch");
  return ok();
}

tlg_status tlg_vjp_gather_add(const uint32_t* offsets, const uint32_t* entries, int64_t num_nodes, int gdim,
                              const void* local, int local_dtype, double* grad, void* stream) {
  if (!offsets || !grad || num_nodes < 0 || gdim < 1 || gdim > 3 || (local_dtype != 4 && local_dtype != 8))
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_vjp_gather_add: bad arguments");
  if (num_nodes == 0) return ok();
  cudaError_t e = tlg::launch_vjp_gather(offsets, entries, num_nodes, gdim, local, local_dtype, grad,
                                         static_cast<cudaStream_t>(stream), true);
  if (e != cudaSuccess) return cuda_fail(e, "tlg_vjp_gather_add launch");
  return ok();
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// Adjoint batches: the per-cell contributions of every block on parallel branches of one CUDA
// graph, then the node sums block by block onto one gradient.

struct tlg_vjp_batch {
  std::vector<const tlg_tables*> tables;
  std::vector<tlg_block> blocks;
  std::vector<tlg_outputs> outputs;
  std::vector<tlg_cotangents> cotangents;
  std::vector<void*> locals;
  std::vector<int64_t> local_cells;
  std::vector<const uint32_t*> offsets, entries;
  // Tables of a separate forward evaluation per block (tlg_vjp_batch_set_forward), or empty.
  std::vector<const tlg_tables*> forward;
  // tlg_vjp_batch_set_two_pass: blocks whose adjoint can read det J and K back run the policy's
  // forward, then the adjoint from those fields.
  bool two_pass = false;
  int64_t num_nodes = 0;
  int gdim = 0;
  double* grad = nullptr;
  cudaStream_t capture = nullptr;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> events;
  cudaGraphExec_t exec = nullptr;
};

extern "C" {

tlg_status tlg_vjp_batch_create(const tlg_tables* const* tables, const tlg_block* blocks, const tlg_outputs* outputs,
                                const tlg_cotangents* cotangents, void* const* locals, const int64_t* local_cells,
                                const uint32_t* const* offsets, const uint32_t* const* entries, int64_t num_nodes,
                                int gdim, double* grad, int num_blocks, tlg_vjp_batch** out) {
  if (!out || num_blocks < 0 || !grad || gdim < 1 || gdim > 3 || num_nodes < 0 ||
      (num_blocks > 0 && (!tables || !blocks || !outputs || !cotangents || !locals || !local_cells || !offsets ||
                          !entries)))
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_vjp_batch_create: NULL or bad argument");
  *out = nullptr;
  auto b = new tlg_vjp_batch();
  for (int i = 0; i < num_blocks; ++i) {
    if (!tables[i] || !offsets[i] || tables[i]->gd != gdim ||
        (tables[i]->dtype == TLG_SPLIT32) != (tables[0]->dtype == TLG_SPLIT32)) {
      delete b;
      return fail(TLG_ERR_INVALID_ARGUMENT,
                  "tlg_vjp_batch_create: NULL tables or CSR, another gdim, or split and f64 tables mixed");
    }
    b->tables.push_back(tables[i]);
    b->blocks.push_back(blocks[i]);
    b->outputs.push_back(outputs[i]);
    b->cotangents.push_back(cotangents[i]);
    b->locals.push_back(locals[i]);
    b->local_cells.push_back(local_cells[i]);
    b->offsets.push_back(offsets[i]);
    b->entries.push_back(entries[i]);
  }
  b->num_nodes = num_nodes;
  b->gdim = gdim;
  b->grad = grad;
  cudaError_t e = cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking);
  for (int i = 0; i < num_blocks && e == cudaSuccess; ++i) {
    cudaStream_t st;
    e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) b->streams.push_back(st);
  }
  for (int i = 0; i < num_blocks + 1 && e == cudaSuccess; ++i) {
    cudaEvent_t ev;
    e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e == cudaSuccess) b->events.push_back(ev);
  }
  if (e != cudaSuccess) {
    tlg_vjp_batch_destroy(b);
    return cuda_fail(e, "tlg_vjp_batch_create");
  }
  *out = b;
  return ok();
}

tlg_status tlg_vjp_batch_destroy(tlg_vjp_batch* b) {
  if (!b) return ok();
  if (b->exec) cudaGraphExecDestroy(b->exec);
  for (auto st : b->streams) cudaStreamDestroy(st);
  for (auto ev : b->events) cudaEventDestroy(ev);
  if (b->capture) cudaStreamDestroy(b->capture);
  delete b;
  return ok();
}

tlg_status tlg_vjp_batch_set_forward(tlg_vjp_batch* b, const tlg_tables* const* forward) {
  if (!b) return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_vjp_batch_set_forward: NULL batch");
  std::vector<const tlg_tables*> f;
  if (forward) {
    for (size_t i = 0; i < b->tables.size(); ++i) {
      if (!forward[i] || forward[i]->gd != b->gdim)
        return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_vjp_batch_set_forward: NULL tables or another gdim");
      f.push_back(forward[i]);
    }
  }
  b->forward = f;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
  return ok();
}

tlg_status tlg_vjp_batch_set_two_pass(tlg_vjp_batch* b, int on) {
  if (!b || (on != 0 && on != 1)) return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_vjp_batch_set_two_pass: NULL batch or not 0/1");
  b->two_pass = on != 0;
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
  return ok();
}

tlg_status tlg_vjp_batch_launch(tlg_vjp_batch* b, void* stream) {
  if (!b) return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_vjp_batch_launch: NULL batch");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!b->exec) {
    // Capture: the blocks' contributions on parallel branches, then the node sums in block order:
    // the first block's sums written over the whole gradient (zero at nodes it does not touch),
    // each further block's added onto it (deterministic).
    cudaError_t e = cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(e, "tlg_vjp_batch_launch: begin capture");
    tlg_status st = TLG_OK;
    const size_t nb = b->tables.size();
    if (nb == 0) e = cudaMemsetAsync(b->grad, 0, (size_t)b->num_nodes * b->gdim * sizeof(double), b->capture);
    if (e == cudaSuccess) e = cudaEventRecord(b->events[nb], b->capture);
    for (size_t i = 0; i < nb && e == cudaSuccess && st == TLG_OK; ++i) {
      e = cudaStreamWaitEvent(b->streams[i], b->events[nb], 0);
      if (e != cudaSuccess) break;
      if (!b->forward.empty()) {
        // The forward fields from their own tables, then the adjoint alone on the same branch.
        st = tlg_eval_block(b->forward[i], &b->blocks[i], &b->outputs[i], b->streams[i]);
        tlg_outputs adj = b->outputs[i];
        adj.points = adj.jacobian = adj.detj = adj.pinv = adj.normals = adj.facet_normals = nullptr;
        adj.cell_measure = nullptr;
        if (st == TLG_OK)
          st = tlg_vjp_block(b->tables[i], &b->blocks[i], &adj, &b->cotangents[i], b->locals[i], b->local_cells[i],
                             b->streams[i]);
      } else if (b->two_pass && from_fields_applies(b->tables[i]) && b->outputs[i].detj && b->outputs[i].pinv) {
        st = tlg_eval_block(b->tables[i], &b->blocks[i], &b->outputs[i], b->streams[i]);
        if (st == TLG_OK)
          st = tlg_vjp_block_from_fields(b->tables[i], &b->blocks[i], &b->outputs[i], &b->cotangents[i], b->locals[i],
                                         b->local_cells[i], b->streams[i]);
      } else {
        st = tlg_vjp_block(b->tables[i], &b->blocks[i], &b->outputs[i], &b->cotangents[i], b->locals[i],
                           b->local_cells[i], b->streams[i]);
      }
      if (st == TLG_OK) e = cudaEventRecord(b->events[i], b->streams[i]);
      if (e == cudaSuccess && st == TLG_OK) e = cudaStreamWaitEvent(b->capture, b->events[i], 0);
    }
    // The node sums in groups of up to kGatherMaxBlocks blocks per pass over the nodes (rows of
    // one dtype: a batch has one precision), the first group writing the gradient.
    for (size_t i0 = 0; i0 < nb && e == cudaSuccess && st == TLG_OK && b->num_nodes > 0;
         i0 += tlg::kGatherMaxBlocks) {
      tlg::GatherBlocks gb;
      std::memset(&gb, 0, sizeof(gb));
      const size_t i1 = std::min(nb, i0 + (size_t)tlg::kGatherMaxBlocks);
      for (size_t i = i0; i < i1; ++i) {
        gb.offsets[i - i0] = b->offsets[i];
        gb.entries[i - i0] = b->entries[i];
        gb.local[i - i0] = b->locals[i];
      }
      gb.count = (int)(i1 - i0);
      const int ldt = b->tables[i0]->dtype == TLG_SPLIT32 ? 4 : 8;
      e = tlg::launch_vjp_gather_blocks(gb, b->num_nodes, b->gdim, ldt, b->grad, b->capture, i0 > 0);
    }
    cudaGraph_t graph = nullptr;
    const std::string msg = tlg_last_error();
    cudaError_t ee = cudaStreamEndCapture(b->capture, &graph);
    if (st != TLG_OK) {
      if (graph) cudaGraphDestroy(graph);
      return fail(st, msg);
    }
    if (e == cudaSuccess) e = ee;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, "tlg_vjp_batch_launch: capture");
  }
  cudaError_t e = cudaGraphLaunch(b->exec, s);
  if (e != cudaSuccess) return cuda_fail(e, "tlg_vjp_batch_launch");
  return ok();
}

}  // extern "C"

extern "C" {

// ---------------------------------------------------------------------------------------
// Batches: every block of a hybrid mesh in one CUDA graph launch, launch shapes autotuned.

namespace {

std::mutex g_tune_mutex;
std::map<std::string, std::pair<int, int>> g_tune_cache;  // launch-shape key -> (strategy, grid multiplier)
std::map<std::string, std::vector<int>> g_joint_cache;  // batch key -> grids after the joint pass,
                                                        // then 1 for a serial chain, 0 for branches

std::string tune_key(const tlg_tables* t, const tlg_outputs* o, int64_t cells) {
  int bucket = 0;
  while ((int64_t(1) << bucket) < cells) ++bucket;
  char buf[160];
  std::snprintf(buf, sizeof(buf), "d%d%s t%d g%d k%lld q%lld c%d o%d%d%d%d%d%d", t->dtype, t->df ? "df" : "", t->td, t->gd,
                (long long)t->k, (long long)t->q, bucket, o->points != nullptr, o->jacobian != nullptr,
                o->detj != nullptr, o->pinv != nullptr, o->normals != nullptr, o->facet_normals != nullptr);
  return buf;
}

void destroy_graph(tlg_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
}

// Block i's launch with its grid and strategy (every family's override set for the launch and
// restored after it).
tlg_status eval_with_grid(tlg_batch* b, size_t i, cudaStream_t s, int grid) {
  const int forced = b->strategy[i];
  int saved[kFamilies];
  if (forced >= 0)
    for (int f = 0; f < kFamilies; ++f) {
      saved[f] = g_override[f];
      g_override[f] = forced;
    }
  tlg::g_grid_override = grid;
  tlg_status st = tlg_eval_block(b->tables[i], &b->blocks[i], &b->outputs[i], s);
  tlg::g_grid_override = 0;
  if (forced >= 0)
    for (int f = 0; f < kFamilies; ++f) g_override[f] = saved[f];
  return st;
}

// The strategies worth timing for a block: the policy, and the forced strategies whose kernels
// apply to its tables (the others would run the loops kernel): the unrolled or paired kernels,
// sum factorisation (tensor-product point sets), the cooperative kernel (not for double-float
// tables, which it runs in FP64), the tensor-core kernels (f32 and split tables).
std::vector<int> strategy_candidates(const tlg_tables* t) {
  std::vector<int> c = {-1, TLG_STRATEGY_DIRECT};
  if (t->sf_ok) c.push_back(TLG_STRATEGY_SUMFACT);
  if (t->td >= 2 && t->k <= 128 && !t->df) c.push_back(TLG_STRATEGY_COOPERATIVE);
  if ((t->umma_kpad > 0 || t->tc_ksteps > 0) && (t->dtype == TLG_F32 || t->dtype == TLG_SPLIT32))
    c.push_back(TLG_STRATEGY_TENSOR);
  return c;
}

}  // namespace

tlg_status tlg_batch_create(const tlg_tables* const* tables, const tlg_block* blocks, const tlg_outputs* outputs,
                            int num_blocks, tlg_batch** out) {
  if (!out || num_blocks < 0 || (num_blocks > 0 && (!tables || !blocks || !outputs)))
    return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_batch_create: NULL argument");
  *out = nullptr;
  auto b = new tlg_batch();
  for (int i = 0; i < num_blocks; ++i) {
    if (!tables[i]) {
      delete b;
      return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_batch_create: NULL tables");
    }
    b->tables.push_back(tables[i]);
    b->blocks.push_back(blocks[i]);
    b->outputs.push_back(outputs[i]);
    b->grid.push_back(0);
    b->strategy.push_back(-1);
  }
  cudaError_t e = cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking);
  for (int i = 0; i < num_blocks && e == cudaSuccess; ++i) {
    cudaStream_t s;
    e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e == cudaSuccess) b->streams.push_back(s);
  }
  for (int i = 0; i < num_blocks + 1 && e == cudaSuccess; ++i) {
    cudaEvent_t ev;
    e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e == cudaSuccess) b->events.push_back(ev);
  }
  if (e != cudaSuccess) {
    tlg_batch_destroy(b);
    return cuda_fail(e, "tlg_batch_create");
  }
  *out = b;
  return ok();
}

tlg_status tlg_batch_destroy(tlg_batch* b) {
  if (!b) return ok();
  destroy_graph(b);
  for (auto s : b->streams) cudaStreamDestroy(s);
  for (auto ev : b->events) cudaEventDestroy(ev);
  if (b->capture) cudaStreamDestroy(b->capture);
  delete b;
  return ok();
}

tlg_status tlg_batch_tune(tlg_batch* b, void* stream, int* grids) {
  if (!b) return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_batch_tune: NULL batch");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  // The median of `n` launches timed one by one (after `fn` has run once untimed): robust
  // against a launch slowed by a clock or power transition, which an average of back-to-back
  // launches is not.
  auto median_ms = [&](auto fn, float* ms, int n = 7, float* mean = nullptr) -> tlg_status {
    tlg_status st = fn();
    float t[15];
    n = std::min(n, 15);
    for (int r = 0; r < n && st == TLG_OK; ++r) {
      cudaEventRecord(t0, s);
      st = fn();
      cudaEventRecord(t1, s);
      cudaEventSynchronize(t1);
      cudaEventElapsedTime(&t[r], t0, t1);
    }
    std::sort(t, t + n);
    *ms = t[n / 2];
    if (mean) {
      float sum = 0.0f;
      for (int r = 0; r < n; ++r) sum += t[r];
      *mean = sum / n;
    }
    return st;
  };
  auto finish = [&](tlg_status st) {
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    return st;
  };
  const int cands[] = {0, 1, 2, 3, 4, 6, 8};  // CTAs per SM of the persistent grid (0: occupancy)
  // A strategy set by the caller (a scoped override or TLG_GEOM_STRATEGY) is kept; otherwise each
  // block's strategy is a candidate too: the kernel families tile the work differently (paired
  // kernels: 16-cell tiles, two points per instruction; sum factorisation: a cell's planes and
  // rows per thread; cooperative: four lanes per cell; tcgen05: 64-cell tiles by 8-point chunks).
  int fixed = TLG_STRATEGY_AUTO;
  if (!wanted_strategy(TLG_FAMILY_JACOBIAN, &fixed)) return finish(TLG_ERR_INVALID_ARGUMENT);
  bool caller_fixed = fixed != TLG_STRATEGY_AUTO;
  for (int f = 0; f < kFamilies; ++f) caller_fixed = caller_fixed || g_override[f] >= 0;
  for (size_t i = 0; i < b->tables.size(); ++i) {
    const std::string key = tune_key(b->tables[i], &b->outputs[i], b->outputs[i].num_cells) +
                            (caller_fixed ? " fixed" : "");
    std::pair<int, int> choice(-1, -1);
    {
      std::lock_guard<std::mutex> lock(g_tune_mutex);
      auto it = g_tune_cache.find(key);
      if (it != g_tune_cache.end()) choice = it->second;
    }
    if (choice.second < 0) {
      // The strategy at the occupancy grid (a forced strategy replaces the policy only when more
      // than 1 % faster), then the grid for it.
      b->grid[i] = 0;
      float best = 1e30f;
      int strat = -1;
      const std::vector<int> strats = caller_fixed ? std::vector<int>{-1} : strategy_candidates(b->tables[i]);
      for (int c : strats) {
        b->strategy[i] = c;
        float ms = 0.0f;
        tlg_status st = median_ms([&] { return eval_with_grid(b, i, s, 0); }, &ms);
        if (st != TLG_OK) {
          b->strategy[i] = -1;
          return finish(st);
        }
        if (ms < (c == -1 ? best : 0.97f * best)) {  // a forced strategy: more than 3 % faster
          best = ms;
          strat = c;
        }
      }
      b->strategy[i] = strat;
      int mult = 0;
      for (int c : cands) {
        if (c == 0) continue;  // timed above
        const int grid = c * sms;
        float ms = 0.0f;
        tlg_status st = median_ms([&] { return eval_with_grid(b, i, s, grid); }, &ms);
        if (st != TLG_OK) return finish(st);
        // A candidate replaces the occupancy default only when more than 1 % faster.
        if (ms < 0.99f * best) {
          best = ms;
          mult = c;
        }
      }
      choice = {strat, mult};
      std::lock_guard<std::mutex> lock(g_tune_mutex);
      g_tune_cache[key] = choice;
    }
    b->strategy[i] = choice.first;
    b->grid[i] = choice.second == 0 ? 0 : choice.second * sms;
  }
  // Joint pass: the graph runs the blocks concurrently (or in turn), so each block's best grid
  // alone is only the start. Every comparison times the whole graph (time_graph), and a change
  // is kept only when more than 1 % faster, so that run-to-run noise does not pick the
  // configuration: parallel branches against a serial chain (the concurrent branches of
  // persistent kernels share the SMs in an order the hardware picks; the chain is kept unless
  // the branches are more than 3 % faster in the median and the slowest round), one round of
  // coordinate descent over each block's grid candidates, and the result against every block at
  // its occupancy default.
  std::string batch_key = caller_fixed ? "fixed;" : "";
  for (size_t i = 0; i < b->tables.size(); ++i)
    batch_key += tune_key(b->tables[i], &b->outputs[i], b->outputs[i].num_cells) + ";";
  std::vector<int> joint;
  {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_joint_cache.find(batch_key);
    if (it != g_joint_cache.end()) joint = it->second;
  }
  // A graph is timed as it runs in use, launch after launch: the median over five rounds of the
  // mean of four back-to-back launches (consecutive graphs with parallel branches can interfere,
  // which launches timed one by one do not show; the median of rounds still drops a round slowed
  // by a clock or power transition).
  auto time_graph = [&](float* ms, float* spread = nullptr) -> tlg_status {
    destroy_graph(b);
    tlg_status st = tlg_batch_launch(b, s);
    float r[5];
    for (int k = 0; k < 5 && st == TLG_OK; ++k) {
      cudaEventRecord(t0, s);
      for (int l = 0; l < 4 && st == TLG_OK; ++l) st = tlg_batch_launch(b, s);
      cudaEventRecord(t1, s);
      cudaEventSynchronize(t1);
      cudaEventElapsedTime(&r[k], t0, t1);
      r[k] /= 4.0f;
    }
    if (st != TLG_OK) return st;
    std::sort(r, r + 5);
    *ms = r[2];
    if (spread) *spread = r[4];
    return st;
  };
  if (joint.size() == b->tables.size() + 1) {
    for (size_t i = 0; i < b->tables.size(); ++i) b->grid[i] = joint[i];
    b->serial = joint.back() != 0;
  } else if (b->tables.size() > 1) {
    float serial_ms = 0.0f, par_ms = 0.0f, serial_max = 0.0f, par_max = 0.0f, best = 0.0f;
    b->serial = true;
    tlg_status st = time_graph(&serial_ms, &serial_max);
    if (st == TLG_OK) {
      b->serial = false;
      st = time_graph(&par_ms, &par_max);
    }
    if (st != TLG_OK) return finish(st);
    // Branches only when faster in the median and in the slowest round (their times spread more).
    b->serial = !(par_ms < 0.97f * serial_ms && par_max < 0.97f * serial_max);
    best = b->serial ? serial_ms : par_ms;
    for (size_t i = 0; i < b->tables.size() && st == TLG_OK; ++i) {
      const int keep = b->grid[i];
      int chosen = keep;
      for (int c : cands) {
        const int grid = c == 0 ? 0 : c * sms;
        if (grid == keep) continue;
        b->grid[i] = grid;
        float ms = 0.0f;
        st = time_graph(&ms);
        if (st != TLG_OK) break;
        if (ms < 0.99f * best) {
          best = ms;
          chosen = grid;
        }
      }
      b->grid[i] = chosen;
    }
    if (st != TLG_OK) return finish(st);
    // The untuned graph (occupancy grids, serial chain) against the result, timed again.
    const std::vector<int> tuned = b->grid;
    const bool tuned_serial = b->serial;
    float base_ms = 0.0f, again_ms = 0.0f;
    for (auto& gi : b->grid) gi = 0;
    b->serial = true;
    st = time_graph(&base_ms);
    b->grid = tuned;
    b->serial = tuned_serial;
    if (st == TLG_OK) st = time_graph(&again_ms);
    if (st != TLG_OK) return finish(st);
    if (!(again_ms < 0.99f * base_ms)) {
      for (auto& gi : b->grid) gi = 0;
      b->serial = true;
    }
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    std::vector<int> rec = b->grid;
    rec.push_back(b->serial ? 1 : 0);
    g_joint_cache[batch_key] = rec;
  }
  if (!b->tables.empty()) {
    float ms = 0.0f;
    tlg_status st = time_graph(&ms);
    if (st != TLG_OK) return finish(st);
    b->tuned_ms = ms;
  }
  if (grids)
    for (size_t i = 0; i < b->tables.size(); ++i) grids[i] = b->grid[i];
  finish(TLG_OK);
  destroy_graph(b);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "tlg_batch_tune");
  return ok();
}

tlg_status tlg_batch_tuning(const tlg_batch* b, int* serial, float* ms, int* strategies) {
  if (!b) return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_batch_tuning: NULL batch");
  if (serial) *serial = b->serial ? 1 : 0;
  if (ms) *ms = b->tuned_ms;
  if (strategies)
    for (size_t i = 0; i < b->strategy.size(); ++i) strategies[i] = b->strategy[i];
  return ok();
}

tlg_status tlg_batch_launch(tlg_batch* b, void* stream) {
  if (!b) return fail(TLG_ERR_INVALID_ARGUMENT, "tlg_batch_launch: NULL batch");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (!b->exec) {
    // Capture every block's launch as a parallel branch of one graph: fork from the capture
    // stream, one stream per block, join back.
    cudaError_t e = cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(e, "tlg_batch_launch: begin capture");
    tlg_status st = TLG_OK;
    if (b->serial) {
      for (size_t i = 0; i < b->tables.size() && st == TLG_OK; ++i)
        st = eval_with_grid(b, i, b->capture, b->grid[i]);
    } else {
      cudaEventRecord(b->events[0], b->capture);
      for (size_t i = 0; i < b->tables.size() && st == TLG_OK; ++i) {
        cudaStreamWaitEvent(b->streams[i], b->events[0], 0);
        st = eval_with_grid(b, i, b->streams[i], b->grid[i]);
        cudaEventRecord(b->events[i + 1], b->streams[i]);
        cudaStreamWaitEvent(b->capture, b->events[i + 1], 0);
      }
    }
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(b->capture, &graph);
    if (st != TLG_OK) {
      if (graph) cudaGraphDestroy(graph);
      return st;
    }
    if (e != cudaSuccess) return cuda_fail(e, "tlg_batch_launch: end capture");
    e = cudaGraphInstantiate(&b->exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) {
      b->exec = nullptr;
      return cuda_fail(e, "tlg_batch_launch: instantiate");
    }
  }
  cudaError_t e = cudaGraphLaunch(b->exec, s);
  if (e != cudaSuccess) return cuda_fail(e, "tlg_batch_launch");
  return ok();
}

}  // extern "C"
