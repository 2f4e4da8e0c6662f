/*
 * tlgeom: GB300-native (sm_103a) evaluation of the geometric factors of unstructured-mesh cell
 * blocks, behind a plain C ABI.
 *
 * This is the boundary a host program binds to replace the device kernels of tetraloma's
 * geometry path (tbetcke/gridcl). Every entry point takes plain pointers and sizes: device
 * pointers for mesh data and outputs, host pointers for reference points and small tables,
 * and a CUDA stream (`cudaStream_t`, passed as `void*`). No entry point of the evaluation
 * itself allocates device memory; `tlg_tables_create` allocates once per (element, point set)
 * and `tlg_tables_destroy` frees it.
 *
 * Status codes mirror `GridError` (tetraloma-device/src/error.rs:80-105):
 * TooLarge, LengthMismatch{expected, found}, AllocationTooLarge, Server(..). The message of
 * the last failure on the calling thread is `tlg_last_error()`.
 *
 * Data layouts (all as in the reference):
 *  - nodes: the node L-vector `[node][gdim]` of F, relative to the grid's origin
 *    (tetraloma/src/pipeline/upload.rs:65-73);
 *  - dofmap: `[cell][K]` u32 node indices of one block in the reference's Lagrange node order
 *    (tetraloma-refcell/src/lagrange.rs:163-266); indices past the last node read the last node
 *    (tetraloma-geometry/src/evector.rs:221-222);
 *  - outputs: QuadField chunks (tetraloma-geometry/src/field.rs:121-162): component k at point q
 *    of cell c at ((c / tile) * Q * LEN + q * LEN + k) * tile + c % tile, counted from the chunk's
 *    first cell; cells are padded to whole tiles and padding lanes hold the block's last cell;
 *  - J(g, d) at component d * GD + g (column-major GD x TD); K = J^+ (t, g) at g * TD + t;
 *    det J one component (sqrt(det(J^T J)) when TD < GD); normals and points GD components
 *    (tetraloma-geometry/src/layout.rs:91-131, 133-369).
 */
#ifndef TLGEOM_H
#define TLGEOM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TLG_ABI_VERSION 1

typedef enum tlg_status {
  TLG_OK = 0,
  TLG_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad tile, bad dimension pair, ... */
  TLG_ERR_LENGTH_MISMATCH = 2,  /* GridError::LengthMismatch */
  TLG_ERR_TOO_LARGE = 3,        /* GridError::TooLarge: a count does not fit the kernel's u32 */
  TLG_ERR_UNSUPPORTED = 4,      /* cell type / degree / factor this build has no kernel for */
  TLG_ERR_CUDA = 5,             /* GridError::Server: a CUDA runtime failure */
  TLG_ERR_DEVICE_TIMEOUT = 6,   /* a bounded device-side wait expired; the context is intact */
  TLG_ERR_ALLOCATION_TOO_LARGE = 7 /* GridError::AllocationTooLarge */
} tlg_status;

/* Scalar type of nodes and outputs: the byte size of F. TLG_SPLIT32 (tables only) selects the
 * split-precision evaluation: an f64 mesh, FP32 arithmetic on cell-shifted coordinates, f32
 * outputs, FP64 recompute of det J and K at points flagged by a condition estimate. TLG_DF64
 * (tables only) selects the double-float evaluation: an f64 mesh and f64 outputs, computed on the
 * FP32 pipe in pairs of f32 (about 48 significant bits; errors of a few 1e-14 relative to the
 * fields' largest values) where a double-float kernel exists for the element, by the f64 kernels
 * elsewhere; its tables serve the f64 kernels too. */
typedef enum tlg_dtype { TLG_F32 = 4, TLG_F64 = 8, TLG_SPLIT32 = 12, TLG_DF64 = 16 } tlg_dtype;

/* tetraloma_dims::CellType (tetraloma-dims/src/dim.rs). */
typedef enum tlg_cell {
  TLG_POINT = 0,
  TLG_INTERVAL = 1,
  TLG_TRIANGLE = 2,
  TLG_QUADRILATERAL = 3,
  TLG_TETRAHEDRON = 4,
  TLG_HEXAHEDRON = 5,
  TLG_PRISM = 6,
  TLG_PYRAMID = 7
} tlg_cell;

/* tetraloma_refcell::NodeFamily (tetraloma-refcell/src/lagrange.rs:22-27). */
typedef enum tlg_family { TLG_EQUISPACED = 0, TLG_GLL = 1 } tlg_family;

/* Thread-local message of the last failing call on this thread ("" after success). */
const char* tlg_last_error(void);
int tlg_abi_version(void);

/* ---------------------------------------------------------------------------------------
 * Reference cells (host, f64). Replace tetraloma-refcell's public functions
 * (tetraloma-refcell/src/lib.rs:58-69) for callers without the Rust crate.
 * ------------------------------------------------------------------------------------- */

/* num_lagrange_nodes (tetraloma-refcell/src/lagrange.rs:59-78); -1 for an unknown cell. */
int64_t tlg_num_lagrange_nodes(int cell, int degree);

/* lagrange_points (lagrange.rs:163-266): `[node][tdim]` into out (capacity `cap` doubles). */
tlg_status tlg_lagrange_points(int cell, int degree, int family, double* out, int64_t cap);

/* gauss_rule (tetraloma-refcell/src/quadrature.rs:77-128) with `counts[d]` points in collapsed
 * direction d (counts all equal to degree / 2 + 1 gives the reference's rule). Points
 * `[q][tdim]`, weights `[q]`; *num_points receives Q. */
tlg_status tlg_collapsed_rule(int cell, const int* counts, double* points, double* weights,
                              int64_t cap_points, int64_t* num_points);

/* LagrangeElement::tabulate (tetraloma-refcell/src/tabulation.rs:266): `[deriv][q][k]`,
 * deriv 0 the values, 1 + d the derivative in reference direction d (nderivs 0 or 1). */
tlg_status tlg_tabulate(int cell, int degree, int family, const double* points, int64_t npoints,
                        int nderivs, double* out, int64_t cap);

/* reference_facet_normals (tetraloma-refcell/src/facet.rs): `[facet][tdim]`. */
tlg_status tlg_reference_facet_normals(int cell, double* out, int64_t cap);

/* ---------------------------------------------------------------------------------------
 * Tables: the device-resident tabulation of one coordinate element at one point set, in F.
 * Replaces PointSet::tabulate / tabulate_derivatives and their per-element cache
 * (tetraloma-geometry/src/point_set.rs:312-398). Created once, read by every launch.
 * ------------------------------------------------------------------------------------- */
typedef struct tlg_tables tlg_tables;

/* `points` `[q][tdim]` in reference coordinates; `ref_normals` `[q][tdim]` or NULL (the
 * per-point reference facet normals of a FacetPointSet, facet_rule.rs). gdim is the
 * geometric dimension of the grids the tables will serve. Every cell type but the point, pyramids
 * included (their rational Lagrange space, tetraloma-refcell/src/polynomials/pyramid.rs; GLL
 * nodes on intervals, quadrilaterals and hexahedra only, as the reference). Allocates device
 * memory. */
tlg_status tlg_tables_create(int cell, int degree, int family, int gdim, int dtype,
                             const double* points, int64_t npoints, const double* ref_normals,
                             tlg_tables** out);
tlg_status tlg_tables_destroy(tlg_tables* tables);
int64_t tlg_tables_num_points(const tlg_tables* tables);
/* Synchronises `stream` and reports TLG_ERR_DEVICE_TIMEOUT (then clears it) if a kernel that read
 * these tables gave up a bounded wait for its table copy; TLG_OK otherwise. */
tlg_status tlg_tables_device_status(const tlg_tables* tables, void* stream);
int64_t tlg_tables_nodes_per_cell(const tlg_tables* tables);
/* The bounded wait for the table copy, for tests of the timeout path: each of the wait's two
 * rounds polls `polls` times (0: the default 2^22); issue_copy = 0 leaves the copy unissued, so
 * that the wait runs out with nothing in flight: the kernels that read these tables then record
 * TLG_ERR_DEVICE_TIMEOUT (tlg_tables_device_status) and compute nothing, the context stays usable.
 * (0, 1) restores the default. No counterpart in the reference. */
tlg_status tlg_tables_set_wait(tlg_tables* tables, int64_t polls, int issue_copy);

/* ---------------------------------------------------------------------------------------
 * One cell block of a Geometry (tetraloma-geometry/src/geometry.rs:187-288,
 * element.rs:29-154).
 * ------------------------------------------------------------------------------------- */
typedef struct tlg_block {
  int dtype;              /* tlg_dtype of nodes and outputs */
  int gdim;               /* 1, 2 or 3 */
  int64_t num_cells;      /* cells of the block */
  int64_t num_nodes;      /* nodes of the L-vector */
  const void* nodes;      /* device [num_nodes][gdim] F, relative to the origin */
  const uint32_t* dofmap; /* device [num_cells][K] */
  const uint32_t* flags;  /* device [num_flags] cell flags (bit 0 flips normals), or NULL */
  int64_t num_flags;
  double origin[3];       /* host; narrowed to F and added to physical points */
} tlg_block;

/* Outputs of one evaluation: one QuadField chunk range. NULL pointers are not computed. */
typedef struct tlg_outputs {
  int64_t first_cell;     /* first cell of the range, in the block */
  int64_t num_cells;      /* cells of the range, padding excluded */
  int64_t out_first_cell; /* the range's first cell within the output chunks; a multiple of tile */
  int tile;               /* cells per tile: 1, 2, 4, 8 or 16 (the GPU policy's 16) */
  void* points;           /* X, GD components */
  void* jacobian;         /* J, TD * GD */
  void* detj;             /* det J, 1 */
  void* pinv;             /* K, TD * GD */
  void* normals;          /* codimension 1: unit normals, GD */
  void* facet_normals;    /* codimension 0: K^T n_ref / |K^T n_ref|, GD (tables need ref_normals) */
  /* Split precision only (TLG_SPLIT32 tables): points whose condition estimate
   * |J|_F |K|_F / TD exceeds cond_limit (or is not finite) get J, det J and K from FP64; 0
   * selects 256. `recomputed` (device u64, may be NULL) is incremented once per such point. */
  double cond_limit;
  unsigned long long* recomputed;
  /* The measure of each cell of the range, sum_q det J(c, q) w_q in F, into cell_measure[c]
   * (c = 0 .. num_cells - 1, counted from first_cell), summed in point order (d_0 w_0, then one
   * fma per point) over the det J values written to `detj`: the values tlg_measure_cell_sums
   * gives on that field (measure.rs:15-41), so tlg_sum over them is the block's measure. Needs
   * `detj` and `weights` (device [Q] of F); NULL: not computed. The paired kernels sum as they
   * evaluate; the other kernels are followed by a launch that reads det J back. tlg_eval_block
   * and batches only. */
  const void* weights;
  void* cell_measure;
} tlg_outputs;

/* Fused evaluation of every requested factor of one block range in one launch: the
 * connectivity gather, J at each point, and X / J / det J / K / normals / facet normals from
 * it. Replaces `launch_factor` (tetraloma-geometry/src/layout.rs:488-772), which launches one
 * kernel per factor over a gathered E-vector; a single non-NULL output gives exactly that
 * factor. Empty ranges or point sets launch nothing (layout.rs:509-511). */
tlg_status tlg_eval_block(const tlg_tables* tables, const tlg_block* block,
                          const tlg_outputs* outputs, void* stream);

/* ---------------------------------------------------------------------------------------
 * Batches: all blocks of a hybrid mesh (different cell types and degrees) evaluated by one CUDA
 * graph launch, the blocks' persistent kernels running as parallel branches of the graph, their
 * launch shapes picked by an autotuner. Replaces the host loop over blocks of Mesh::per_block
 * (tetraloma/src/mesh.rs:249-257), which launches each factor of each block separately.
 * ------------------------------------------------------------------------------------- */
typedef struct tlg_batch tlg_batch;

/* num_blocks (tables, block, outputs) triples, copied; the pointed-to device memory must stay
 * valid while the batch is used. */
tlg_status tlg_batch_create(const tlg_tables* const* tables, const tlg_block* blocks,
                            const tlg_outputs* outputs, int num_blocks, tlg_batch** out);
tlg_status tlg_batch_destroy(tlg_batch* batch);

/* Times, for each block on `stream` (the median of 7 launches), the strategies whose kernels
 * apply to its tables (the policy, direct, sumfact, cooperative, tensor; none when the caller has
 * set a strategy: an override on this thread or TLG_GEOM_STRATEGY), keeps the fastest (a forced
 * strategy replaces the policy only when more than 3 % faster), then candidate persistent grids
 * (0 and 1..8 CTAs per SM) for it (a grid replaces the occupancy limit only when more than 1 %
 * faster), and caches the choice per launch shape for the process; then, timing the
 * whole graph as it runs in use (the median over 5 rounds of the mean of 4 back-to-back
 * launches), takes parallel branches over a serial chain only when more than 3 % faster in the
 * median and in the slowest round, runs one round of coordinate descent over each block's candidates
 * (changes kept when more than 1 % faster), and keeps the result only when more than 1 % faster
 * than every block at its occupancy limit in a serial chain (cached per batch shape). grids[i]
 * (may be NULL) receives block i's grid (0: the occupancy limit). Runs the blocks' kernels; call
 * it outside stream capture. Rebuilds the graph on the next launch. */
tlg_status tlg_batch_tune(tlg_batch* batch, void* stream, int* grids);

/* After tlg_batch_tune: whether the graph runs the blocks as a serial chain (1) or as parallel
 * branches (0), the tuner's median time of the chosen graph in ms, and per block (strategies may
 * be NULL) the strategy its launch forces on every kernel family (TLG_STRATEGY_*; -1: the
 * caller's, i.e. the override or TLG_GEOM_STRATEGY in effect, else the policy). No counterpart in
 * the reference. */
tlg_status tlg_batch_tuning(const tlg_batch* batch, int* serial, float* ms, int* strategies);

/* Evaluates every block: one launch of a CUDA graph (captured on the first call). */
tlg_status tlg_batch_launch(tlg_batch* batch, void* stream);

/* The E-vector chunk of cells [first_cell, first_cell + chunk_cells): out[(k * gdim + g) * stride
 * + c] for c < roundup(chunk_cells, 16) <= stride, padding lanes repeating the block's last cell
 * and node indices clamped to the last node; a bit-exact gather
 * (tetraloma-geometry/src/evector.rs:195-236, 296-390). */
tlg_status tlg_evector(const tlg_block* block, int nodes_per_cell, int64_t first_cell,
                       int64_t chunk_cells, int64_t stride, void* out, void* stream);

/* ---------------------------------------------------------------------------------------
 * Adjoint: cotangents of the geometric factors mapped back to the node coordinates, for shape
 * optimisation (no counterpart kernel in the reference, which has no adjoint; the sums follow
 * its node-to-cell incidence recipe, tetraloma-topology/src/connectivity.rs:1-3).
 * ------------------------------------------------------------------------------------- */

/* Bytes of workspace tlg_csr_build needs for num_cells cells of nodes_per_cell nodes. */
int64_t tlg_csr_workspace_bytes(int64_t num_cells, int nodes_per_cell);

/* The node-to-(cell, local node) incidence of a dofmap as CSR, by a stable device radix sort:
 * node n's entries e = cell * K + k are entries[offsets[n] .. offsets[n + 1]) in ascending e
 * (offsets has num_nodes + 1 values). Indices past the last node count for the last node, as
 * in the gather. Deterministic. Device pointers; the workspace is caller-provided. */
tlg_status tlg_csr_build(const uint32_t* dofmap, int64_t num_cells, int nodes_per_cell, int64_t num_nodes,
                         void* workspace, int64_t workspace_bytes, uint32_t* offsets, uint32_t* entries,
                         void* stream);

/* Cotangent fields (QuadField chunks of the evaluated range, tile 16); NULL means zero. */
typedef struct tlg_cotangents {
  const void* points;  /* dL/dx, GD components */
  const void* detj;    /* dL/d(det J), or dL/da of the area element below codimension 0 */
  const void* pinv;    /* dL/dK, TD * GD components, K(t, g) at g * TD + t */
  const void* normals; /* dL/dn, GD components (TD + 1 = GD only) */
} tlg_cotangents;

/* Per-cell contributions to the node cotangents of a block range, J, det J and K recomputed:
 * local[(cell * K + k) * R + g] = sum_q phi_k(q) xbar(q, g) + sum_d Jbar(q)(g, d) dphi_k(q)[d],
 * Jbar = dbar det J K^T - K^T Kbar K^T in codimension 0; below it (curves, surfaces: TD < GD)
 * Jbar = dbar a K^T - K^T Kbar K^T + P Kbar^T G^-1 + the normal term (a the area element,
 * G = J^T J, P = I - J K, normals n = s v / |v| with v = J0 x J1 or (J0_y, -J0_x), s from bit 0 of
 * the block's flags; the forward fields may include normals), for the cells of the
 * range (cell = block cell index; rows of R = 4 values for GD = 3, the fourth zero, else R = GD;
 * local holds local_cells >= block->num_cells cells, 16-byte aligned). With
 * TLG_F64 tables everything is f64; with TLG_SPLIT32 tables the mesh is f64, the arithmetic FP32
 * on cell-shifted coordinates, and cotangents, contributions and any forward fields are f32.
 * Forward pointers set in `outputs` (points, jacobian, detj, pinv) are written in the same pass
 * (fused forward + adjoint; no FP64 recompute of ill-conditioned points there);
 * outputs->tile must be 16. */
tlg_status tlg_vjp_block(const tlg_tables* tables, const tlg_block* block, const tlg_outputs* outputs,
                         const tlg_cotangents* cotangents, void* local, int64_t local_cells,
                         void* stream);

/* The contributions of tlg_vjp_block from forward fields already written: outputs->detj and
 * outputs->pinv (det J and K of the range, tiled as tlg_eval_block writes them) are read instead
 * of recomputed, the other output pointers are ignored. Volume cells (TD = GD = 3), f64 or
 * split-precision tables: hexahedra Q1/Q2 at tensor-product rules by the sum-factorised
 * transposed contraction (rows as tlg_vjp_block's sum-factorised adjoint, bit for bit), other
 * cells and rules from the tables' node rows where they and 12 * 16 values per point fit in
 * shared memory; TLG_ERR_UNSUPPORTED otherwise. A forward pass plus this adjoint moves more bytes
 * than the fused pass but needs neither the coordinates nor the forward contraction here. No
 * counterpart in the reference. */
tlg_status tlg_vjp_block_from_fields(const tlg_tables* tables, const tlg_block* block, const tlg_outputs* outputs,
                                     const tlg_cotangents* cotangents, void* local, int64_t local_cells,
                                     void* stream);

/* grad[n * gdim + g] = sum over node n's CSR entries e, in entry order, of local[e * R + g]
 * (R as in tlg_vjp_block; local_dtype 4 or 8 is the contributions' type): f64 sums of f64
 * contributions; f32 contributions summed as an FP32 TwoSum pair (about 48 significant bits)
 * rounded once to f64. Deterministic. */
tlg_status tlg_vjp_gather(const uint32_t* offsets, const uint32_t* entries, int64_t num_nodes,
                          int gdim, const void* local, int local_dtype, double* grad, void* stream);
/* The same sums added onto grad (one f64 addition per node and component), nodes without entries
 * untouched: node cotangents of several blocks, block by block. */
tlg_status tlg_vjp_gather_add(const uint32_t* offsets, const uint32_t* entries, int64_t num_nodes,
                              int gdim, const void* local, int local_dtype, double* grad, void* stream);

/* Adjoint batches (the hybrid mesh's fused forward + adjoint in one CUDA graph launch): per block
 * its tables, block, outputs (forward fields or none), cotangents, contribution rows (local,
 * local_cells as in tlg_vjp_block) and node CSR (tlg_csr_build of its dofmap over num_nodes
 * nodes); grad [num_nodes][gdim] f64; the tables all TLG_SPLIT32 or none. The graph runs every
 * block's tlg_vjp_block on its own branch, then the node sums of tlg_vjp_gather for the first block
 * (every node written, zero where the block has no entries) and of tlg_vjp_gather_add for the
 * others, in block order, eight blocks to a pass over the nodes (the same gradient bit for bit as
 * those calls one after another; no blocks: grad zeroed). Captured on the first launch; the
 * pointers are used as given at every launch. */
typedef struct tlg_vjp_batch tlg_vjp_batch;
tlg_status tlg_vjp_batch_create(const tlg_tables* const* tables, const tlg_block* blocks,
                                const tlg_outputs* outputs, const tlg_cotangents* cotangents,
                                void* const* locals, const int64_t* local_cells,
                                const uint32_t* const* offsets, const uint32_t* const* entries,
                                int64_t num_nodes, int gdim, double* grad, int num_blocks,
                                tlg_vjp_batch** out);
/* Forward fields from other tables: with forward[i] set (num_blocks tables, or NULL to undo), block
 * i's branch runs tlg_eval_block(forward[i], ...) for the batch's forward outputs, then the adjoint
 * from the batch's tables with no forward outputs; e.g. TLG_DF64 tables (f64-accurate fields) with
 * TLG_SPLIT32 adjoint tables (FP32 contributions summed per node in f64). Recaptures on the next
 * launch. No counterpart in the reference, which has no adjoint. */
tlg_status tlg_vjp_batch_set_forward(tlg_vjp_batch* batch, const tlg_tables* const* forward);
/* on = 1: blocks whose adjoint tlg_vjp_block_from_fields serves (and whose outputs include det J
 * and K) run tlg_eval_block (the policy's forward kernel) and then that adjoint on their branch;
 * the others, and every block while forward tables are set, the fused pass. Recaptures on the
 * next launch. No counterpart in the reference. */
tlg_status tlg_vjp_batch_set_two_pass(tlg_vjp_batch* batch, int on);
tlg_status tlg_vjp_batch_launch(tlg_vjp_batch* batch, void* stream);
tlg_status tlg_vjp_batch_destroy(tlg_vjp_batch* batch);

/* ---------------------------------------------------------------------------------------
 * Pull-back (tetraloma-geometry/src/pull_back.rs:94-330, 566): the reference point xi of each
 * physical point of a block by Newton's method on the cell's Lagrange map. Every point starts
 * at the reference cell's vertex centroid (rounded to f32) and runs exactly max_iterations
 * steps delta = K(xi) (y - X(xi)) (K the pseudo-inverse when TD < GD: Gauss-Newton); a point
 * not yet frozen moves to xi + delta clamped to [-0.1, 1.1]^TD, records |delta|_inf (the
 * largest finite value when a component is not finite) and freezes once that is at most the
 * tolerance (<= 0 selects 1e-13 in f64, 1e-5 in f32); frozen points keep xi and their step.
 * A point has converged when its step is at most the tolerance. */
typedef struct tlg_basis tlg_basis;
/* The Lagrange basis of (cell, degree, family) at arbitrary reference points (device). */
tlg_status tlg_basis_create(int cell, int degree, int family, tlg_basis** out);
tlg_status tlg_basis_destroy(tlg_basis* basis);
/* Points x: a QuadField chunk of GD components (absolute coordinates), x_first_cell the range's
 * first cell in it; outputs xi (TD components) and step (1) chunks at out_first_cell; the same
 * tile and num_points for all three. Replaces pull_back_block's kernels. refinements = 0: the
 * iteration in the block's scalar type. refinements > 0 (f64 blocks): mixed precision, the
 * iteration in FP32 on coordinates shifted by the cell's first node (frozen at 1e-5), then that
 * many steps with the residual in FP64 and the correction through the FP32 inverse Jacobian
 * (frozen at the tolerance); xi and step are f64, step that of the last refinement. */
tlg_status tlg_pull_back_block(const tlg_basis* basis, const tlg_block* block, const void* x,
                               int64_t x_first_cell, int64_t first_cell, int64_t num_cells,
                               int64_t out_first_cell, int num_points, int tile, double tolerance,
                               int max_iterations, int refinements, void* xi, void* step,
                               void* stream);

/* ---------------------------------------------------------------------------------------
 * Cell orderings before upload (tetraloma/src/pipeline/order.rs:24-192, builder.rs:95-113):
 * the order in which the kernels visit cells. Host functions (no device). INPUT keeps the
 * order; HILBERT sorts by the Hilbert key of each cell's vertex centroid quantised to 2^21 steps
 * per axis in the node bounding box, then by position; RCM is reverse Cuthill-McKee on the facet
 * graph (components from their least (degree, position) cell, neighbours by (degree,
 * position)). order receives num_cells old cell indices. tlg_number_nodes numbers nodes by
 * first use in `cells` (already in the new order): new_cells receives the renumbered cells and
 * node_order the old node index of each new index (unused nodes last). */
typedef enum tlg_ordering { TLG_ORDER_INPUT = 0, TLG_ORDER_HILBERT = 1, TLG_ORDER_RCM = 2 } tlg_ordering;
tlg_status tlg_order_cells(int ordering, int cell, const uint32_t* cells, int64_t num_cells,
                           int nodes_per_cell, const double* nodes, int64_t num_nodes, int gdim,
                           int64_t* order);
tlg_status tlg_number_nodes(const uint32_t* cells, int64_t num_cells, int nodes_per_cell,
                            int64_t num_nodes, uint32_t* new_cells, int64_t* node_order);
/* The Hilbert index of a point of a grid of 2^bits points per axis (d axes, d * bits <= 64), and
 * the quantisation of a coordinate to [0, 2^21) in [lo, hi]. */
uint64_t tlg_hilbert_key(const uint32_t* x, int d, int bits);
uint32_t tlg_quantise(double x, double lo, double hi);

/* Evaluation strategy (the reference's strategy::choose, tetraloma-geometry/src/strategy.rs:
 * 311-407, with its precedence per kernel family: this thread's setting, then the environment,
 * then the built-in policy; the five strategies of strategy.rs:23-34). AUTO picks per element:
 * for quadrilaterals, hexahedra and prisms at tensor-product point sets, sum factorisation in f64
 * and above the degrees with paired kernels (Q1-Q2, P1-P2) in f32 and split precision; otherwise
 * the paired / unrolled kernels where compiled, the cooperative kernel for cells of more than 27
 * nodes, the loops kernels else (tables staged where they fit: recorded as SHARED, else LOOPS).
 * The others force a kernel family where it applies, and otherwise the
 * loops kernel runs, as in the reference (recorded as LOOPS):
 *  - DIRECT: the paired / unrolled kernels (compiled elements, tile 16 for f32 and split);
 *  - LOOPS: K at run time, tables read from global memory;
 *  - SUMFACT: a quadrilateral, hexahedron or prism at a tensor-product point set, no facet
 *    normals, tile 16 in split precision;
 *  - SHARED: the loops kernels with the tables staged in shared memory (where they fit);
 *  - COOPERATIVE: four lanes per cell (cells of 2 or 3 dimensions, up to 128 nodes, 64 in f64);
 *  - TENSOR (an extension; the reference has none): the node-by-basis contraction on the tensor
 *    cores (mma.sync TF32 in three products, FP32-level error), f32 and split tables, TD >= 2,
 *    tile 16, more than 10 nodes (not in the AUTO policy: no faster than COOPERATIVE here).
 * A fused launch follows the strategy of its principal family: Jacobian when J, det J or K is
 * among its outputs, else Normals, FacetNormals, Points. The adjoint follows the Jacobian family
 * (sum factorisation where it applies, else the node-row kernel); the E-vector and the pull-back
 * have one kernel each (recorded as LOOPS: K and the degree at run time). The environment variable
 * TLG_GEOM_STRATEGY is read once: one strategy name (policy or auto, direct, loops, sumfact,
 * shared, cooperative, tensor) for every family, or a comma list <family>=<strategy> of the families
 * EVector, Points, Jacobian, Normals, FacetNormals, PullBack (each at most once); an invalid value
 * makes every launch fail with TLG_ERR_INVALID_ARGUMENT. tlg_set_strategy sets this thread's
 * setting of every family, tlg_set_family_strategy of one (-1 clears it, 0 selects the policy). */
typedef enum tlg_kernel_family {
  TLG_FAMILY_EVECTOR = 0,
  TLG_FAMILY_POINTS = 1,
  TLG_FAMILY_JACOBIAN = 2,
  TLG_FAMILY_NORMALS = 3,
  TLG_FAMILY_FACET_NORMALS = 4,
  TLG_FAMILY_PULL_BACK = 5
} tlg_kernel_family;
typedef enum tlg_strategy {
  TLG_STRATEGY_AUTO = 0,
  TLG_STRATEGY_DIRECT = 1,
  TLG_STRATEGY_LOOPS = 2,
  TLG_STRATEGY_SUMFACT = 3,
  TLG_STRATEGY_SHARED = 4,
  TLG_STRATEGY_COOPERATIVE = 5,
  TLG_STRATEGY_TENSOR = 6
} tlg_strategy;
tlg_status tlg_set_strategy(int strategy);
tlg_status tlg_set_family_strategy(int family, int strategy);
/* This thread's setting of a family (-1: none). */
int tlg_get_family_override(int family);
/* The strategy in effect for a family (setting, environment, policy). */
tlg_status tlg_get_family_strategy(int family, int* strategy);
/* The strategy in effect for the Jacobian family; -1 when the environment variable is invalid. */
int tlg_get_strategy(void);
/* The strategy that ran in this thread's last launch (tlg_eval_block, tlg_vjp_block, tlg_evector,
 * tlg_pull_back_block): DIRECT (paired or unrolled), LOOPS, SUMFACT, SHARED or COOPERATIVE; 0
 * before any (the reference's record_strategies test hook, tetraloma-geometry/src/testing.rs:
 * 34-43). */
int tlg_last_kernel_family(void);
/* The family (TLG_FAMILY_*) whose strategy decided that launch; -1 before any. */
int tlg_last_launch_family(void);

/* ---------------------------------------------------------------------------------------
 * Measure (tetraloma-geometry/src/measure.rs:15-185): per-cell sums of det J * w over the
 * points of a det J QuadField chunk, then a sum tree of 64-value blocks, all in F and in a
 * fixed order. The caller reads the F result (the reference finishes it in f64 on the host).
 * ------------------------------------------------------------------------------------- */

/* sums[c] = sum_q detj(c, q) * weights[q] for the chunk's cells (cell_sums_kernel, measure.rs:
 * 15-41); detj is a QuadField chunk of tile `tile`, weights device [num_points] of F. */
tlg_status tlg_measure_cell_sums(const void* detj, int dtype, int64_t num_cells, int64_t num_points,
                                 int tile, const void* weights, void* sums, void* stream);

/* Bytes of workspace tlg_sum needs for n values (-1 for a bad dtype). */
int64_t tlg_sum_workspace_bytes(int dtype, int64_t n);

/* result[0] = the sum of x[0..n) by levels of 64-value block sums (measure.rs:44-102); result
 * and workspace are device memory; an empty input sums to 0. */
tlg_status tlg_sum(const void* x, int dtype, int64_t n, void* workspace, int64_t workspace_bytes,
                   void* result, void* stream);

/* The measure of one det J chunk without any device allocation, for callers that cannot call
 * cudaMalloc: hosts whose device memory is owned by another allocator (a caching allocator or a
 * pool that reserves the free memory up front, as PyTorch's and CubeCL's runtimes do), where an
 * extra cudaMalloc can fail and a cudaFree synchronises the whole device. No counterpart in the
 * reference, whose measure_block allocates its per-cell sums (measure.rs:141-185).
 *
 * Same inputs and the same result bits as tlg_measure_cell_sums followed by tlg_sum: the caller
 * passes det J (a QuadField chunk), the weights and a device result of F. The sum tree's
 * levels live in one fixed array of 2,130,944 bytes inside this library, which every GPU that
 * loads the library holds until the process exits; chunks of more than
 * tlg_measure_static_max_cells() = 16,777,216 cells are rejected with
 * TLG_ERR_ALLOCATION_TOO_LARGE. The first call on each device looks up the array's device
 * address (with that device current); make that first call before any stream capture. Later calls
 * check that the address is still the device's (one runtime query) and look it up again after a
 * device reset. Every call
 * shares the array: calls whose kernels may overlap on the GPU (other streams, other threads)
 * race and must be serialised by the caller. No value of the array needs to start at zero:
 * each is written before it is read. */
tlg_status tlg_measure_static(const void* detj, int dtype, int64_t num_cells, int64_t num_points,
                              int tile, const void* weights, void* result, void* stream);
int64_t tlg_measure_static_max_cells(void);
/* The same measure with a workspace of the caller (no size limit, no shared scratch):
 * tlg_measure_workspace_bytes(dtype, num_cells) bytes, 0 for up to 64 cells; -1 for bad
 * arguments. Level 1 of the tree comes straight from the det J field (one launch fewer than
 * tlg_measure_cell_sums + tlg_sum), with the same bits. */
int64_t tlg_measure_workspace_bytes(int dtype, int64_t num_cells);
tlg_status tlg_measure(const void* detj, int dtype, int64_t num_cells, int64_t num_points, int tile,
                       const void* weights, void* workspace, int64_t workspace_bytes, void* result,
                       void* stream);

/* Self-test of the split kernels' integer f64 -> f32 rounding and f32 -> f64 widening against
 * the conversion instructions: mismatches[0] += the number of x[0..n) (device f64 values) whose
 * rounded f32 bits differ, mismatches[1] += those whose widened round trip differs (NaN
 * payloads compared as NaN). No counterpart in the reference. */
tlg_status tlg_selftest_conversions(const double* x, int64_t n, unsigned long long* mismatches,
                                    void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TLGEOM_H */
