"""The host side of the geometry path, mirroring tetraloma-geometry's public API over the C ABI.

Names, argument meaning and error kinds follow the reference (paths inside its project):

- :class:`CoordinateElement`, :class:`GeometryBlock` — tetraloma-geometry/src/element.rs:29-154;
- :class:`Geometry` — tetraloma-geometry/src/geometry.rs:187-288: node L-vector relative to the
  origin, per-block dofmaps, the E-vector cache; ``Geometry.new`` checks lengths only;
- :class:`PointSet`, :class:`QuadRule` — point_set.rs:57-398 and rule.rs:49-104; a point set
  caches its device tables per (element, scalar type, gdim), as the reference caches its
  tabulations;
- :class:`QuadField` — field.rs:162-409, one tiled chunk per field (or several when
  ``max_chunk_cells`` is given), ``to_host_cell_major`` undoes the tiling;
- ``physical_points_block``, ``jacobians_block``, ``detj_block``, ``pseudo_inverse_block``,
  ``normals_block``, ``facet_normals_block`` — points_jac.rs:637,685, detj_pinv.rs:739,787,
  facets.rs:46,107, all through one launcher like ``launch_factor`` (layout.rs:488-772);
  ``geometric_factors_block`` computes several factors in one fused launch.

Device memory, streams and tensors come from PyTorch; every computation runs in the native
library (``libtlgeom.so``). Mesh arrays are torch tensors on the current CUDA device.
"""

from __future__ import annotations

import ctypes
import dataclasses
from typing import Iterable

import numpy as np
import torch

from . import refcell
from .strategy import _note_launch
from ._lib import CELL_IDS, FAMILY_IDS, GridError, TlgBlock, TlgOutputs, check, lib

VECTOR_PAD = 16  # tetraloma-device/src/buffer.rs:28
GPU_QUAD_TILE = 16  # tetraloma-device/vector-policy.toml:59

FACTOR_LEN = {
    "points": lambda td, gd: gd,
    "jacobian": lambda td, gd: td * gd,
    "detj": lambda td, gd: 1,
    "pinv": lambda td, gd: td * gd,
    "normals": lambda td, gd: gd,
    "facet_normals": lambda td, gd: gd,
}

_DTYPES = {torch.float32: 4, torch.float64: 8}


def current_stream_handle() -> int:
    return torch.cuda.current_stream().cuda_stream


@dataclasses.dataclass(frozen=True)
class CoordinateElement:
    cell: str
    degree: int
    family: str = "Equispaced"

    @property
    def nodes_per_cell(self) -> int:
        return refcell.num_lagrange_nodes(self.cell, self.degree)

    @property
    def tdim(self) -> int:
        return refcell.tdim(self.cell)


@dataclasses.dataclass
class GeometryBlock:
    """One cell block: its coordinate element, dofmap ``[cells][K]`` (u32 bit patterns held in an
    int32 tensor) and cell flags (bit 0 flips normals)."""

    element: CoordinateElement
    dofmap: torch.Tensor
    flags: torch.Tensor | None = None

    @property
    def num_cells(self) -> int:
        return self.dofmap.shape[0]


@dataclasses.dataclass
class EVectorChunk:
    first_cell: int
    num_cells: int
    data: torch.Tensor  # [K][GD][stride]


class Geometry:
    """Blocks of one grid, the node L-vector relative to `origin`, and the E-vector cache."""

    def __init__(self, blocks: list, nodes: torch.Tensor, origin):
        gd = nodes.shape[1] if nodes.dim() == 2 else 0
        if nodes.dtype not in _DTYPES:
            raise GridError(1, f"nodes must be float32 or float64, not {nodes.dtype}")
        if not nodes.is_cuda:
            raise GridError(1, "nodes must be a CUDA tensor")
        for b in blocks:
            k = b.element.nodes_per_cell
            if b.dofmap.dim() != 2 or b.dofmap.shape[1] != k:
                raise GridError(2, f"LengthMismatch {{ expected: {k}, found: {tuple(b.dofmap.shape)} }}")
            if nodes.shape[0] == 0 and b.dofmap.numel() != 0:
                raise GridError(2, "LengthMismatch { expected: 0 cells without nodes }")
            if b.dofmap.dtype != torch.int32 or not b.dofmap.is_cuda or not b.dofmap.is_contiguous():
                raise GridError(1, "dofmap must be a contiguous int32 CUDA tensor of u32 indices")
        self.blocks = blocks
        self.nodes = nodes.contiguous()
        self.gdim = gd
        self.origin = tuple(float(x) for x in origin) + (0.0,) * (3 - len(tuple(origin)))
        self._evectors: dict[int, list[EVectorChunk]] = {}

    @property
    def dtype(self) -> torch.dtype:
        return self.nodes.dtype

    @classmethod
    def from_host(cls, mesh, dtype=torch.float64, device="cuda", flags=None) -> "Geometry":
        """Uploads a host mesh: origin = centre of the bounding box, nodes stored as
        F(x - origin) (tetraloma/src/pipeline/nodes.rs:39-45, upload.rs:65-73)."""
        x = np.asarray(mesh.nodes, dtype=np.float64)
        if x.shape[0]:
            origin = 0.5 * (x.min(axis=0) + x.max(axis=0))
        else:
            origin = np.zeros(mesh.gdim)
        rel = x - origin
        nodes = torch.from_numpy(np.ascontiguousarray(rel)).to(dtype=dtype).to(device)
        blocks = []
        for i, hb in enumerate(mesh.blocks):
            dm = torch.from_numpy(np.ascontiguousarray(hb.cells.astype(np.uint32).view(np.int32))).to(device)
            fl = None
            if flags is not None and flags[i] is not None:
                fl = torch.from_numpy(np.ascontiguousarray(np.asarray(flags[i], dtype=np.uint32).view(np.int32))).to(device)
            blocks.append(GeometryBlock(CoordinateElement(hb.cell, hb.degree, hb.family), dm, fl))
        return cls(blocks, nodes, origin)

    def block_desc(self, b: int) -> TlgBlock:
        blk = self.blocks[b]
        d = TlgBlock()
        d.dtype = _DTYPES[self.dtype]
        d.gdim = self.gdim
        d.num_cells = blk.num_cells
        d.num_nodes = self.nodes.shape[0]
        d.nodes = self.nodes.data_ptr()
        d.dofmap = blk.dofmap.data_ptr()
        d.flags = blk.flags.data_ptr() if blk.flags is not None else None
        d.num_flags = blk.flags.numel() if blk.flags is not None else 0
        for g in range(3):
            d.origin[g] = self.origin[g]
        return d

    def evector(self, b: int, max_chunk_cells: int | None = None) -> list[EVectorChunk]:
        """Block b's E-vector, built on first use and cached (geometry.rs:462-488): chunks of
        ``[K][GD][stride]`` with stride = chunk cells rounded up to 16, padding lanes
        repeating the block's last cell (evector.rs:296-390)."""
        if b in self._evectors and max_chunk_cells is None:
            return self._evectors[b]
        blk = self.blocks[b]
        k, gd, n = blk.element.nodes_per_cell, self.gdim, blk.num_cells
        per = n if max_chunk_cells is None else max(VECTOR_PAD, max_chunk_cells // VECTOR_PAD * VECTOR_PAD)
        chunks = []
        desc = self.block_desc(b)
        first = 0
        while first < n:
            cnt = min(per, n - first)
            stride = -(-cnt // VECTOR_PAD) * VECTOR_PAD
            data = torch.empty((k, gd, stride), dtype=self.dtype, device=self.nodes.device)
            check(lib().tlg_evector(ctypes.byref(desc), k, first, cnt, stride, data.data_ptr(),
                                    current_stream_handle()))
            _note_launch()
            chunks.append(EVectorChunk(first, cnt, data))
            first += cnt
        if max_chunk_cells is None:
            self._evectors[b] = chunks
        return chunks


class PointSet:
    """Reference points and weights of one cell type; caches the device tables of each element
    it is tabulated for (point_set.rs:57-398)."""

    def __init__(self, cell: str, points, weights, ref_normals=None):
        td = refcell.tdim(cell)
        self.cell = cell
        self.points = np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(-1, td))
        self.weights = np.ascontiguousarray(np.asarray(weights, dtype=np.float64).reshape(-1))
        if self.points.shape[0] != self.weights.shape[0]:
            raise GridError(2, "points and weights differ in count")
        self.ref_normals = None if ref_normals is None else np.ascontiguousarray(
            np.asarray(ref_normals, dtype=np.float64).reshape(-1, td))
        self._tables: dict = {}
        self._weights_dev: dict = {}

    def __len__(self) -> int:
        return self.points.shape[0]

    def tables(self, element: CoordinateElement, gdim: int, dtype):
        """Device tables for `element`; `dtype` is a torch dtype or the ABI code 12 for the
        split-precision tables (f32 tables plus the f64 derivative table)."""
        code = dtype if isinstance(dtype, int) else _DTYPES[dtype]
        key = (element, gdim, code)
        t = self._tables.get(key)
        if t is None:
            if element.cell != self.cell:
                raise GridError(1, f"a {self.cell} point set cannot tabulate a {element.cell} element")
            h = ctypes.c_void_p()
            pts = self.points if len(self) else np.zeros(1)
            rn = None if self.ref_normals is None else self.ref_normals.ctypes.data_as(ctypes.c_void_p)
            check(lib().tlg_tables_create(CELL_IDS[element.cell], element.degree,
                                          FAMILY_IDS[element.family], gdim, code,
                                          pts.ctypes.data_as(ctypes.c_void_p), len(self), rn,
                                          ctypes.byref(h)))
            t = _Tables(h)
            self._tables[key] = t
        return t

    def weights_device(self, dtype: torch.dtype, device="cuda") -> torch.Tensor:
        w = self._weights_dev.get(dtype)
        if w is None:
            w = torch.from_numpy(self.weights).to(dtype=dtype).to(device)
            self._weights_dev[dtype] = w
        return w


class _Tables:
    def __init__(self, handle: ctypes.c_void_p):
        self.handle = handle

    def __del__(self):
        try:
            lib().tlg_tables_destroy(self.handle)
        except Exception:
            pass


class QuadRule:
    """One point set per distinct cell type (rule.rs:49-104)."""

    def __init__(self, sets: Iterable[PointSet]):
        self.sets = list(sets)

    @classmethod
    def gauss(cls, cells: Iterable[str], degree: int) -> "QuadRule":
        out = []
        for c in dict.fromkeys(cells):
            pts, w = refcell.gauss_rule(c, degree)
            out.append(PointSet(c, pts, w))
        return cls(out)

    @classmethod
    def for_grid(cls, g: Geometry, degree: int) -> "QuadRule":
        return cls.gauss([b.element.cell for b in g.blocks], degree)

    def get(self, cell: str) -> PointSet:
        for s in self.sets:
            if s.cell == cell:
                return s
        raise GridError(1, f"CellNotInRule({cell})")


@dataclasses.dataclass
class QuadChunk:
    first_cell: int
    num_cells: int
    data: torch.Tensor  # flat, padded cells * Q * LEN


class QuadField:
    """Values at the points of one block, tiled: component k at point q of cell c at
    ((c / tile) Q LEN + q LEN + k) tile + c % tile within its chunk (field.rs:121-162)."""

    def __init__(self, chunks, num_cells: int, num_points: int, length: int, tile: int):
        self.chunks = chunks
        self.num_cells = num_cells
        self.num_points = num_points
        self.length = length
        self.tile = tile

    @classmethod
    def uninit(cls, num_cells: int, num_points: int, length: int, tile: int, dtype,
               device="cuda", max_chunk_cells: int | None = None) -> "QuadField":
        if tile not in (1, 2, 4, 8, 16):
            raise GridError(1, f"QuadField::uninit: tile {tile} is not 1, 2, 4, 8 or 16")
        per = num_cells if not max_chunk_cells else max(tile, max_chunk_cells // tile * tile)
        chunks, first = [], 0
        while first < num_cells:
            n = min(per, num_cells - first)
            padded = -(-n // tile) * tile
            chunks.append(QuadChunk(first, n, torch.empty(padded * num_points * length,
                                                          dtype=dtype, device=device)))
            first += n
        return cls(chunks, num_cells, num_points, length, tile)

    def to_host_cell_major(self) -> np.ndarray:
        """``[cell][point][component]`` on the host, padding excluded (field.rs:380-408)."""
        parts = []
        for ch in self.chunks:
            t, q, l = self.tile, self.num_points, self.length
            nt = -(-ch.num_cells // t)
            a = ch.data.detach().cpu().numpy().reshape(nt, q, l, t).transpose(0, 3, 1, 2)
            parts.append(a.reshape(nt * t, q, l)[: ch.num_cells])
        if not parts:
            return np.zeros((0, self.num_points, self.length))
        return np.concatenate(parts, axis=0)


def _factor_names(g: Geometry, b: int, factors) -> list:
    td = g.blocks[b].element.tdim
    names = list(factors)
    for f in names:
        if f not in FACTOR_LEN:
            raise GridError(1, f"unknown factor {f}")
    if "normals" in names and td + 1 != g.gdim:
        raise GridError(1, "normals need a block of codimension 1")
    if "facet_normals" in names and td != g.gdim:
        raise GridError(1, "facet normals need a block of codimension 0")
    return names


SPLIT32 = 12  # ABI code of the split-precision tables
DF64 = 16  # ABI code of the double-float tables (f64 fields computed on the FP32 pipe)


def geometric_factors_block(g: Geometry, b: int, pts: PointSet, factors=("points", "jacobian", "detj", "pinv"),
                            tile: int = GPU_QUAD_TILE, max_chunk_cells: int | None = None,
                            out: dict | None = None, precision: str = "native",
                            cond_limit: float = 0.0, recomputed: torch.Tensor | None = None,
                            cell_measure: torch.Tensor | None = None) -> dict:
    """Every factor in `factors` of block b at the points of `pts`, in one fused launch per
    chunk; returns ``{factor: QuadField}``. `out` may pass preallocated fields.

    `cell_measure` (a contiguous CUDA tensor of the fields' type, one value per cell; "detj" among
    the factors) receives each cell's sum of det J * w over the points, the values
    :func:`measure_block` sums; the paired kernels add them up as they evaluate.

    ``precision="native"`` computes in the mesh's scalar type. ``precision="split"`` (f64 meshes)
    computes in FP32 on cell-shifted coordinates and returns f32 fields; points whose condition
    estimate exceeds `cond_limit` (0: 256) get det J and K from FP64, and `recomputed` (an int64
    CUDA tensor of one element) counts them. ``precision="df64"`` (f64 meshes) returns f64 fields
    computed in double-float arithmetic on the FP32 pipe (pairs of f32, about 48 significant bits)
    where the library has a double-float kernel for the element, and by the f64 kernels
    elsewhere."""
    blk = g.blocks[b]
    names = _factor_names(g, b, factors)
    td, gd = blk.element.tdim, g.gdim
    nq = len(pts)
    if precision == "split":
        if g.dtype != torch.float64:
            raise GridError(1, "split precision evaluates f64 meshes")
        tables = pts.tables(blk.element, gd, SPLIT32)
        out_dtype = torch.float32
    elif precision == "df64":
        if g.dtype != torch.float64:
            raise GridError(1, "double-float precision evaluates f64 meshes")
        tables = pts.tables(blk.element, gd, DF64)
        out_dtype = torch.float64
    elif precision == "native":
        tables = pts.tables(blk.element, gd, g.dtype)
        out_dtype = g.dtype
    else:
        raise GridError(1, f"unknown precision {precision!r}")
    fields = out if out is not None else {
        f: QuadField.uninit(blk.num_cells, nq, FACTOR_LEN[f](td, gd), tile, out_dtype,
                            g.nodes.device, max_chunk_cells)
        for f in names}
    desc = g.block_desc(b)
    stream = current_stream_handle()
    nchunks = len(next(iter(fields.values())).chunks) if fields else 0
    wptr = None
    if cell_measure is not None:
        if "detj" not in names:
            raise GridError(1, "cell_measure needs detj among the factors")
        if (cell_measure.dtype != out_dtype or not cell_measure.is_cuda or not cell_measure.is_contiguous()
                or cell_measure.numel() < blk.num_cells):
            raise GridError(1, f"cell_measure must be a contiguous CUDA {out_dtype} tensor of {blk.num_cells} values")
        wptr = pts.weights_device(out_dtype, cell_measure.device).data_ptr()
    for ci in range(nchunks):
        o = TlgOutputs()
        ch0 = fields[names[0]].chunks[ci]
        o.first_cell = ch0.first_cell
        o.num_cells = ch0.num_cells
        o.out_first_cell = 0
        o.tile = tile
        o.cond_limit = cond_limit
        o.recomputed = recomputed.data_ptr() if recomputed is not None else None
        for f in names:
            setattr(o, f, fields[f].chunks[ci].data.data_ptr())
        if cell_measure is not None:
            o.weights = wptr
            o.cell_measure = cell_measure.data_ptr() + ch0.first_cell * cell_measure.element_size()
        check(lib().tlg_eval_block(tables.handle, ctypes.byref(desc), ctypes.byref(o), stream))
        _note_launch()
    return fields


def physical_points_block(g: Geometry, b: int, pts: PointSet, **kw) -> QuadField:
    return geometric_factors_block(g, b, pts, ("points",), **kw)["points"]


def jacobians_block(g: Geometry, b: int, pts: PointSet, **kw) -> QuadField:
    return geometric_factors_block(g, b, pts, ("jacobian",), **kw)["jacobian"]


def detj_block(g: Geometry, b: int, pts: PointSet, **kw) -> QuadField:
    return geometric_factors_block(g, b, pts, ("detj",), **kw)["detj"]


def pseudo_inverse_block(g: Geometry, b: int, pts: PointSet, **kw) -> QuadField:
    return geometric_factors_block(g, b, pts, ("pinv",), **kw)["pinv"]


def normals_block(g: Geometry, b: int, pts: PointSet, **kw) -> QuadField:
    return geometric_factors_block(g, b, pts, ("normals",), **kw)["normals"]


def facet_normals_block(g: Geometry, b: int, pts: PointSet, **kw) -> QuadField:
    if pts.ref_normals is None:
        raise GridError(1, "facet normals need a facet point set (with reference normals)")
    return geometric_factors_block(g, b, pts, ("facet_normals",), **kw)["facet_normals"]


def facet_point_set(cell: str, degree: int) -> PointSet:
    """The facet Gauss rule of `cell` mapped to the cell, facet by facet, with each point's
    reference facet normal (tetraloma-geometry/src/facet_rule.rs:16-70)."""
    td = refcell.tdim(cell)
    normals = refcell.reference_facet_normals(cell)
    from ._facets import facet_points_to_cell, facet_types
    pts, w, rn = [], [], []
    for f, ft in enumerate(facet_types(cell)):
        fp, fw = refcell.gauss_rule(ft, degree)
        pts.append(facet_points_to_cell(cell, f, fp))
        w.append(fw)
        rn.append(np.repeat(normals[f:f + 1], fw.size, axis=0))
    return PointSet(cell, np.concatenate(pts).reshape(-1, td), np.concatenate(w),
                    np.concatenate(rn).reshape(-1, td))


def measure_block(g: Geometry, b: int, pts: PointSet, detj: QuadField | None = None,
                  sync: bool = True, cell_sums: torch.Tensor | None = None):
    """The measure of block b: sum over cells and points of det J * w, per cell then by a tree of
    64-value sums, all on the device in the det J field's type, read back once
    (tetraloma-geometry/src/measure.rs:141-185). `detj` may pass an already computed det J field
    of the same point set (an f32 field of split precision sums in f32). With ``sync=False`` the
    result stays on the device: a one-element tensor, ready when the current stream reaches it.
    `cell_sums` may pass the per-cell sums an evaluation wrote (its ``cell_measure``); only the
    tree over them runs then."""
    blk = g.blocks[b]
    dev = g.nodes.device
    if blk.num_cells == 0 or len(pts) == 0:
        return 0.0 if sync else torch.zeros(1, dtype=g.dtype, device=dev)
    if cell_sums is not None:
        dt = cell_sums.dtype
        if (dt not in _DTYPES or not cell_sums.is_cuda or not cell_sums.is_contiguous()
                or cell_sums.numel() < blk.num_cells):
            raise GridError(1, f"cell_sums must be a contiguous CUDA f32 or f64 tensor of {blk.num_cells} values")
        nbytes = int(lib().tlg_sum_workspace_bytes(_DTYPES[dt], blk.num_cells))
        work = torch.empty(max(nbytes, 8), dtype=torch.uint8, device=dev)
        result = torch.empty(1, dtype=dt, device=dev)
        check(lib().tlg_sum(cell_sums.data_ptr(), _DTYPES[dt], blk.num_cells, work.data_ptr(), nbytes,
                            result.data_ptr(), current_stream_handle()))
        return float(result.item()) if sync else result
    if detj is None:
        detj = detj_block(g, b, pts)
    dt = detj.chunks[0].data.dtype
    es = _DTYPES[dt]
    w = pts.weights_device(dt, dev)
    stream = current_stream_handle()
    if len(detj.chunks) == 1:  # one launch for the cell sums and the tree's first level
        nbytes = int(lib().tlg_measure_workspace_bytes(es, blk.num_cells))
        work = torch.empty(max(nbytes, es), dtype=torch.uint8, device=dev)  # stream-ordered reuse
        result = torch.empty(1, dtype=dt, device=dev)
        check(lib().tlg_measure(detj.chunks[0].data.data_ptr(), es, blk.num_cells, detj.num_points, detj.tile,
                                w.data_ptr(), work.data_ptr(), nbytes, result.data_ptr(), stream))
        return float(result.item()) if sync else result
    sums = torch.empty(blk.num_cells, dtype=dt, device=dev)
    for ch in detj.chunks:
        check(lib().tlg_measure_cell_sums(ch.data.data_ptr(), es, ch.num_cells, detj.num_points,
                                          detj.tile, w.data_ptr(),
                                          sums.data_ptr() + ch.first_cell * es, stream))
    nbytes = int(lib().tlg_sum_workspace_bytes(es, blk.num_cells))
    work = torch.empty(max(nbytes, es), dtype=torch.uint8, device=dev)
    result = torch.empty(1, dtype=dt, device=dev)
    check(lib().tlg_sum(sums.data_ptr(), es, blk.num_cells, work.data_ptr(), nbytes,
                        result.data_ptr(), stream))
    return float(result.item()) if sync else result


_BASES: dict = {}


def _basis(el: CoordinateElement):
    """The device Lagrange basis at arbitrary points of a coordinate element (cached)."""
    key = (el.cell, el.degree, el.family)
    h = _BASES.get(key)
    if h is None:
        h = ctypes.c_void_p()
        check(lib().tlg_basis_create(CELL_IDS[el.cell], el.degree, FAMILY_IDS[el.family], ctypes.byref(h)))
        _BASES[key] = h
    return h


def pull_back_block(g: Geometry, b: int, x: QuadField, tolerance: float | None = None,
                    max_iterations: int = 16, precision: str = "native", refinements: int = 3):
    """Reference points of the physical points `x` (a QuadField of block b, GD components) by
    Newton's method (tetraloma-geometry/src/pull_back.rs:566): returns ``(xi, step)``, xi with
    TD components and step = |delta xi|_inf of each point's last iteration, tiled and chunked as
    `x`. Every point starts at the reference cell's vertex centroid and runs `max_iterations`
    steps (no early exit), clamped to [-0.1, 1.1]^TD and frozen once its step is at most the
    tolerance (None: 1e-13 in f64, 1e-5 in f32); a point has converged when its step is at most
    the tolerance.

    ``precision="split"`` (f64 meshes): the iteration in FP32 on cell-shifted coordinates, then
    `refinements` steps with the residual in FP64 and the correction through the FP32 inverse
    Jacobian; xi and step are f64, step that of the last refinement."""
    blk = g.blocks[b]
    td = blk.element.tdim
    if x.num_cells != blk.num_cells:
        raise GridError(2, f"LengthMismatch {{ expected: {blk.num_cells}, found: {x.num_cells} }}")
    if x.length != g.gdim:
        raise GridError(1, f"pull_back_block: points of {x.length} components on a grid of dimension {g.gdim}")
    if max_iterations < 0:
        raise GridError(1, "pull_back_block: max_iterations must be >= 0")
    if precision not in ("native", "split"):
        raise GridError(1, f"unknown precision {precision!r}")
    if precision == "split" and (g.dtype != torch.float64 or refinements < 1):
        raise GridError(1, "pull_back_block: split precision refines f64 meshes (refinements >= 1)")
    nref = refinements if precision == "split" else 0
    nq, tile = x.num_points, x.tile
    xi_chunks, step_chunks = [], []
    for ch in x.chunks:
        if ch.data.dtype != g.dtype:
            raise GridError(1, f"pull_back_block: points of {ch.data.dtype} on a {g.dtype} grid")
        padded = -(-ch.num_cells // tile) * tile
        xi_chunks.append(QuadChunk(ch.first_cell, ch.num_cells,
                                   torch.empty(padded * nq * td, dtype=g.dtype, device=g.nodes.device)))
        step_chunks.append(QuadChunk(ch.first_cell, ch.num_cells,
                                     torch.empty(padded * nq, dtype=g.dtype, device=g.nodes.device)))
    xi = QuadField(xi_chunks, blk.num_cells, nq, td, tile)
    step = QuadField(step_chunks, blk.num_cells, nq, 1, tile)
    if blk.num_cells == 0 or nq == 0:
        return xi, step
    h = _basis(blk.element)
    desc = g.block_desc(b)
    stream = current_stream_handle()
    tol = 0.0 if tolerance is None else float(tolerance)
    for ch, cxi, cst in zip(x.chunks, xi_chunks, step_chunks):
        check(lib().tlg_pull_back_block(h, ctypes.byref(desc), ch.data.data_ptr(), 0, ch.first_cell,
                                        ch.num_cells, 0, nq, tile, tol, max_iterations, nref,
                                        cxi.data.data_ptr(), cst.data.data_ptr(), stream))
        _note_launch()
    return xi, step


@dataclasses.dataclass
class NodeIncidence:
    """Node-to-(cell, local node) CSR of one block: node n's dofmap entries e = cell * K + k
    are ``entries[offsets[n]:offsets[n + 1]]`` in ascending e (u32 bit patterns in int32)."""

    offsets: torch.Tensor
    entries: torch.Tensor


def node_incidence(g: Geometry, b: int) -> NodeIncidence:
    """The block's CSR, built on the device by a stable radix sort and cached on the grid."""
    cache = g.__dict__.setdefault("_incidence", {})
    if b in cache:
        return cache[b]
    blk = g.blocks[b]
    k = blk.element.nodes_per_cell
    nn = g.nodes.shape[0]
    dev = g.nodes.device
    offsets = torch.empty(nn + 1, dtype=torch.int32, device=dev)
    entries = torch.empty(max(blk.num_cells * k, 1), dtype=torch.int32, device=dev)
    nbytes = int(lib().tlg_csr_workspace_bytes(blk.num_cells, k))
    work = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=dev)
    check(lib().tlg_csr_build(blk.dofmap.data_ptr(), blk.num_cells, k, nn, work.data_ptr(), nbytes,
                              offsets.data_ptr(), entries.data_ptr(), current_stream_handle()))
    inc = NodeIncidence(offsets, entries)
    cache[b] = inc
    return inc


def vjp_block(g: Geometry, b: int, pts: PointSet, cotangents: dict, precision: str = "native",
              forward=(), out: dict | None = None, local: torch.Tensor | None = None,
              from_fields: dict | None = None):
    """Cotangents of the node coordinates (``[node][GD]`` f64) for the cotangent fields
    ``{"points", "detj", "pinv", "normals"}`` (QuadFields of tile 16, f64, or f32 with
    ``precision="split"``; missing entries are zero; "detj" is the area element and "normals"
    the unit normals of curves and surfaces, TD + 1 = GD) of block b. J, det J and K are
    recomputed. The factors named in `forward` are evaluated in the same pass (fused forward +
    adjoint) and returned: ``(grad, fields)``.

    `from_fields`: the "detj" and "pinv" fields of a forward evaluation of the same block and
    points already run (tile 16, the adjoint's field dtype); the adjoint reads them instead of
    recomputing them (``tlg_vjp_block_from_fields``: volume cells)."""
    from ._lib import TlgCotangents

    blk = g.blocks[b]
    td, gd = blk.element.tdim, g.gdim
    if g.dtype != torch.float64:
        raise GridError(1, "the adjoint reads f64 meshes")
    if precision == "split":
        tables = pts.tables(blk.element, gd, SPLIT32)
        fdt = torch.float32
    elif precision == "native":
        tables = pts.tables(blk.element, gd, g.dtype)
        fdt = torch.float64
    else:
        raise GridError(1, f"unknown precision {precision!r}")
    for name in forward:
        if name not in ("points", "jacobian", "detj", "pinv", "normals") or (name == "normals" and td + 1 != gd):
            raise GridError(1, f"no fused forward factor {name}")
    k = blk.element.nodes_per_cell
    nq = len(pts)
    dev = g.nodes.device
    fields = out if out is not None else {
        f: QuadField.uninit(blk.num_cells, nq, FACTOR_LEN[f](td, gd), GPU_QUAD_TILE, fdt, dev)
        for f in forward}
    if local is None:
        local = torch.empty((max(blk.num_cells, 1), k, 4 if gd == 3 else gd), dtype=fdt, device=dev)
    ct = TlgCotangents()
    for name in ("points", "detj", "pinv", "normals"):
        f = cotangents.get(name)
        if f is not None:
            if f.tile != GPU_QUAD_TILE or len(f.chunks) != 1 or f.chunks[0].data.dtype != fdt:
                raise GridError(1, f"cotangent {name}: one chunk of tile 16 and dtype {fdt} expected")
            setattr(ct, name, f.chunks[0].data.data_ptr())
    o = TlgOutputs()
    o.first_cell, o.num_cells, o.out_first_cell, o.tile = 0, blk.num_cells, 0, GPU_QUAD_TILE
    for name, f in fields.items():
        setattr(o, name, f.chunks[0].data.data_ptr())
    desc = g.block_desc(b)
    stream = current_stream_handle()
    if from_fields is not None:
        if forward:
            raise GridError(1, "from_fields reads the forward fields: no fused forward")
        for name in ("detj", "pinv"):
            f = from_fields.get(name)
            if f is None or f.tile != GPU_QUAD_TILE or len(f.chunks) != 1 or f.chunks[0].data.dtype != fdt:
                raise GridError(1, f"from_fields {name}: one chunk of tile 16 and dtype {fdt} expected")
            if f.num_cells != blk.num_cells or f.num_points != nq:
                raise GridError(2, f"from_fields {name}: another block's or point set's field")
            setattr(o, name, f.chunks[0].data.data_ptr())
        check(lib().tlg_vjp_block_from_fields(tables.handle, ctypes.byref(desc), ctypes.byref(o), ctypes.byref(ct),
                                              local.data_ptr(), local.shape[0], stream))
    else:
        check(lib().tlg_vjp_block(tables.handle, ctypes.byref(desc), ctypes.byref(o), ctypes.byref(ct),
                                  local.data_ptr(), local.shape[0], stream))
    _note_launch()
    inc = node_incidence(g, b)
    grad = torch.empty((g.nodes.shape[0], gd), dtype=torch.float64, device=dev)
    check(lib().tlg_vjp_gather(inc.offsets.data_ptr(), inc.entries.data_ptr(), g.nodes.shape[0], gd,
                               local.data_ptr(), 4 if fdt == torch.float32 else 8, grad.data_ptr(), stream))
    return grad, fields


class Batch:
    """Every block of `g` evaluated by one CUDA graph launch (``tlg_batch_*``): the point set of
    each block from `rule`, the same factors and precision for all; fields allocated once
    (``self.fields[b]``). ``tune()`` picks the launch shapes; ``launch()`` runs the graph. With
    ``cell_measure=True`` (det J among the factors) each launch also writes the per-cell sums of
    det J * w to ``self.cell_measure[b]``; ``measure()`` sums them into the mesh's measure."""

    def __init__(self, g: Geometry, rule: "QuadRule", factors=("points", "jacobian", "detj", "pinv"),
                 precision: str = "native", cell_measure: bool = False):
        self.g, self.rule, self.precision = g, rule, precision
        self.cell_measure = []
        n = len(g.blocks)
        if precision not in ("native", "split", "df64"):
            raise GridError(1, f"unknown precision {precision!r}")
        if precision != "native" and g.dtype != torch.float64:
            raise GridError(1, f"{precision} precision evaluates f64 meshes")
        out_dtype = torch.float32 if precision == "split" else g.dtype
        code = {"split": SPLIT32, "df64": DF64}.get(precision, g.dtype)
        self.fields, self._tables = [], []
        descs = (TlgBlock * max(n, 1))()
        outs = (TlgOutputs * max(n, 1))()
        handles = (ctypes.c_void_p * max(n, 1))()
        for b, blk in enumerate(g.blocks):
            pts = rule.get(blk.element.cell)
            td, gd = blk.element.tdim, g.gdim
            names = _factor_names(g, b, factors)
            t = pts.tables(blk.element, gd, code)
            self._tables.append(t)
            f = {name: QuadField.uninit(blk.num_cells, len(pts), FACTOR_LEN[name](td, gd), GPU_QUAD_TILE,
                                        out_dtype, g.nodes.device) for name in names}
            self.fields.append(f)
            descs[b] = g.block_desc(b)
            o = outs[b]
            o.first_cell, o.num_cells, o.out_first_cell, o.tile = 0, blk.num_cells, 0, GPU_QUAD_TILE
            for name in names:
                setattr(o, name, f[name].chunks[0].data.data_ptr() if f[name].chunks else None)
            if cell_measure:
                if "detj" not in names:
                    raise GridError(1, "cell_measure needs detj among the factors")
                cm = torch.zeros(max(blk.num_cells, 1), dtype=out_dtype, device=g.nodes.device)
                self.cell_measure.append(cm)
                o.weights = pts.weights_device(out_dtype, g.nodes.device).data_ptr()
                o.cell_measure = cm.data_ptr()
            handles[b] = t.handle
        self._descs, self._outs, self._handles = descs, outs, handles
        h = ctypes.c_void_p()
        check(lib().tlg_batch_create(handles, descs, outs, n, ctypes.byref(h)))
        self.handle = h
        self.grids = [0] * n

    def tune(self) -> list:
        grids = (ctypes.c_int * max(len(self.fields), 1))()
        check(lib().tlg_batch_tune(self.handle, current_stream_handle(), grids))
        self.grids = list(grids)[: len(self.fields)]
        return self.grids

    def tuning(self) -> dict:
        """The tuner's choice: ``{"grids", "strategies" (per block the strategy name its launch
        forces, "caller" for the override or policy in effect), "serial" (a chain rather than
        parallel branches), "tuned_ms" (its median time of the chosen graph)}``."""
        serial, ms = ctypes.c_int(0), ctypes.c_float(0.0)
        n = len(self.fields)
        codes = (ctypes.c_int * max(n, 1))()
        check(lib().tlg_batch_tuning(self.handle, ctypes.byref(serial), ctypes.byref(ms), codes))
        names = {-1: "caller", 0: "auto", 1: "direct", 2: "loops", 3: "sumfact", 4: "shared", 5: "cooperative",
                 6: "tensor"}
        return {"grids": list(self.grids), "strategies": [names.get(c, str(c)) for c in list(codes)[:n]],
                "serial": bool(serial.value), "tuned_ms": float(ms.value)}

    def launch(self) -> None:
        check(lib().tlg_batch_launch(self.handle, current_stream_handle()))

    def measure(self) -> float:
        """The mesh's measure from the last launch's per-cell sums: the tree of each block, summed
        over the blocks in order in f64 on the host."""
        if not self.cell_measure:
            raise GridError(1, "the batch was created without cell_measure")
        return sum(measure_block(self.g, b, self.rule.get(blk.element.cell), cell_sums=self.cell_measure[b])
                   for b, blk in enumerate(self.g.blocks))

    def __del__(self):
        try:
            lib().tlg_batch_destroy(self.handle)
        except Exception:
            pass


class AdjointBatch:
    """The fused forward + adjoint of every block of `g` in one CUDA graph launch
    (``tlg_vjp_batch_*``): the point set of each block from `rule`, the cotangent fields of block b
    in ``cotangents[b]`` (as for :func:`vjp_block`), the forward fields `forward` written in the
    same pass (``self.fields[b]``), the node cotangents of the whole mesh in ``self.grad``
    (``[node][GD]`` f64, summed block by block). ``launch()`` runs the graph.

    ``precision="df64"``: the forward fields are f64 and come from the double-float kernels
    (f64-accurate), each block's adjoint is the split-precision one (f32 cotangents, FP32
    contributions summed per node in f64), both on the block's branch of the graph.

    ``two_pass=True`` (``tlg_vjp_batch_set_two_pass``; det J and K among `forward`): blocks of
    volume cells run the policy's forward kernel, then the adjoint from the det J and K fields it
    wrote (``tlg_vjp_block_from_fields``); the others the fused pass. ``None`` (the default): two
    passes in split precision with det J and K among `forward` (faster there: 3.35 against
    3.67 ms on the hybrid mesh), else the fused pass."""

    def __init__(self, g: Geometry, rule: "QuadRule", cotangents: list, precision: str = "split", forward=(),
                 two_pass: bool | None = None):
        from ._lib import TlgCotangents

        if g.dtype != torch.float64:
            raise GridError(1, "the adjoint reads f64 meshes")
        if precision not in ("native", "split", "df64"):
            raise GridError(1, f"unknown precision {precision!r}")
        n = len(g.blocks)
        fdt = torch.float64 if precision == "native" else torch.float32  # cotangents, contributions
        out_dt = torch.float32 if precision == "split" else torch.float64  # forward fields
        code = g.dtype if precision == "native" else SPLIT32
        dev = g.nodes.device
        self.g, self.fields, self.locals, self._keep = g, [], [], []
        descs = (TlgBlock * max(n, 1))()
        outs = (TlgOutputs * max(n, 1))()
        cts = (TlgCotangents * max(n, 1))()
        handles = (ctypes.c_void_p * max(n, 1))()
        locals_ = (ctypes.c_void_p * max(n, 1))()
        lcells = (ctypes.c_int64 * max(n, 1))()
        offs = (ctypes.c_void_p * max(n, 1))()
        ents = (ctypes.c_void_p * max(n, 1))()
        gd = g.gdim
        for b, blk in enumerate(g.blocks):
            pts = rule.get(blk.element.cell)
            td, k = blk.element.tdim, blk.element.nodes_per_cell
            t = pts.tables(blk.element, gd, code)
            if precision == "df64":
                self._keep.append(pts.tables(blk.element, gd, DF64))
            f = {name: QuadField.uninit(blk.num_cells, len(pts), FACTOR_LEN[name](td, gd), GPU_QUAD_TILE, out_dt, dev)
                 for name in forward}
            self.fields.append(f)
            loc = torch.empty((max(blk.num_cells, 1), k, 4 if gd == 3 else gd), dtype=fdt, device=dev)
            self.locals.append(loc)
            inc = node_incidence(g, b)
            self._keep += [t, inc]
            descs[b] = g.block_desc(b)
            o = outs[b]
            o.first_cell, o.num_cells, o.out_first_cell, o.tile = 0, blk.num_cells, 0, GPU_QUAD_TILE
            for name, fld in f.items():
                setattr(o, name, fld.chunks[0].data.data_ptr())
            for name in ("points", "detj", "pinv", "normals"):
                fld = cotangents[b].get(name)
                if fld is not None:
                    if fld.tile != GPU_QUAD_TILE or len(fld.chunks) != 1 or fld.chunks[0].data.dtype != fdt:
                        raise GridError(1, f"cotangent {name}: one chunk of tile 16 and dtype {fdt} expected")
                    setattr(cts[b], name, fld.chunks[0].data.data_ptr())
            handles[b] = t.handle
            locals_[b] = loc.data_ptr()
            lcells[b] = loc.shape[0]
            offs[b] = inc.offsets.data_ptr()
            ents[b] = inc.entries.data_ptr()
        self.grad = torch.empty((g.nodes.shape[0], gd), dtype=torch.float64, device=dev)
        self._ctypes = (descs, outs, cts, handles, locals_, lcells, offs, ents, cotangents)
        h = ctypes.c_void_p()
        check(lib().tlg_vjp_batch_create(handles, descs, outs, cts, locals_, lcells, offs, ents, g.nodes.shape[0],
                                         gd, self.grad.data_ptr(), n, ctypes.byref(h)))
        self.handle = h
        if precision == "df64":
            fwd = (ctypes.c_void_p * max(n, 1))()
            for b, blk in enumerate(g.blocks):
                fwd[b] = rule.get(blk.element.cell).tables(blk.element, gd, DF64).handle
            self._fwd = fwd
            check(lib().tlg_vjp_batch_set_forward(h, fwd))
        if two_pass is None:
            two_pass = precision == "split" and "detj" in forward and "pinv" in forward
        self.two_pass = bool(two_pass)
        if two_pass:
            check(lib().tlg_vjp_batch_set_two_pass(h, 1))

    def launch(self) -> None:
        check(lib().tlg_vjp_batch_launch(self.handle, current_stream_handle()))

    def __del__(self):
        try:
            lib().tlg_vjp_batch_destroy(self.handle)
        except Exception:
            pass


def fd_check(g: Geometry, b: int, pts: PointSet, cotangents: dict, grad: np.ndarray, sample,
             h: float = 1e-6) -> dict:
    """Central differences of L = sum over cells and points of (xbar . x + dbar det J + Kbar : K
    + nbar . n) against the node cotangents `grad` ([node][GD]) at the node indices `sample`, with
    the f64 forward kernels. Each (node, coordinate, sign) perturbs a private copy of the cells
    around the node only (the other cells do not change L), and all copies are evaluated in one
    launch. `cotangents` holds cell-major host arrays ("points" [c][q][GD], "detj" [c][q], "pinv"
    [c][q][TD GD], "normals" [c][q][GD]), missing ones zero. Returns the largest
    |fd - grad| / max(1, |grad|)."""
    blk = g.blocks[b]
    k = blk.element.nodes_per_cell
    gd = g.gdim
    dofmap = blk.dofmap.cpu().numpy().view(np.uint32).reshape(-1, k)
    inc = node_incidence(g, b)
    offsets = inc.offsets.cpu().numpy().view(np.uint32).astype(np.int64)
    entries = inc.entries.cpu().numpy().view(np.uint32)
    stored = g.nodes.double().cpu().numpy()
    cells_of = []
    for n in sample:
        e = entries[offsets[n]:offsets[n + 1]]
        cells_of.append(np.unique(e // k))
    copies, owner, local_pos = [], [], []
    for i, cells in enumerate(cells_of):
        for c in range(gd):
            for s in (1.0, -1.0):
                copies.append(cells)
                owner.append((i, c, s))
    all_cells = np.concatenate(copies)
    dm = dofmap[all_cells]  # [m][K]
    nodes = stored[dm].reshape(-1, gd).copy()  # private copies, [m * K][GD]
    start = 0
    for (i, c, s), cells in zip(owner, copies):
        n = sample[i]
        for j in range(cells.size):
            row = dm[start + j]
            for kk in np.nonzero(row == n)[0]:
                nodes[(start + j) * k + kk, c] += s * h
        start += cells.size
    sub_dofmap = np.arange(all_cells.size * k, dtype=np.uint32).reshape(-1, k)
    sub_flags = None if blk.flags is None or blk.flags.numel() == 0 else \
        blk.flags[torch.from_numpy(np.minimum(all_cells, blk.flags.numel() - 1).astype(np.int64)).to(blk.flags.device)]
    sub = Geometry([GeometryBlock(blk.element, torch.from_numpy(sub_dofmap.view(np.int32)).to(g.nodes.device),
                                  sub_flags)],
                   torch.from_numpy(nodes).to(g.nodes.device), g.origin)
    names = [f for f in ("points", "detj", "pinv", "normals") if cotangents.get(f) is not None]
    fields = geometric_factors_block(sub, 0, pts, names)
    per_cell = np.zeros(all_cells.size)
    for f in names:
        vals = fields[f].to_host_cell_major()  # [copy][q][LEN]
        ct = np.asarray(cotangents[f], dtype=np.float64)
        if f == "detj":
            ct = ct[..., None]
        per_cell += (vals * ct[all_cells]).sum(axis=(1, 2))
    worst = 0.0
    start = 0
    sums = {}
    for (i, c, s), cells in zip(owner, copies):
        sums[(i, c, s)] = per_cell[start:start + cells.size].sum()
        start += cells.size
    for i, n in enumerate(sample):
        for c in range(gd):
            fd = (sums[(i, c, 1.0)] - sums[(i, c, -1.0)]) / (2.0 * h)
            worst = max(worst, abs(fd - grad[n, c]) / max(1.0, abs(grad[n, c])))
    return {"max_rel_err": worst, "nodes": int(len(sample)), "step": h}
