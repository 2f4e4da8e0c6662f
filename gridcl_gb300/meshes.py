"""Synthetic host meshes: the structured boxes, the subdivided-icosahedron sphere and the node
perturbations of the benchmark workloads, numbered like the reference's test meshes.

Restates (paths inside the reference project):

- ``cube_box`` / ``square_box``: tetraloma-testing/src/meshes/boxes.rs:96-151 — the unit box in
  n^d subcells on the integer lattice of resolution 2 n p, cells numbered x fastest, then y,
  then z, the cells of one subcell consecutive; tetrahedra by the Kuhn split (one per path
  0 -> e_a -> e_a + e_b -> 7), prisms by the z-face diagonal (0,0)-(1,1), pyramids one per
  face of the subcell (faces in the hexahedron's sub-entity order) with the apex at its centre
  (boxes.rs:44-58, 182-187), each cell oriented positively (swap of vertices 1 and 2, and 4
  and 5 on prisms);
- node numbering: the order of first use by the cells, with shared high-order nodes found
  exactly through their lattice keys (meshes/lattice.rs:95-230);
- the Lagrange nodes of a cell are the equispaced reference nodes mapped affinely through its
  vertices (lattice.rs:187-213);
- ``SplitMix64`` (meshes/lattice.rs:333-354) for every seeded perturbation.

Everything is vectorised with numpy so that the benchmark meshes (millions of cells) build in
seconds.
"""

from __future__ import annotations

import dataclasses
import math

import numpy as np

from . import refcell

_TDIM = {"Interval": 1, "Triangle": 2, "Quadrilateral": 2, "Tetrahedron": 3, "Hexahedron": 3,
         "Prism": 3, "Pyramid": 3}


@dataclasses.dataclass
class HostBlock:
    cell: str
    degree: int
    cells: np.ndarray  # [num_cells][K] uint32
    family: str = "Equispaced"

    @property
    def num_cells(self) -> int:
        return self.cells.shape[0]

    @property
    def nodes_per_cell(self) -> int:
        return self.cells.shape[1]


@dataclasses.dataclass
class HostMesh:
    gdim: int
    nodes: np.ndarray  # [num_nodes][gdim] float64
    blocks: list

    @property
    def num_nodes(self) -> int:
        return self.nodes.shape[0]

    def first_cells(self, n: int) -> "HostMesh":
        """The first n cells (over the blocks in order) and the nodes they use, renumbered in
        their old order (meshes/mod.rs:337-382)."""
        blocks, used = [], np.zeros(self.num_nodes, dtype=bool)
        left = n
        for b in self.blocks:
            keep = b.cells[: max(left, 0)]
            left -= keep.shape[0]
            used[keep.ravel()] = True
            blocks.append(HostBlock(b.cell, b.degree, keep, b.family))
        new = np.cumsum(used) - 1
        return HostMesh(self.gdim, self.nodes[used],
                        [HostBlock(b.cell, b.degree, new[b.cells].astype(np.uint32), b.family)
                         for b in blocks])


def splitmix64(seed: int, count: int) -> np.ndarray:
    """The first `count` outputs of SplitMix64 from `seed` (meshes/lattice.rs:342-348)."""
    with np.errstate(over="ignore"):
        gamma = np.uint64(0x9E3779B97F4A7C15)
        z = np.uint64(seed) + gamma * np.arange(1, count + 1, dtype=np.uint64)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, shape) -> np.ndarray:
    """Seeded uniform values in [-1, 1): the top 53 bits of SplitMix64, shape `shape`."""
    n = int(np.prod(shape))
    u = (splitmix64(seed, n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return (2.0 * u - 1.0).reshape(shape)


def _axis_vertices(cell: str):
    return {"Interval": [1], "Triangle": [1, 2], "Quadrilateral": [1, 2],
            "Tetrahedron": [1, 2, 3], "Prism": [1, 2, 3], "Hexahedron": [1, 2, 4],
            "Pyramid": [1, 2, 4]}[cell]


def _node_keys(cell: str, p: int, verts: np.ndarray, lagrange_points=None) -> np.ndarray:
    """Lattice keys [ncells][K][3] of the Lagrange nodes of cells given by vertex keys `verts`
    [ncells][nv][3] (int64): the reference nodes mapped affinely through the vertices 0 and the
    axis vertices. `lagrange_points(cell, p)` gives the reference nodes (the library's refcell by
    default)."""
    ref = (lagrange_points or refcell.lagrange_points)(cell, p)  # [K][td] in [0, 1]
    r = np.rint(ref * p).astype(np.int64)
    assert np.allclose(r, ref * p), "equispaced nodes lie on the lattice"
    axes = verts[:, _axis_vertices(cell), :] - verts[:, :1, :]  # [ncells][td][3]
    s = np.einsum("kt,ctg->ckg", r, axes)
    assert np.all(s % p == 0)
    return verts[:, :1, :] + s // p


def _number(flat: np.ndarray, side: int):
    """First-use numbering of the flat keys (in the order given). Returns (node keys [N][3],
    node index of every key)."""
    uniq, first, inverse = np.unique(flat, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")  # unique keys in order of first use
    rank = np.empty_like(order)
    rank[order] = np.arange(order.size)
    node_keys = np.stack([uniq[order] // (side * side), (uniq[order] // side) % side,
                          uniq[order] % side], axis=1)
    return node_keys, rank[inverse]


def _assemble(cell: str, p: int, verts: np.ndarray, gdim: int, resolution: int, lagrange_points=None):
    """Lagrange-node lattice keys of cells given by vertex keys `verts` [ncells][nv][3] (int64),
    nodes numbered by first use. Returns (node keys [N][3], dofmap [ncells][K] uint32)."""
    keys = _node_keys(cell, p, verts, lagrange_points)
    side = resolution + 1
    flat = (keys[..., 0] * side + keys[..., 1]) * side + keys[..., 2]
    node_keys, idx = _number(flat.ravel(), side)
    return node_keys, idx.reshape(flat.shape).astype(np.uint32)


_CELL_ORDER = ("Interval", "Triangle", "Quadrilateral", "Tetrahedron", "Hexahedron", "Prism", "Pyramid")


def _assemble_blocks(parts, p: int, resolution: int) -> HostMesh:
    """A mesh of several cell types: `parts` maps a cell type to (vertex keys [n][nv][3], the
    cells' positions in the generation order [n]). Nodes are numbered by first use over all
    cells in generation order; blocks follow the cell-type order (meshes/lattice.rs:95-230)."""
    side = resolution + 1
    cells = sorted(parts, key=_CELL_ORDER.index)
    keys = {c: _node_keys(c, p, parts[c][0]) for c in cells}
    flat = {c: (k[..., 0] * side + k[..., 1]) * side + k[..., 2] for c, k in keys.items()}
    seq = np.concatenate([np.repeat(parts[c][1], flat[c].shape[1]) for c in cells])
    allk = np.concatenate([flat[c].ravel() for c in cells])
    order = np.argsort(seq, kind="stable")  # cells in generation order, nodes in local order
    node_keys, idx_sorted = _number(allk[order], side)
    idx = np.empty_like(idx_sorted)
    idx[order] = idx_sorted
    blocks, at = [], 0
    for c in cells:
        n = flat[c].size
        blocks.append(HostBlock(c, p, idx[at: at + n].reshape(flat[c].shape).astype(np.uint32)))
        at += n
    return HostMesh(3, node_keys.astype(np.float64) / resolution, blocks)


def _orient(cell: str, verts: np.ndarray) -> np.ndarray:
    """Swaps vertices so that every cell's axis determinant is positive (lattice.rs:52-78)."""
    axes = (verts[:, _axis_vertices(cell), :] - verts[:, :1, :]).astype(np.float64)
    td = len(_axis_vertices(cell))
    det = np.linalg.det(axes[:, :, :td]) if td > 1 else axes[:, 0, 0]
    neg = det < 0
    if np.any(neg):
        if cell in ("Triangle", "Tetrahedron", "Pyramid"):
            v = verts[neg]
            v[:, [1, 2]] = v[:, [2, 1]]
            verts[neg] = v
        elif cell == "Prism":
            v = verts[neg]
            v[:, [1, 2]] = v[:, [2, 1]]
            v[:, [4, 5]] = v[:, [5, 4]]
            verts[neg] = v
        else:
            raise ValueError(f"negatively oriented {cell}")
    return verts


def cube_box(cell: str, n: int, p: int, lagrange_points=None) -> HostMesh:
    """The unit cube in n^3 subcells of `cell` cells of degree p (boxes.rs:129-167)."""
    if n < 1 or p < 1:
        raise ValueError("a box needs n >= 1 and p >= 1")
    res = 2 * n * p
    h = 2 * p
    i, j, k = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    # x fastest: order subcells by (k, j, i).
    origin = np.stack([i.transpose(2, 1, 0).ravel(), j.transpose(2, 1, 0).ravel(),
                       k.transpose(2, 1, 0).ravel()], axis=1).astype(np.int64) * h
    bits = np.array([[(v >> b) & 1 for b in range(3)] for v in range(8)], dtype=np.int64)
    corners = origin[:, None, :] + bits[None, :, :] * h  # [nsub][8][3]
    if cell == "Hexahedron":
        verts = corners
    elif cell == "Tetrahedron":
        paths = [(0, 1), (0, 2), (1, 0), (1, 2), (2, 0), (2, 1)]
        sel = [[0, 1 << a, (1 << a) | (1 << b), 7] for a, b in paths]
        verts = corners[:, sel, :].reshape(-1, 4, 3)
    elif cell == "Prism":
        sel = [[a, b, d, a + 4, b + 4, d + 4] for a, b, d in ([0, 1, 3], [0, 3, 2])]
        verts = corners[:, sel, :].reshape(-1, 6, 3)
    elif cell == "Pyramid":
        verts = _pyramids(corners, origin + p).reshape(-1, 5, 3)
    else:
        raise ValueError(f"cube_box has no {cell} cells in this build")
    verts = _orient(cell, verts.copy())
    keys, dofmap = _assemble(cell, p, verts, 3, res, lagrange_points)
    return HostMesh(3, keys.astype(np.float64) / res, [HostBlock(cell, p, dofmap)])


_HEX_FACES = [[0, 1, 2, 3], [0, 1, 4, 5], [0, 2, 4, 6], [1, 3, 5, 7], [2, 3, 6, 7], [4, 5, 6, 7]]


def _subcells(n: int, p: int):
    """Per subcell (x fastest, then y, then z): its index (i, j, k), its 8 corner keys in tensor
    order and its centre key, on the lattice of resolution 2 n p."""
    h = 2 * p
    i, j, k = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    ijk = np.stack([i.transpose(2, 1, 0).ravel(), j.transpose(2, 1, 0).ravel(),
                    k.transpose(2, 1, 0).ravel()], axis=1).astype(np.int64)
    bits = np.array([[(v >> b) & 1 for b in range(3)] for v in range(8)], dtype=np.int64)
    corners = ijk[:, None, :] * h + bits[None, :, :] * h
    return ijk, corners, ijk * h + p


def _pyramids(corners: np.ndarray, centres: np.ndarray, faces=_HEX_FACES) -> np.ndarray:
    """[n][len(faces)][5][3]: the pyramid on each face with the apex at the centre."""
    base = corners[:, faces, :]
    apex = np.broadcast_to(centres[:, None, None, :], base.shape[:2] + (1, 3))
    return np.concatenate([base, apex], axis=2)


def mixed_box(n: int, p: int) -> HostMesh:
    """The conforming tetrahedron/hexahedron/pyramid box (boxes.rs:194-245): subcells with an
    even index sum split into six pyramids around their centre, the pyramid on the face x = 0 of
    the subcells at i = 0 split into two tetrahedra along its base diagonal v0-v3; the other
    subcells stay hexahedra. Blocks: tetrahedra, hexahedra, pyramids."""
    if n < 1 or p < 1:
        raise ValueError("a box needs n >= 1 and p >= 1")
    ijk, corners, centres = _subcells(n, p)
    even = ijk.sum(1) % 2 == 0
    # Generation order: per subcell, its cells; six slots per subcell (the split pyramid's two
    # tetrahedra share its slot, the hexahedron takes slot 0).
    base_seq = np.arange(ijk.shape[0]) * 6
    hexes = corners[~even]
    pyr = _pyramids(corners[even], centres[even])  # [ne][6][5][3]
    pseq = base_seq[even][:, None] + np.arange(6)[None, :]
    split = np.zeros(pyr.shape[:2], dtype=bool)
    split[:, 2] = ijk[even][:, 0] == 0  # face 2 is x = 0 (vertices 0, 2, 4, 6)
    tets = []
    for a, b, d in ((0, 1, 3), (0, 3, 2)):
        t = pyr[split][:, [a, b, d, 4], :]
        tets.append(t)
    tv = np.stack(tets, axis=1).reshape(-1, 4, 3) if split.any() else np.zeros((0, 4, 3), np.int64)
    tseq = np.repeat(pseq[split], 2)
    parts = {}
    if tv.shape[0]:
        parts["Tetrahedron"] = (_orient("Tetrahedron", tv.copy()), tseq)
    if hexes.shape[0]:
        parts["Hexahedron"] = (hexes, base_seq[~even])
    parts["Pyramid"] = (_orient("Pyramid", pyr[~split].copy()), pseq[~split])
    return _assemble_blocks(parts, p, 2 * n * p)


def hex_prism_pyramid_box(n: int, p: int) -> HostMesh:
    """The conforming hexahedron/prism/pyramid box (boxes.rs:247-302): the subcells of the
    columns i < n // 3 split into two prisms each (as `cube_box`'s prisms), of the others those
    with an even index sum into six pyramids around their centre, the rest hexahedra."""
    if n < 1 or p < 1:
        raise ValueError("a box needs n >= 1 and p >= 1")
    ijk, corners, centres = _subcells(n, p)
    prism_col = ijk[:, 0] < n // 3
    even = (ijk.sum(1) % 2 == 0) & ~prism_col
    hexa = ~prism_col & ~even
    seq = np.arange(ijk.shape[0]) * 6
    parts = {}
    if hexa.any():
        parts["Hexahedron"] = (corners[hexa], seq[hexa])
    if prism_col.any():
        sel = [[a, b, d, a + 4, b + 4, d + 4] for a, b, d in ([0, 1, 3], [0, 3, 2])]
        pv = corners[prism_col][:, sel, :].reshape(-1, 6, 3)
        parts["Prism"] = (_orient("Prism", pv.copy()),
                          (seq[prism_col][:, None] + np.arange(2)[None, :]).ravel())
    if even.any():
        pyr = _pyramids(corners[even], centres[even]).reshape(-1, 5, 3)
        parts["Pyramid"] = (_orient("Pyramid", pyr.copy()),
                            (seq[even][:, None] + np.arange(6)[None, :]).ravel())
    return _assemble_blocks(parts, p, 2 * n * p)


def square_box(cell: str, n: int, p: int) -> HostMesh:
    """The unit square in n^2 squares, quadrilaterals or two triangles along (0,0)-(1,1)
    (boxes.rs:96-123)."""
    res = 2 * n * p
    h = 2 * p
    i, j = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    origin = np.stack([i.T.ravel(), j.T.ravel(), np.zeros(n * n, dtype=np.int64)], 1).astype(np.int64) * h
    bits = np.array([[v & 1, (v >> 1) & 1, 0] for v in range(4)], dtype=np.int64)
    c = origin[:, None, :] + bits[None] * h
    if cell == "Quadrilateral":
        verts = c
    elif cell == "Triangle":
        verts = c[:, [[0, 1, 3], [0, 3, 2]], :].reshape(-1, 3, 3)
    else:
        raise ValueError(cell)
    verts = _orient(cell, verts.copy())
    keys, dofmap = _assemble(cell, p, verts, 2, res)
    return HostMesh(2, keys[:, :2].astype(np.float64) / res, [HostBlock(cell, p, dofmap)])


def sin_map(x: np.ndarray, amplitude: float = 0.05) -> np.ndarray:
    """x' = x + a sin(2 pi y) sin(2 pi z), cyclically in (x, y, z)."""
    s = np.sin(2.0 * math.pi * x)
    out = x.copy()
    out[:, 0] += amplitude * s[:, 1] * s[:, 2]
    out[:, 1] += amplitude * s[:, 2] * s[:, 0]
    out[:, 2] += amplitude * s[:, 0] * s[:, 1]
    return out


def jitter_interior(x: np.ndarray, boundary_of: np.ndarray, amplitude: float, seed: int) -> np.ndarray:
    """Adds seeded uniform values in [-amplitude, amplitude) to every coordinate of the nodes
    that are not on the unit box's boundary (judged on the unperturbed coordinates
    `boundary_of`)."""
    eps = 1e-12
    on_boundary = np.any((boundary_of <= eps) | (boundary_of >= 1.0 - eps), axis=1)
    out = x.copy()
    out[~on_boundary] += amplitude * uniform(seed, x.shape)[~on_boundary]
    return out


def curved_box(cell: str, n: int, p: int, jitter: float, seed: int = 2026, amplitude: float = 0.05,
               lagrange_points=None) -> HostMesh:
    """The benchmark boxes: cube_box mapped by `sin_map`, then interior nodes jittered by
    `jitter` * h (h = 1 / n)."""
    m = cube_box(cell, n, p, lagrange_points)
    x = sin_map(m.nodes, amplitude) if amplitude else m.nodes
    m.nodes = jitter_interior(x, m.nodes, jitter / n, seed) if jitter else x
    return m


# ------------------------------------------------------------------------------------------
# Sphere (meshes/sphere.rs): icosahedron faces split into 4^r flat triangles, nodes projected.

def _icosahedron():
    phi = (1.0 + math.sqrt(5.0)) / 2.0
    v = []
    for axis in range(3):
        for s1 in (-1.0, 1.0):
            for s2 in (-phi, phi):
                x = [0.0, 0.0, 0.0]
                x[(axis + 1) % 3] = s1
                x[(axis + 2) % 3] = s2
                v.append(x)
    v = np.array(v)
    faces = []
    for a in range(12):
        for b in range(a + 1, 12):
            for c in range(b + 1, 12):
                d = lambda i, j: np.sum((v[i] - v[j]) ** 2)
                if abs(d(a, b) - 4) < 1e-9 and abs(d(b, c) - 4) < 1e-9 and abs(d(a, c) - 4) < 1e-9:
                    det = np.linalg.det(np.stack([v[a], v[b], v[c]]))
                    faces.append((a, b, c) if det > 0 else (a, c, b))
    assert len(faces) == 20
    return v, faces


def sphere(refinements: int, p: int, max_cells: int | None = None) -> HostMesh:
    """Degree-p triangles on the unit sphere from the icosahedron refined `refinements` times
    (meshes/sphere.rs:105-160), optionally truncated to the first `max_cells` cells."""
    v, faces = _icosahedron()
    n = 1 << refinements
    res = n * p
    ref = np.rint(refcell.lagrange_points("Triangle", p) * p).astype(np.int64)  # [K][2]
    # Local cells of one face: up (i, j), (i + 1, j), (i, j + 1) and down triangles.
    loc = []
    for j in range(n):
        for i in range(n - j):
            loc.append(((i, j), (i + 1, j), (i, j + 1)))
            if i + j + 1 < n:
                loc.append(((i + 1, j), (i + 1, j + 1), (i, j + 1)))
    loc = np.array(loc, dtype=np.int64) * p  # [ncf][3][2]
    ncf = loc.shape[0]
    total = 20 * ncf
    if max_cells is not None:
        total = min(total, max_cells)
    faces_needed = -(-total // ncf)
    axes = loc[:, 1:, :] - loc[:, :1, :]  # [ncf][2][2]
    s = np.einsum("kt,ctg->ckg", ref, axes)
    local = loc[:, None, 0, :] + s // p  # [ncf][K][2] lattice (a, b) in the face
    keys, cells = [], []
    for f in range(faces_needed):
        a, b = local[..., 0], local[..., 1]
        w = np.stack([res - a - b, a, b], axis=-1)  # weights of the face's three vertices
        verts = np.array(faces[f], dtype=np.int64)
        # Canonical key: (vertex id, weight) pairs sorted by vertex id, zero weights dropped.
        vid = np.broadcast_to(verts, w.shape).copy()
        vid[w == 0] = 99
        order = np.argsort(vid, axis=-1, kind="stable")
        vs = np.take_along_axis(vid, order, -1)
        ws = np.take_along_axis(w, order, -1)
        ws[vs == 99] = 0
        key = ((vs[..., 0] * 4096 + ws[..., 0]) * 128 + vs[..., 1]) * 4096 + ws[..., 1]
        key = key * 128 + vs[..., 2]
        key = key * 4096 + ws[..., 2]
        keys.append(key)
        cells.append((vs, ws))
    flat = np.concatenate([k.ravel() for k in keys])[: total * ref.shape[0]]
    uniq, first, inverse = np.unique(flat, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")
    rank = np.empty_like(order)
    rank[order] = np.arange(order.size)
    dofmap = rank[inverse].reshape(total, ref.shape[0]).astype(np.uint32)
    vs = np.concatenate([c[0].reshape(-1, 3) for c in cells])[: total * ref.shape[0]]
    ws = np.concatenate([c[1].reshape(-1, 3) for c in cells])[: total * ref.shape[0]]
    pick = first[order]
    vv = np.where(vs[pick] == 99, 0, vs[pick])
    x = np.einsum("na,nag->ng", ws[pick].astype(np.float64), v[vv])
    x /= np.linalg.norm(x, axis=1, keepdims=True)
    return HostMesh(3, x, [HostBlock("Triangle", p, dofmap)])


def perturbed_radius(m: HostMesh, amplitude: float, seed: int = 2026) -> HostMesh:
    """Scales every node's radius by 1 + amplitude * U[0, 1) (seeded)."""
    u = 0.5 * (uniform(seed, (m.num_nodes,)) + 1.0)
    return HostMesh(m.gdim, m.nodes * (1.0 + amplitude * u)[:, None], m.blocks)


def combine(parts, offsets) -> HostMesh:
    """One mesh of the blocks of `parts` (3D meshes), each translated by its offset, with the
    node arrays concatenated (the blocks share no nodes)."""
    nodes, blocks, base = [], [], 0
    for m, off in zip(parts, offsets):
        nodes.append(m.nodes + np.asarray(off, dtype=np.float64))
        for b in m.blocks:
            blocks.append(HostBlock(b.cell, b.degree, (b.cells.astype(np.int64) + base).astype(np.uint32),
                                    b.family))
        base += m.num_nodes
    return HostMesh(parts[0].gdim, np.concatenate(nodes), blocks)


def hybrid_box(hexes: int, prisms: int, tets: int, jitter: float = 0.02, seed: int = 2026) -> HostMesh:
    """A hybrid mesh of three blocks of uneven size: `hexes` Q2 hexahedra, `prisms` P2 prisms and
    `tets` P3 tetrahedra, each the first cells of a sin-mapped, jittered box, the boxes side by
    side along x."""
    parts = []
    for cell, p, count, per in (("Hexahedron", 2, hexes, 1), ("Prism", 2, prisms, 2), ("Tetrahedron", 3, tets, 6)):
        n = 1
        while per * n ** 3 < count:
            n += 1
        m = curved_box(cell, n, p, jitter=jitter, seed=seed)
        parts.append(m.first_cells(count))
    return combine(parts, [(0.0, 0.0, 0.0), (1.5, 0.0, 0.0), (3.0, 0.0, 0.0)])


# ------------------------------------------------------------------------------------------
# Cell orderings before upload (tetraloma/src/pipeline/order.rs:24-192, builder.rs:95-113),
# computed by the native library.

ORDERINGS = {"input": 0, "hilbert": 1, "rcm": 2}


def reorder(mesh: HostMesh, ordering: str = "hilbert"):
    """The mesh with each block's cells in `ordering` ("input", "hilbert": by the Hilbert key of
    the vertex centroid; "rcm": reverse Cuthill-McKee on the facet graph) and the nodes numbered
    by first use (blocks in order, each cell's nodes in Lagrange order; unused nodes last).
    Returns ``(mesh, cell_orders, node_order)``: per block the old index of each new cell, and the
    old index of each new node."""
    import ctypes

    from ._lib import CELL_IDS, check, lib

    if ordering not in ORDERINGS:
        raise ValueError(f"unknown ordering {ordering!r}")
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    nodes = np.ascontiguousarray(mesh.nodes, dtype=np.float64)
    orders, ordered = [], []
    for blk in mesh.blocks:
        cells = np.ascontiguousarray(blk.cells, dtype=np.uint32)
        order = np.empty(cells.shape[0], dtype=np.int64)
        check(lib().tlg_order_cells(ORDERINGS[ordering], CELL_IDS[blk.cell], ptr(cells), cells.shape[0],
                                    cells.shape[1], ptr(nodes), nodes.shape[0], mesh.gdim, ptr(order)))
        orders.append(order)
        ordered.append(np.ascontiguousarray(cells[order]))
    flat = np.concatenate([c.ravel() for c in ordered]) if ordered else np.zeros(0, dtype=np.uint32)
    flat = np.ascontiguousarray(flat, dtype=np.uint32)
    renumbered = np.empty_like(flat)
    node_order = np.empty(nodes.shape[0], dtype=np.int64)
    check(lib().tlg_number_nodes(ptr(flat), flat.size, 1, nodes.shape[0], ptr(renumbered), ptr(node_order)))
    blocks, at = [], 0
    for blk, c in zip(mesh.blocks, ordered):
        blocks.append(HostBlock(blk.cell, blk.degree, renumbered[at: at + c.size].reshape(c.shape), blk.family))
        at += c.size
    return HostMesh(mesh.gdim, nodes[node_order], blocks), orders, node_order


def shuffled(mesh: HostMesh, seed: int = 2026) -> HostMesh:
    """The mesh with the cells of each block and the nodes in a seeded random order (a mesh as an
    unordered generator or file would deliver it)."""
    rng = np.random.default_rng(seed)
    node_perm = rng.permutation(mesh.num_nodes)  # new index -> old index
    new_of_old = np.empty_like(node_perm)
    new_of_old[node_perm] = np.arange(mesh.num_nodes)
    blocks = []
    for blk in mesh.blocks:
        cells = blk.cells[rng.permutation(blk.num_cells)]
        blocks.append(HostBlock(blk.cell, blk.degree, new_of_old[cells].astype(np.uint32), blk.family))
    return HostMesh(mesh.gdim, mesh.nodes[node_perm], blocks)
