"""Cell orderings before upload (tetraloma/src/pipeline/order.rs): the Hilbert keys against the
reference's hand-computed keys and curve properties, quantisation, reverse Cuthill-McKee on a
shuffled grid, and node numbering by first use (CPU)."""

import ctypes

import numpy as np
import pytest

from gridcl_gb300 import meshes
from gridcl_gb300._lib import lib


def key(x, bits):
    a = np.ascontiguousarray(x, dtype=np.uint32)
    return int(lib().tlg_hilbert_key(a.ctypes.data_as(ctypes.c_void_p), len(x), bits))


def test_hilbert_keys_by_hand():
    """order.rs:197-220: the U of order 1 in 2D, the first quadrant of order 2, the Gray-code cube
    of order 1 in 3D, and one axis."""
    assert [key(x, 1) for x in [[0, 0], [0, 1], [1, 1], [1, 0]]] == [0, 1, 2, 3]
    assert [key(x, 2) for x in [[0, 0], [1, 0], [1, 1], [0, 1]]] == [0, 1, 2, 3]
    cube = [[0, 0, 0], [0, 0, 1], [0, 1, 1], [0, 1, 0], [1, 1, 0], [1, 1, 1], [1, 0, 1], [1, 0, 0]]
    assert [key(x, 1) for x in cube] == list(range(8))
    assert key([12345], 21) == 12345


@pytest.mark.parametrize("d,bits", [(2, 1), (2, 3), (2, 4), (3, 1), (3, 2), (3, 3)])
def test_hilbert_curves_are_continuous(d, bits):
    """A bijection onto 0..2^(d bits), consecutive keys at neighbouring grid points, starting at
    the origin (order.rs:222-244)."""
    side = 1 << bits
    points = [None] * (1 << (d * bits))
    for p in range(len(points)):
        x = [(p >> (g * bits)) % side for g in range(d)]
        k = key(x, bits)
        assert points[k] is None
        points[k] = x
    assert all(c == 0 for c in points[0])
    for a, b in zip(points, points[1:]):
        assert sum(abs(u - v) for u, v in zip(a, b)) == 1


def test_full_resolution_keys_follow_the_first_level():
    half = 1 << 20
    rng = np.random.default_rng(3)
    for d in (2, 3):
        for _ in range(200):
            x = rng.integers(0, 2 * half, size=d)
            k = key(x, 21)
            assert k < 1 << (21 * d)
            assert k >> (20 * d) == key(x // half, 1)
    assert key([0, 0, 0], 21) == 0


def test_quantisation_covers_the_box():
    q = lib().tlg_quantise
    top = (1 << 21) - 1
    assert q(-1.0, -1.0, 3.0) == 0 and q(3.0, -1.0, 3.0) == top
    assert q(1.0, -1.0, 3.0) == 1 << 20 and q(5.0, 5.0, 5.0) == 0


def bandwidth(mesh):
    """The facet-graph bandwidth of a tetrahedral block: the largest position difference of two
    cells that share a face (three vertices)."""
    c = mesh.blocks[0].cells[:, :4].astype(np.int64)
    owners = {}
    for i, row in enumerate(c):
        for f in ((0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3)):
            owners.setdefault(tuple(sorted(row[list(f)])), []).append(i)
    return max(abs(v[0] - v[1]) for v in owners.values() if len(v) == 2)


@pytest.mark.parametrize("ordering", ["hilbert", "rcm"])
def test_orderings_restore_locality(ordering):
    """On a shuffled tetrahedral box, both orderings permute the cells, renumber the nodes by
    first use, keep every cell's geometry, and bring consecutive cells close: the mean index
    distance between consecutive cells' first nodes drops five-fold, and so does the facet-graph
    bandwidth under reverse Cuthill-McKee."""
    base = meshes.cube_box("Tetrahedron", 6, 2)
    mix = meshes.shuffled(base, seed=5)
    out, orders, node_order = meshes.reorder(mix, ordering)
    assert sorted(orders[0].tolist()) == list(range(mix.blocks[0].num_cells))
    assert sorted(node_order.tolist()) == list(range(mix.num_nodes))
    # The same cells with the same coordinates, node by node.
    np.testing.assert_array_equal(out.nodes[out.blocks[0].cells], mix.nodes[mix.blocks[0].cells[orders[0]]])
    # Nodes numbered by first use: the first appearances are 0, 1, 2, ...
    flat = out.blocks[0].cells.ravel()
    _, first = np.unique(flat, return_index=True)
    assert np.array_equal(flat[np.sort(first)], np.arange(len(first)))
    spread = lambda m: np.abs(np.diff(m.blocks[0].cells[:, 0].astype(np.int64))).mean()
    assert spread(out) * 5 < spread(mix)
    if ordering == "rcm":  # what reverse Cuthill-McKee minimises
        assert bandwidth(out) * 5 < bandwidth(mix)


def test_rcm_components_and_reversal():
    """Two disjoint triangles: each component starts at its least (degree, position) cell and the
    order is reversed; a single cell orders trivially."""
    nodes = np.array([[0, 0], [1, 0], [0, 1], [5, 5], [6, 5], [5, 6], [6, 6.0]])
    cells = np.array([[0, 1, 2], [3, 4, 5], [4, 6, 5]], dtype=np.uint32)
    m = meshes.HostMesh(2, nodes, [meshes.HostBlock("Triangle", 1, cells)])
    _, orders, _ = meshes.reorder(m, "rcm")
    # Degrees: cell 0 -> 0, cells 1, 2 -> 1. BFS from 0: [0]; from 1: [1, 2]. Reversed: 2, 1, 0.
    assert orders[0].tolist() == [2, 1, 0]
    _, orders, _ = meshes.reorder(m, "input")
    assert orders[0].tolist() == [0, 1, 2]


def rcm_restated(cell: str, cells: np.ndarray) -> list:
    """Reverse Cuthill-McKee as order.rs states it, in plain Python: the facet graph from the
    reference cell's facets (the golden tables), components started at the least (degree,
    position) cell, neighbours queued by (degree, position), the whole order reversed."""
    import json
    import pathlib

    tables = json.loads((pathlib.Path(__file__).parent / "golden" / "refcell_tables.json").read_text())
    td = {"Triangle": 2, "Quadrilateral": 2, "Tetrahedron": 3, "Hexahedron": 3, "Prism": 3}[cell]
    facets = tables[cell]["sub_entities"][td - 1]
    owners = {}
    for c, row in enumerate(cells):
        for f in facets:
            owners.setdefault(tuple(sorted(int(row[j]) for j in f)), []).append(c)
    adj = [set() for _ in range(len(cells))]
    for cs in owners.values():
        for a in cs:
            adj[a].update(b for b in cs if b != a)
    rank = lambda c: (len(adj[c]), c)
    seen, order = [False] * len(cells), []
    for s in sorted(range(len(cells)), key=rank):
        if seen[s]:
            continue
        seen[s] = True
        head = len(order)
        order.append(s)
        while head < len(order):
            a = order[head]
            head += 1
            nxt = sorted((b for b in adj[a] if not seen[b]), key=rank)
            for b in nxt:
                seen[b] = True
            order.extend(nxt)
    return order[::-1]


@pytest.mark.parametrize("cell,dim,n,degree", [("Tetrahedron", 3, 4, 2), ("Hexahedron", 3, 4, 1), ("Prism", 3, 3, 2),
                                                ("Triangle", 2, 7, 3), ("Quadrilateral", 2, 6, 2)])
def test_rcm_matches_the_restatement(cell, dim, n, degree):
    """The library's reverse Cuthill-McKee (a sorted facet-key graph) against the plain-Python
    restatement on shuffled boxes, prisms' triangle and quadrilateral facets included."""
    box = meshes.cube_box(cell, n, degree) if dim == 3 else meshes.square_box(cell, n, degree)
    mix = meshes.shuffled(box, seed=11)
    _, orders, _ = meshes.reorder(mix, "rcm")
    assert orders[0].tolist() == rcm_restated(cell, mix.blocks[0].cells)
