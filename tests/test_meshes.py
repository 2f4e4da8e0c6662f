"""Synthetic meshes: counts, numbering and orientation like the reference's generators (CPU)."""

import numpy as np
import pytest

from gridcl_gb300 import meshes
from oracle import oracle as orc
from oracle import refcell as rc


@pytest.mark.parametrize("cell,n,p,cells,nodes", [
    ("Tetrahedron", 8, 1, 3072, 729),
    ("Tetrahedron", 4, 2, 384, 9 ** 3),
    ("Hexahedron", 3, 2, 27, 7 ** 3),
    ("Prism", 3, 2, 54, 7 ** 3),
    ("Pyramid", 2, 1, 48, 27 + 8),
    ("Pyramid", 1, 2, 6, 27 + 8),  # the 3^3 P2 lattice of the cube, the 8 corner-to-apex midpoints
])
def test_cube_box_counts(cell, n, p, cells, nodes):
    m = meshes.cube_box(cell, n, p)
    assert m.blocks[0].num_cells == cells
    assert m.num_nodes == nodes
    # every node used; first-use numbering: node ids appear in increasing order of first use
    flat = m.blocks[0].cells.ravel()
    _, first = np.unique(flat, return_index=True)
    assert np.all(np.diff(first) > 0)


@pytest.mark.parametrize("cell", ["Tetrahedron", "Hexahedron", "Prism", "Pyramid"])
def test_cells_are_positively_oriented(cell):
    m = meshes.curved_box(cell, 3, 2, jitter=0.02)
    pts, _ = rc.gauss_rule(cell, 4)
    d = orc.eval_block(cell, 2, m.nodes, m.blocks[0].cells, pts, factors=("detj",))["detj"]
    assert np.all(d > 0)


def test_lagrange_nodes_are_the_mapped_reference_nodes():
    m = meshes.cube_box("Tetrahedron", 2, 2)
    ref = rc.lagrange_points("Tetrahedron", 2)
    c = m.blocks[0].cells
    x = m.nodes[c]  # [cell][K][3]
    v = x[:, :4]
    mapped = v[:, :1] + np.einsum("kt,ctg->ckg", ref, v[:, 1:4] - v[:, :1])
    assert np.abs(mapped - x).max() < 1e-15


def test_sphere_counts_and_radius():
    m = meshes.sphere(2, 2)
    assert m.blocks[0].num_cells == 20 * 16
    assert np.allclose(np.linalg.norm(m.nodes, axis=1), 1.0)
    # Euler: V = 10 * 4^r * p^2 + 2 for the degree-p lattice of the refined icosahedron
    assert m.num_nodes == 10 * 16 * 4 + 2
    t = meshes.sphere(2, 2, max_cells=100)
    assert t.blocks[0].num_cells == 100


def test_splitmix64_first_values():
    # SplitMix64(0): the published first outputs of the generator.
    z = meshes.splitmix64(0, 2)
    assert int(z[0]) == 0xE220A8397B1DCDAF
    assert int(z[1]) == 0x6E789E6AA1B965F4


def test_mixed_boxes_match_the_reference_examples():
    """boxes.rs's documented examples: mixed_box(2, 1) has 4 tetrahedra, 4 hexahedra and 22
    pyramids on 27 corners and 4 centres; hex_prism_pyramid_box(3, 1) 9 hexahedra, 18 prisms and
    54 pyramids."""
    m = meshes.mixed_box(2, 1)
    assert [(b.cell, b.num_cells) for b in m.blocks] == [("Tetrahedron", 4), ("Hexahedron", 4), ("Pyramid", 22)]
    assert m.num_nodes == 27 + 4
    h = meshes.hex_prism_pyramid_box(3, 1)
    assert [(b.cell, b.num_cells) for b in h.blocks] == [("Hexahedron", 9), ("Prism", 18), ("Pyramid", 54)]


@pytest.mark.parametrize("p", [1, 2, 3])
def test_mixed_boxes_are_conforming_with_unit_volume(p):
    """Every node used, numbered by first use over the cells in generation order; no two nodes
    at the same point (shared high-order nodes found across blocks); positive det J at Gauss
    points; volume 1 by the oracle (rule degree 3p integrates the pyramids' rational det J of
    these affine maps exactly)."""
    for m in (meshes.mixed_box(3, p), meshes.hex_prism_pyramid_box(3, p)):
        used = np.zeros(m.num_nodes, dtype=bool)
        for b in m.blocks:
            used[b.cells.ravel()] = True
        assert used.all()
        keys = np.rint(m.nodes * (2 * 3 * p)).astype(np.int64)
        assert np.unique(keys, axis=0).shape[0] == m.num_nodes
        vol = 0.0
        for b in m.blocks:
            pts, w = rc.gauss_rule(b.cell, 3 * p)
            d = orc.eval_block(b.cell, p, m.nodes, b.cells, pts, factors=("detj",))["detj"][..., 0]
            assert d.min() > 0, b.cell
            vol += orc.measure(d, w)
        assert abs(vol - 1.0) < 1e-12
