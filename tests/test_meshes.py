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
])
def test_cube_box_counts(cell, n, p, cells, nodes):
    m = meshes.cube_box(cell, n, p)
    assert m.blocks[0].num_cells == cells
    assert m.num_nodes == nodes
    # every node used; first-use numbering: node ids appear in increasing order of first use
    flat = m.blocks[0].cells.ravel()
    _, first = np.unique(flat, return_index=True)
    assert np.all(np.diff(first) > 0)


@pytest.mark.parametrize("cell", ["Tetrahedron", "Hexahedron", "Prism"])
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
