"""The product's native reference-cell tables against the golden fixtures and the oracle (CPU)."""

import json
import pathlib

import numpy as np
import pytest

from gridcl_gb300 import refcell as pr
from oracle import refcell as rc

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
CELLS = ["Interval", "Triangle", "Quadrilateral", "Tetrahedron", "Hexahedron", "Prism"]


def test_lagrange_points_match_fixture():
    fixture = json.loads((GOLDEN / "lagrange_points.json").read_text())
    for name, families in fixture.items():
        for family, degrees in families.items():
            for p, want in degrees.items():
                ours = pr.lagrange_points(name, int(p), family).ravel()
                assert np.abs(ours - np.array(want)).max() <= 1e-14, (name, family, p)


@pytest.mark.parametrize("cell", CELLS + ["Pyramid"])
def test_rules_match_the_oracle(cell):
    for n in range(0, 16):
        a, b = pr.gauss_rule(cell, n), rc.gauss_rule(cell, n)
        assert np.abs(a[0] - b[0]).max() < 1e-14 and np.abs(a[1] - b[1]).max() < 1e-14


@pytest.mark.parametrize("cell", CELLS)
def test_tabulation_matches_the_oracle(cell):
    # Degrees 1-8, as the reference's high-order acceptance tests; values and derivatives
    # relative to their largest magnitude.
    for p in range(1, 9):
        pts, _ = rc.gauss_rule(cell, 2 * p)
        for fam in (["Equispaced", "Gll"] if cell in ("Interval", "Quadrilateral", "Hexahedron") else ["Equispaced"]):
            want = rc.tabulate(cell, p, pts, 1, fam)
            err = np.abs(pr.tabulate(cell, p, pts, 1, fam) - want).max() / np.abs(want).max()
            assert err < 5e-14, (cell, p, fam, err)


def test_pyramid_tabulation_matches_the_oracle():
    """The product's orthogonal-rationomial expansion (LU in f64) against the oracle's centred
    rationomials (inverted exactly), degrees 1-5, values and derivatives at Gauss points, the
    Lagrange nodes and the apex."""
    for p in range(1, 6):
        pts, _ = rc.gauss_rule("Pyramid", 2 * p)
        for x in (pts, rc.lagrange_points("Pyramid", p), np.array([[0.0, 0.0, 1.0]])):
            want = rc.tabulate("Pyramid", p, x, 1)
            err = np.abs(pr.tabulate("Pyramid", p, x, 1) - want).max() / np.abs(want).max()
            assert err < 5e-14, (p, err)


@pytest.mark.parametrize("cell", CELLS + ["Pyramid"])
def test_facet_normals_match_the_oracle(cell):
    assert np.array_equal(pr.reference_facet_normals(cell), rc.reference_facet_normals(cell))


def test_unsupported_and_bad_input():
    from gridcl_gb300 import GridError

    with pytest.raises(GridError) as e:
        pr.lagrange_points("Triangle", 2, "Gll")
    assert e.value.kind == "InvalidArgument"
    with pytest.raises(GridError):
        pr.tabulate("Pyramid", 2, np.zeros((1, 3)), family="Gll")
