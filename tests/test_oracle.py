"""The oracle pinned against the reference's golden fixtures and known-answer tests (CPU)."""

import json
import math
import pathlib

import numpy as np
import pytest

from oracle import oracle as orc
from oracle import refcell as rc

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
CELLS = ["Interval", "Triangle", "Quadrilateral", "Tetrahedron", "Hexahedron", "Prism"]
VOLUME = {"Interval": 1.0, "Quadrilateral": 1.0, "Hexahedron": 1.0, "Triangle": 0.5,
          "Prism": 0.5, "Tetrahedron": 1.0 / 6.0, "Pyramid": 1.0 / 3.0}


def test_reference_cell_tables_match_fixture():
    """tetraloma-refcell/tests/fixtures.rs:55-89 (tables.json, exported from ndelement)."""
    tables = json.loads((GOLDEN / "refcell_tables.json").read_text())
    assert len(tables) == 8
    for name, t in tables.items():
        assert rc.tdim(name) == t["tdim"]
        want = np.array([x for v in t["vertices"] for x in v])
        assert np.array_equal(rc.vertices(name).ravel(), want), name
        for dim in range(4):
            assert rc.sub_entities(name, dim) == t["sub_entities"][dim], (name, dim)
            assert rc.sub_entity_types(name, dim) == t["sub_entity_types"][dim], (name, dim)


def test_lagrange_points_match_fixture():
    """fixtures.rs:132-193: node by node, 1e-14 absolute, p = 1..4, equispaced and GLL."""
    fixture = json.loads((GOLDEN / "lagrange_points.json").read_text())
    assert sorted(fixture) == ["Hexahedron", "Interval", "Quadrilateral", "Tetrahedron", "Triangle"]
    for name, families in fixture.items():
        for family, degrees in families.items():
            assert sorted(int(p) for p in degrees) == [1, 2, 3, 4]
            for p, want in degrees.items():
                ours = rc.lagrange_points(name, int(p), family).ravel()
                assert ours.size == len(want)
                assert np.abs(ours - np.array(want)).max() <= 1e-14, (name, family, p)


@pytest.mark.parametrize("cell", CELLS + ["Pyramid"])
def test_rule_weights_sum_to_the_volume(cell):
    """quadrature.rs:206-220 and point_count_is_m_to_the_tdim (quadrature.rs:240-249)."""
    for n in range(0, 21):
        pts, w = rc.gauss_rule(cell, n)
        v = VOLUME[cell]
        assert abs(w.sum() - v) / v <= 1e-14
        assert np.all(w > 0)
        assert w.size == (n // 2 + 1) ** rc.tdim(cell)


def test_gauss_jacobi_closed_forms():
    """jacobi.rs tests: Gauss-Legendre m = 2, 3 and Gauss-Jacobi(1) m = 1, 2 closed forms."""
    x, w = rc.gauss_jacobi(2, 0.0)
    d = 0.5 / math.sqrt(3.0)
    assert np.allclose(x, [0.5 - d, 0.5 + d], atol=1e-15) and np.allclose(w, [0.5, 0.5], atol=1e-15)
    x, w = rc.gauss_jacobi(3, 0.0)
    d = 0.5 * math.sqrt(0.6)
    assert np.allclose(x, [0.5 - d, 0.5, 0.5 + d], atol=1e-15)
    assert np.allclose(w, [5 / 18, 8 / 18, 5 / 18], atol=1e-15)
    x, w = rc.gauss_jacobi(1, 1.0)
    assert abs(x[0] - 1 / 3) < 1e-15 and abs(w[0] - 0.5) < 1e-15
    x, w = rc.gauss_jacobi(2, 1.0)
    d = math.sqrt(6.0) / 10.0
    assert np.allclose(x, [0.4 - d, 0.4 + d], atol=1e-15)
    # exactness to degree 2m - 1 for (1 - x)^alpha
    for alpha in (0, 1, 2):
        for m in range(1, 12):
            x, w = rc.gauss_jacobi(m, float(alpha))
            for k in range(2 * m):
                exact = math.factorial(k) * math.factorial(alpha) / math.factorial(k + alpha + 1)
                assert abs(np.dot(w, x ** k) - exact) <= 1e-14 * max(1.0, exact) * 10


@pytest.mark.parametrize("cell", CELLS)
def test_tabulation_is_lagrange(cell):
    """tabulation.rs: Kronecker at the nodes; partition of unity; derivatives reproduce the
    space (exact gradients of linear functions)."""
    td = rc.tdim(cell)
    for p in range(1, 6):
        e = rc.LagrangeElement(cell, p)
        assert np.abs(e.tabulate(e.points, 0)[0] - np.eye(e.dim)).max() < 1e-12
        pts, _ = rc.gauss_rule(cell, 2 * p)
        t = e.tabulate(pts, 1)
        assert np.abs(t[0].sum(axis=1) - 1.0).max() < 1e-12
        for d in range(td):
            # the interpolant of x_d has gradient e_d
            grad = t[1:] @ e.points[:, d]
            want = np.zeros((td, pts.shape[0]))
            want[d] = 1.0
            assert np.abs(grad - want).max() < 1e-10


def test_pyramid_interior_nodes():
    """lagrange.rs's interior block of the P4 pyramid: i2 = 1 gives i0, i1 in 1..=2 (i0 fastest),
    i2 = 2 gives (1, 1)."""
    pts = rc.lagrange_points("Pyramid", 4)
    want = np.array([[1, 1, 1], [2, 1, 1], [1, 2, 1], [2, 2, 1], [1, 1, 2]]) / 4.0
    assert pts.shape == (55, 3)
    assert np.array_equal(pts[-5:], want)


def _rationomial(a, b, c, x):
    """x^a y^b z^c / (1 - z)^min(a, b) and its gradient, strictly inside the pyramid (the value
    also at the apex, where it is 0 for min(a, b) >= 1)."""
    r = min(a, b)
    s = 1.0 - x[:, 2]
    pw = lambda v, k: v ** k if k >= 0 else np.zeros_like(v)
    base = pw(x[:, 0], a) * pw(x[:, 1], b) * pw(x[:, 2], c)
    with np.errstate(divide="ignore", invalid="ignore"):
        v = np.where(s == 0.0, 0.0 if r else base, base / np.where(s == 0.0, 1.0, s) ** r)
    dx = a * pw(x[:, 0], a - 1) * pw(x[:, 1], b) * pw(x[:, 2], c) / s ** r
    dy = b * pw(x[:, 0], a) * pw(x[:, 1], b - 1) * pw(x[:, 2], c) / s ** r
    dz = c * pw(x[:, 0], a) * pw(x[:, 1], b) * pw(x[:, 2], c - 1) / s ** r + r * base / s ** (r + 1)
    return v, np.stack([dx, dy, dz])


def test_pyramid_space_is_reproduced():
    """tabulation.rs:418-520: Kronecker at the nodes; the interpolant of every rationomial of the
    space reproduces its values and first derivatives at the points of gauss_rule(Pyramid, 2p)
    (1e-10 relative to the largest derivative there), p = 1..5."""
    for p in range(1, 6):
        e = rc.LagrangeElement("Pyramid", p)
        assert np.abs(e.tabulate(e.points, 0)[0] - np.eye(e.dim)).max() < 1e-12
        pts, _ = rc.gauss_rule("Pyramid", 2 * p)
        t = e.tabulate(pts, 1)
        for a, b, c in rc.pyramid_exponents(p):
            fn, _ = _rationomial(a, b, c, e.points)
            v, g = _rationomial(a, b, c, pts)
            assert np.abs(t[0] @ fn - v).max() <= 1e-12 * max(1.0, np.abs(v).max())
            if (a, b, c) != (0, 0, 0):
                assert np.abs(t[1:] @ fn - g).max() <= 1e-10 * np.abs(g).max(), (p, a, b, c)


def test_pyramid_apex_is_the_axis_limit():
    """pyramid.rs:176-200: the values and derivatives at the apex are the limits along the axis
    x = y = (1 - z) / 2 (a power of two apart, so the near point is exact)."""
    eps = 2.0 ** -40
    for p in range(1, 5):
        apex = rc.tabulate("Pyramid", p, np.array([[0.0, 0.0, 1.0]]), 1)
        near = rc.tabulate("Pyramid", p, np.array([[eps / 2, eps / 2, 1.0 - eps]]), 1)
        assert np.abs(apex - near).max() <= 1e-6 * max(1.0, np.abs(near).max()), p


def test_pyramid_rules_integrate_the_space():
    """quadrature.rs:39-41: gauss_rule(Pyramid, p) is exact for the rationomials of degree p:
    the integral of x^a y^b z^c / (1 - z)^r over the pyramid (x = xi s, y = eta s) is
    c! q! / (c + q + 1)! / ((a + 1)(b + 1)) with q = a + b - r + 2."""
    for p in range(0, 9):
        pts, w = rc.gauss_rule("Pyramid", p)
        for a, b, c in rc.pyramid_exponents(p):
            q = a + b - min(a, b) + 2
            exact = math.factorial(c) * math.factorial(q) / math.factorial(c + q + 1) / ((a + 1) * (b + 1))
            v, _ = _rationomial(a, b, c, pts)
            assert abs(np.dot(w, v) - exact) <= 1e-14 * 10, (p, a, b, c)


def test_pinv_is_a_left_inverse():
    """tetraloma-testing/src/reference.rs:907-929, through the C oracle's per-point math."""
    cases = [(1, 1, [2.0]), (1, 3, [1.0, 2.0, 0.5]), (2, 2, [1.0, 0.2, -0.3, 2.0]),
             (2, 3, [1.0, 0.2, 0.1, -0.3, 2.0, 0.4]),
             (3, 3, [1.0, 0.2, 0.1, -0.3, 2.0, 0.4, 0.5, 0.1, 3.0])]
    cell = {1: "Interval", 2: "Triangle", 3: "Tetrahedron"}
    for td, gd, j in cases:
        # An affine cell whose J is the given matrix: vertices v0 = 0, v_{d+1} = column d.
        jm = np.array(j).reshape(td, gd)  # row d = column d of J
        verts = np.vstack([np.zeros(gd), jm])
        pts = np.full((1, td), 0.2)
        out = orc.eval_block(cell[td], 1, verts, np.arange(td + 1, dtype=np.uint32)[None, :], pts,
                             factors=("j", "k"))
        jj = out["j"][0, 0].reshape(td, gd)
        assert np.allclose(jj, jm, atol=1e-15)
        k = out["k"][0, 0].reshape(gd, td)  # K(t, g) at g * TD + t
        assert np.abs(k.T @ jj.T - np.eye(td)).max() < 1e-14


def _square_quads():
    # 2 x 2 quadrilaterals of the unit square, Q1, lexicographic vertices.
    nodes, cells = [], []
    for j in range(3):
        for i in range(3):
            nodes.append([i / 2, j / 2])
    for j in range(2):
        for i in range(2):
            v = j * 3 + i
            cells.append([v, v + 1, v + 3, v + 4])
    return np.array(nodes), np.array(cells, dtype=np.uint32)


def test_known_answers_on_quadrilaterals():
    """det J = 1/4, J = I/2, K = 2I on 2 x 2 quadrilaterals (tetraloma-geometry/src/lib.rs:69-76,
    points_jac.rs:672-679, detj_pinv.rs:774-781)."""
    nodes, cells = _square_quads()
    pts, _ = rc.gauss_rule("Quadrilateral", 2)
    out = orc.eval_block("Quadrilateral", 1, nodes, cells, pts, factors=("j", "detj", "k"))
    assert np.allclose(out["detj"], 0.25, atol=1e-15)
    assert np.allclose(out["j"], [0.5, 0.0, 0.0, 0.5], atol=1e-15)
    assert np.allclose(out["k"], [2.0, 0.0, 0.0, 2.0], atol=1e-14)


def test_unit_volume_and_constant_affine_detj():
    """unit_volume.rs (1e-12) and factors.rs:151-185 (det J constant on affine cells)."""
    from gridcl_gb300 import meshes

    for cell in ("Tetrahedron", "Hexahedron", "Prism", "Pyramid"):
        m = meshes.cube_box(cell, 3, 1)
        b = m.blocks[0]
        pts, w = rc.gauss_rule(cell, 2)
        out = orc.eval_block(cell, 1, m.nodes, b.cells, pts, factors=("detj",))
        assert abs(orc.measure(out["detj"][..., 0], w) - 1.0) < 1e-12
        d = out["detj"][..., 0]
        if cell != "Hexahedron" or True:
            assert np.abs(d - d[:, :1]).max() < 1e-14
        assert np.all(d > 0)


def test_evector_clamps_and_pads():
    """evector.rs:195-236: padding lanes repeat the last cell; indices past the last node read
    the last node; the copy is bit-exact."""
    nodes = np.arange(12, dtype=np.float64).reshape(4, 3) + 0.125
    dofmap = np.array([[0, 1], [3, 9]], dtype=np.uint32)  # 9 is past the last node
    xe = orc.evector(nodes, dofmap, 2, 2, 3, 0, 16, 16)
    assert xe.shape == (2, 3, 16)
    assert np.array_equal(xe[1, :, 1], nodes[3])  # clamped
    assert np.array_equal(xe[:, :, 5], xe[:, :, 1])  # padding repeats the last cell
    assert np.array_equal(xe[0, :, 0], nodes[0])


def test_rel_err_semantics():
    """reference.rs:786-817."""
    assert abs(orc.rel_err([1.0, 1.1e-3, 1e-3, 2.0], [1.0, 1e-3, 1e-3, 2.0]) - 5e-5) < 1e-15
    assert orc.rel_err([1e-3], [0.0]) == 1e-3
    assert orc.rel_err([1.0, float("nan")], [1.0, 1.0]) == float("inf")


@pytest.mark.parametrize("cell,degree", [("Tetrahedron", 2), ("Hexahedron", 2), ("Prism", 2), ("Tetrahedron", 1)])
def test_oracle_pull_back_round_trip(cell, degree):
    """The oracle's Newton pull-back returns the Gauss points of curved cells from their images
    (pull_back.rs's documented property), every point converged."""
    from gridcl_gb300 import meshes
    m = meshes.curved_box(cell, 2, degree, jitter=0.02)
    pts, _ = rc.gauss_rule(cell, 4)
    x = orc.eval_block(cell, degree, m.nodes, m.blocks[0].cells, pts, factors=("x",))["x"]
    xi, step = orc.pull_back(cell, degree, m.nodes, m.blocks[0].cells, x)
    assert np.abs(xi - pts[None]).max() < 1e-13
    assert step.max() <= 1e-13


def test_oracle_pull_back_centres_and_outside_points():
    """Cell centres of an affine square pull back to the reference centre (pull_back.rs's
    example); a point outside its cell stays in the clamp box and does not converge."""
    from gridcl_gb300 import meshes
    m = meshes.square_box("Quadrilateral", 2, 1)
    cells = m.blocks[0].cells
    centres = m.nodes[cells].mean(axis=1)[:, None, :]
    xi, step = orc.pull_back("Quadrilateral", 1, m.nodes, cells, centres, tolerance=1e-5)
    assert np.allclose(xi, 0.5, atol=1e-12) and step.max() <= 1e-5
    far = centres + np.array([0.0, 2.0])  # two cell widths away
    xi, step = orc.pull_back("Quadrilateral", 1, m.nodes, cells, far, tolerance=1e-5)
    assert np.all(xi <= float(np.float32(1.1))) and np.all(step > 1e-5)


def _circle(n, degree, radius=1.0):
    """n curved intervals of degree `degree` on a circle (nodes of each interval equispaced in
    angle, interior nodes first after the two vertices, as the interval's Lagrange order)."""
    from gridcl_gb300 import meshes
    nodes, cells = [], []
    per = degree  # nodes per interval beyond its first vertex
    for c in range(n):
        cells.append([c * per, ((c + 1) * per) % (n * per)] + [c * per + i for i in range(1, degree)])
    for i in range(n * per):
        t = 2 * np.pi * i / (n * per)
        r = radius * (1 + 0.05 * np.sin(3 * t))
        nodes.append([r * np.cos(t), r * np.sin(t)])
    return meshes.HostMesh(2, np.array(nodes), [meshes.HostBlock("Interval", degree, np.array(cells, dtype=np.uint32))])


@pytest.mark.parametrize("kind", ["sphere", "circle"])
def test_surface_adjoint_against_central_differences(kind):
    """The oracle's adjoint below codimension 0 (area element, pseudo-inverse, unit normals with
    flipped cells) against central differences (step 1e-6) of the oracle's own forward pass."""
    from gridcl_gb300 import meshes
    if kind == "sphere":
        mesh = meshes.perturbed_radius(meshes.sphere(1, 2), 0.05)
        cell, degree, pts = "Triangle", 2, rc.gauss_rule("Triangle", 4)[0]
    else:
        mesh = _circle(7, 3)
        cell, degree, pts = "Interval", 3, rc.gauss_rule("Interval", 5)[0]
    cells = mesh.blocks[0].cells
    x = np.asarray(mesh.nodes, dtype=np.float64)
    nc, nq, gd, td = cells.shape[0], len(pts), x.shape[1], rc.tdim(cell)
    rng = np.random.default_rng(21)
    xb, db = rng.standard_normal((nc, nq, gd)), rng.standard_normal((nc, nq))
    kb, nb = rng.standard_normal((nc, nq, td * gd)), rng.standard_normal((nc, nq, gd))
    flags = rng.integers(0, 2, nc).astype(np.uint32)
    grad = orc.vjp(cell, degree, x, cells, pts, xb, db, kb, nbar=nb, flags=flags)

    def functional(y):
        f = orc.eval_block(cell, degree, y, cells, pts, factors=("x", "detj", "k", "normals"), flags=flags)
        return (np.sum(f["x"] * xb) + np.sum(f["detj"][..., 0] * db) + np.sum(f["k"] * kb)
                + np.sum(f["normals"] * nb))

    h = 1e-6
    for n in rng.choice(x.shape[0], 6, replace=False):
        for g in range(gd):
            xp, xm = x.copy(), x.copy()
            xp[n, g] += h
            xm[n, g] -= h
            fd = (functional(xp) - functional(xm)) / (2 * h)
            assert abs(fd - grad[n, g]) <= 1e-6 * max(1.0, abs(grad[n, g])), (n, g, fd, grad[n, g])
