"""Evaluation strategies (GPU): the paired/unrolled, loops and sum-factorised kernels against the
oracle for quadrilaterals and hexahedra at tensor-product rules, in f64, f32 and split
precision, with the kernel family that ran recorded per launch (the reference's strategy tests,
tetraloma-geometry/tests/strategy.rs)."""

import numpy as np
import pytest
import torch

import gridcl_gb300 as tg
from gridcl_gb300 import meshes
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

F64, F32 = torch.float64, torch.float32
KEYS = {"points": "x", "jacobian": "j", "detj": "detj", "pinv": "k", "normals": "normals"}


def quad_box(n, degree, gd):
    """The unit square of n^2 quadrilaterals, interior nodes jittered; with gd = 3 lifted to the
    surface z = 0.1 sin(2 pi x) sin(2 pi y)."""
    m = meshes.square_box("Quadrilateral", n, degree)
    x = meshes.jitter_interior(m.nodes, m.nodes, 0.02 / n, 2026)
    if gd == 3:
        z = 0.1 * np.sin(2 * np.pi * x[:, 0]) * np.sin(2 * np.pi * x[:, 1])
        x = np.column_stack([x, z])
        m = meshes.HostMesh(3, x, m.blocks)
    else:
        m.nodes = x
    return m


CASES = [
    # (cell, n, degree, rule degree, gdim)
    ("Hexahedron", 3, 1, 2, 3),
    ("Hexahedron", 3, 2, 4, 3),
    ("Hexahedron", 2, 3, 6, 3),
    ("Quadrilateral", 4, 1, 2, 2),
    ("Quadrilateral", 4, 2, 4, 2),
    ("Quadrilateral", 3, 3, 6, 2),
    ("Quadrilateral", 3, 4, 8, 2),
    ("Quadrilateral", 2, 5, 10, 2),
    ("Quadrilateral", 4, 2, 4, 3),
    ("Quadrilateral", 3, 4, 8, 3),
    ("Prism", 3, 1, 2, 3),
    ("Prism", 3, 2, 4, 3),
    ("Prism", 2, 3, 6, 3),
]


def mesh_for(cell, n, degree, gd):
    return meshes.curved_box(cell, n, degree, jitter=0.02) if cell != "Quadrilateral" else quad_box(n, degree, gd)


def factors_for(gd, td):
    return ("points", "jacobian", "detj", "pinv") + (("normals",) if td + 1 == gd else ())


@pytest.mark.parametrize("precision", ["f64", "f32", "split"])
@pytest.mark.parametrize("strategy", ["direct", "loops", "sumfact", "shared", "cooperative", "tensor"])
@pytest.mark.parametrize("cell,n,degree,rdeg,gd", CASES)
def test_strategies_match_the_oracle(cuda, cell, n, degree, rdeg, gd, strategy, precision):
    mesh = mesh_for(cell, n, degree, gd)
    td = 2 if cell == "Quadrilateral" else 3
    g = tg.Geometry.from_host(mesh, dtype=F32 if precision == "f32" else F64)
    pts, _ = tg.refcell.gauss_rule(cell, rdeg)
    ps = tg.PointSet(cell, pts, np.ones(len(pts)))
    names = factors_for(gd, td)
    with tg.with_strategy(strategy):
        got = tg.geometric_factors_block(g, 0, ps, names, precision="split" if precision == "split" else "native")
        family = tg.last_kernel_family()
    k = mesh.blocks[0].cells.shape[1]
    if strategy == "tensor":  # f32 and split tables of more than 10 nodes; loops elsewhere
        assert family == ("tensor" if precision != "f64" and k > 10 else "loops")
    elif strategy in ("sumfact", "loops", "cooperative"):
        assert family == strategy
    elif strategy == "shared":  # tables beyond the shared-memory budget stay in global memory
        assert family in ("shared", "loops")
    else:  # where no unrolled kernel applies, the loops kernel over staged tables runs
        assert family in ("direct", "loops", "shared")
    absx = g.nodes.double().cpu().numpy() + np.array(g.origin[:gd])
    want = orc.eval_block(cell, degree, absx, mesh.blocks[0].cells, pts, factors=[KEYS[f] for f in names])
    base = orc.TOL_F64 if precision == "f64" else orc.TOL_F32
    nodes = orc.node_ratio(cell, degree)
    s_val = orc.tolerance_scale(cell, degree, "Equispaced", pts, "values") * nodes
    s_der = orc.tolerance_scale(cell, degree, "Equispaced", pts) * nodes
    if precision == "f32":  # coordinates rounded relative to the origin
        ratio = orc.origin_ratio(absx, np.array(g.origin[:gd]), want["j"])
        s_val, s_der = s_val * ratio, s_der * ratio
    cond = orc.condition_scale(want["j"], td, gd)
    scale = {"points": s_val, "jacobian": s_der, "detj": s_der, "pinv": s_der * cond, "normals": s_der * cond}
    for f in names:
        err = orc.rel_err(got[f].to_host_cell_major(), want[KEYS[f]])
        assert err < base * scale[f], (f, err, base * scale[f])


def test_sumfact_needs_a_tensor_rule(cuda):
    """A point set that is not a tensor product (a shuffled Gauss rule) runs another family under
    the sumfact strategy, with the same values."""
    mesh = meshes.curved_box("Hexahedron", 2, 2, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    pts, _ = tg.refcell.gauss_rule("Hexahedron", 4)
    perm = np.random.default_rng(3).permutation(len(pts))
    shuffled = tg.PointSet("Hexahedron", pts[perm], np.ones(len(pts)))
    with tg.with_strategy("sumfact"):
        got = tg.geometric_factors_block(g, 0, shuffled, ("jacobian",))
        assert tg.last_kernel_family() != "sumfact"
    with tg.with_strategy("sumfact"):
        tensor = tg.geometric_factors_block(g, 0, tg.PointSet("Hexahedron", pts, np.ones(len(pts))), ("jacobian",))
        assert tg.last_kernel_family() == "sumfact"
    a = got["jacobian"].to_host_cell_major()
    b = tensor["jacobian"].to_host_cell_major()[:, perm]
    assert orc.rel_err(a, b) < 1e-13


@pytest.mark.parametrize("precision,degree,family", [("f64", 2, "sumfact"), ("f64", 1, "sumfact"),
                                                     ("split", 2, "direct"), ("split", 3, "sumfact"),
                                                     ("f32", 2, "direct"), ("f32", 3, "sumfact")])
def test_auto_policy(cuda, precision, degree, family):
    mesh = meshes.curved_box("Hexahedron", 2, degree, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=F32 if precision == "f32" else F64)
    pts, _ = tg.refcell.gauss_rule("Hexahedron", 2 * degree)
    ps = tg.PointSet("Hexahedron", pts, np.ones(len(pts)))
    with tg.with_strategy("auto"):
        tg.geometric_factors_block(g, 0, ps, ("detj",), precision="split" if precision == "split" else "native")
        assert tg.last_kernel_family() == family


def test_strategy_scopes_nest_and_restore(cuda):
    before = tg.get_strategy()
    with tg.with_strategy("loops"):
        assert tg.get_strategy() == "loops"
        with tg.with_strategy("sumfact"):
            assert tg.get_strategy() == "sumfact"
        assert tg.get_strategy() == "loops"
    assert tg.get_strategy() == before


@pytest.mark.parametrize("order", ["z_slowest", "z_fastest"])
@pytest.mark.parametrize("precision", ["f64", "split"])
def test_prism_rules_in_both_orders(cuda, order, precision):
    """A prism rule as triangle points times z points runs sum factorisation with z the slowest
    or the fastest index; the values match those of the same rule under the direct strategy."""
    mesh = meshes.curved_box("Prism", 2, 2, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    tri, _ = tg.refcell.gauss_rule("Triangle", 4)
    z = np.array([0.1, 0.45, 0.8, 0.95])
    if order == "z_slowest":
        pts = np.array([[a, b, c] for c in z for a, b in tri])
    else:
        pts = np.array([[a, b, c] for a, b in tri for c in z])
    ps = tg.PointSet("Prism", pts, np.ones(len(pts)))
    names = ("points", "jacobian", "detj", "pinv")
    prec = "split" if precision == "split" else "native"
    with tg.with_strategy("sumfact"):
        got = tg.geometric_factors_block(g, 0, ps, names, precision=prec)
        assert tg.last_kernel_family() == "sumfact"
    with tg.with_strategy("direct"):
        want = tg.geometric_factors_block(g, 0, ps, names, precision=prec)
    tol = 1e-13 if precision == "f64" else 2e-6
    for f in names:
        assert orc.rel_err(got[f].to_host_cell_major(), want[f].to_host_cell_major()) < tol, f


def test_prism_without_a_product_rule(cuda):
    """Points that are not unions of (x, y) sets times z sets run loops under sumfact."""
    mesh = meshes.curved_box("Prism", 2, 2, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    rng = np.random.default_rng(12)
    pts = rng.uniform(0.05, 0.45, size=(20, 3))
    with tg.with_strategy("sumfact"):
        tg.geometric_factors_block(g, 0, tg.PointSet("Prism", pts, np.ones(len(pts))), ("detj",))
        assert tg.last_kernel_family() != "sumfact"


HIGH = [
    # (cell, n, degree, rule degree, gdim): beyond the unrolled kernels
    ("Tetrahedron", 2, 4, 5, 3),
    ("Tetrahedron", 1, 5, 6, 3),
    ("Triangle", 3, 6, 8, 2),
    ("Triangle", 0, 5, 6, 3),
    ("Quadrilateral", 2, 6, 8, 2),
    ("Hexahedron", 2, 3, 5, 3),
]


def high_mesh(cell, n, degree, gd):
    if cell == "Triangle" and gd == 3:
        return meshes.perturbed_radius(meshes.sphere(1, degree), 0.02)
    if cell in ("Triangle", "Quadrilateral"):
        m = meshes.square_box(cell, n, degree)
        m.nodes = meshes.jitter_interior(m.nodes, m.nodes, 0.02 / n, 2026)
        return m
    return meshes.curved_box(cell, n, degree, jitter=0.02)


@pytest.mark.parametrize("precision", ["f64", "f32", "split"])
@pytest.mark.parametrize("strategy", ["auto", "loops", "shared", "cooperative", "tensor"])
@pytest.mark.parametrize("cell,n,degree,rdeg,gd", HIGH)
def test_high_degree_strategies(cuda, cell, n, degree, rdeg, gd, strategy, precision):
    """Cells of 21 to 64 nodes under the loops, shared and cooperative kernels (and AUTO, which
    picks the tcgen05 kernel above 27 nodes for f32 and split volume cells in 3D, the cooperative
    kernel for the others) against the oracle; a non-tensor rule (the collapsed Gauss rule of a
    hexahedron, shuffled) keeps sum factorisation out."""
    mesh = high_mesh(cell, n, degree, gd)
    td = refcell_tdim(cell)
    g = tg.Geometry.from_host(mesh, dtype=F32 if precision == "f32" else F64)
    pts, _ = tg.refcell.gauss_rule(cell, rdeg)
    pts = pts[np.random.default_rng(1).permutation(len(pts))]
    ps = tg.PointSet(cell, pts, np.ones(len(pts)))
    names = factors_for(gd, td)
    with tg.with_strategy(strategy):
        got = tg.geometric_factors_block(g, 0, ps, names, precision="split" if precision == "split" else "native")
        family = tg.last_kernel_family()
    k = mesh.blocks[0].cells.shape[1]
    if strategy == "auto":
        if k > 27 and precision != "f64" and td == gd == 3 and k <= 88:
            assert family == "tensor"  # the tcgen05 kernel
        elif k > 27:
            assert family == "cooperative"
        else:
            assert family in ("loops", "shared")
    elif strategy == "shared":  # tables beyond the shared-memory budget stay in global memory
        assert family in ("shared", "loops")
    elif strategy == "tensor":
        assert family == ("loops" if precision == "f64" else "tensor")
    else:
        assert family == strategy
    absx = g.nodes.double().cpu().numpy() + np.array(g.origin[:gd])
    want = orc.eval_block(cell, degree, absx, mesh.blocks[0].cells, pts, factors=[KEYS[f] for f in names])
    base = orc.TOL_F64 if precision == "f64" else orc.TOL_F32
    nodes = orc.node_ratio(cell, degree)
    s_val = orc.tolerance_scale(cell, degree, "Equispaced", pts, "values") * nodes
    s_der = orc.tolerance_scale(cell, degree, "Equispaced", pts) * nodes
    if precision == "f32":
        ratio = orc.origin_ratio(absx, np.array(g.origin[:gd]), want["j"])
        s_val, s_der = s_val * ratio, s_der * ratio
    cond = orc.condition_scale(want["j"], td, gd)
    scale = {"points": s_val, "jacobian": s_der, "detj": s_der, "pinv": s_der * cond, "normals": s_der * cond}
    for f in names:
        err = orc.rel_err(got[f].to_host_cell_major(), want[KEYS[f]])
        assert err < base * scale[f], (f, err, base * scale[f])


def refcell_tdim(cell):
    return tg.refcell.tdim(cell)


@pytest.mark.parametrize("tile", [1, 2, 4, 8, 16])
def test_cooperative_tiles_and_ranges(cuda, tile):
    """The cooperative kernel at every output tile and on a cell range that starts mid-block
    (ragged last warp run): the same values as the loops kernel."""
    mesh = meshes.curved_box("Tetrahedron", 2, 4, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    pts, _ = tg.refcell.gauss_rule("Tetrahedron", 5)
    ps = tg.PointSet("Tetrahedron", pts, np.ones(len(pts)))
    names = ("points", "jacobian", "detj", "pinv")
    with tg.with_strategy("cooperative"):
        got = tg.geometric_factors_block(g, 0, ps, names, tile=tile, max_chunk_cells=37)
        assert tg.last_kernel_family() == "cooperative"
    with tg.with_strategy("loops"):
        want = tg.geometric_factors_block(g, 0, ps, names, tile=tile, max_chunk_cells=37)
    for f in names:
        assert orc.rel_err(got[f].to_host_cell_major(), want[f].to_host_cell_major()) < 1e-14, f


@pytest.mark.parametrize("dtype", [F64, F32])
def test_cooperative_facet_normals(cuda, dtype):
    mesh = meshes.curved_box("Tetrahedron", 2, 4, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=dtype)
    ps = tg.facet_point_set("Tetrahedron", 4)
    with tg.with_strategy("cooperative"):
        got = tg.facet_normals_block(g, 0, ps).to_host_cell_major()
        assert tg.last_kernel_family() == "cooperative"
    with tg.with_strategy("loops"):
        want = tg.facet_normals_block(g, 0, ps).to_host_cell_major()
    assert orc.rel_err(got, want) < (1e-13 if dtype == F64 else 1e-5)


def test_cooperative_split_recomputes(cuda):
    """Split precision under the cooperative kernel counts the FP64 recomputes of points above the
    condition limit as the loops kernel does (up to points whose estimate rounds across the limit
    in the two summation orders)."""
    mesh = meshes.curved_box("Tetrahedron", 2, 4, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    pts, _ = tg.refcell.gauss_rule("Tetrahedron", 5)
    ps = tg.PointSet("Tetrahedron", pts, np.ones(len(pts)))
    counts = {}
    for strat in ("cooperative", "loops"):
        rec = torch.zeros(1, dtype=torch.int64, device="cuda")
        with tg.with_strategy(strat):
            tg.geometric_factors_block(g, 0, ps, ("detj", "pinv"), precision="split", cond_limit=1.5,
                                       recomputed=rec)
        counts[strat] = int(rec.item())
    assert counts["loops"] > 0
    assert abs(counts["cooperative"] - counts["loops"]) <= max(2, counts["loops"] // 100)


def test_per_family_settings_and_records(cuda):
    """A fused launch follows its principal family; a forced strategy that does not apply runs
    loops; record_strategies sees every launch with its family (testing.rs:11-43)."""
    mesh = meshes.curved_box("Hexahedron", 2, 2, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    pts, _ = tg.refcell.gauss_rule("Hexahedron", 4)
    ps = tg.PointSet("Hexahedron", pts, np.ones(len(pts)))
    with tg.record_strategies() as rec:
        with tg.with_strategy("loops", family="Points"), tg.with_strategy("sumfact", family="Jacobian"):
            tg.geometric_factors_block(g, 0, ps, ("points",))
            tg.geometric_factors_block(g, 0, ps, ("points", "detj"))
        with tg.with_strategy("sumfact"):
            tets = meshes.curved_box("Tetrahedron", 1, 2, jitter=0.0)
            gt = tg.Geometry.from_host(tets, dtype=F64)
            tp, _ = tg.refcell.gauss_rule("Tetrahedron", 2)
            tg.geometric_factors_block(gt, 0, tg.PointSet("Tetrahedron", tp, np.ones(len(tp))), ("detj",))
        with tg.with_strategy("direct", family="Normals"):
            sph = tg.Geometry.from_host(meshes.sphere(1, 2), dtype=F64)
            sp, _ = tg.refcell.gauss_rule("Triangle", 2)
            tg.geometric_factors_block(sph, 0, tg.PointSet("Triangle", sp, np.ones(len(sp))), ("normals",))
        g.evector(0, max_chunk_cells=None)
    assert rec[:4] == [("Points", "loops"), ("Jacobian", "sumfact"), ("Jacobian", "loops"), ("Normals", "direct")]
    assert rec[4][0] == "EVector"


def test_forced_strategy_that_does_not_apply_runs_loops(cuda):
    """Cooperative above 128 nodes and sum factorisation at a non-tensor rule fall back to loops
    (strategy.rs:400-404)."""
    mesh = meshes.curved_box("Tetrahedron", 1, 8, jitter=0.0)  # 165 nodes per cell
    g = tg.Geometry.from_host(mesh, dtype=F32)
    pts, _ = tg.refcell.gauss_rule("Tetrahedron", 4)
    ps = tg.PointSet("Tetrahedron", pts, np.ones(len(pts)))
    for strat in ("cooperative", "sumfact", "direct"):
        with tg.with_strategy(strat):
            tg.geometric_factors_block(g, 0, ps, ("detj",))
            assert tg.last_kernel_family() == "loops", strat


@pytest.mark.parametrize("precision", ["f64", "split"])
@pytest.mark.parametrize("cell,n,degree,fdeg", [("Quadrilateral", 3, 2, 4), ("Quadrilateral", 2, 3, 6),
                                                ("Hexahedron", 2, 1, 2), ("Hexahedron", 2, 2, 4),
                                                ("Hexahedron", 2, 3, 6), ("Prism", 2, 1, 2), ("Prism", 2, 2, 4),
                                                ("Prism", 2, 3, 6)])
def test_sumfact_on_facet_rules(cuda, cell, n, degree, fdeg, precision):
    """Facet rules are unions of tensor blocks (one per facet): det J, K and the facet normals run
    sum-factorised and agree with the loops kernel (the reference's
    forced_sumfact_runs_for_derived_factors_and_facet_rules, tests/strategy.rs:363-438)."""
    mesh = mesh_for(cell, n, degree, 2 if cell == "Quadrilateral" else 3)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    ps = tg.facet_point_set(cell, fdeg)
    names = ("detj", "pinv", "facet_normals")
    prec = "split" if precision == "split" else "native"
    with tg.with_strategy("sumfact"):
        got = tg.geometric_factors_block(g, 0, ps, names, precision=prec)
        assert tg.last_kernel_family() == "sumfact"
    with tg.with_strategy("loops"):
        want = tg.geometric_factors_block(g, 0, ps, names, precision=prec)
        assert tg.last_kernel_family() == "loops"
    tol = 1e-13 if precision == "f64" else 2e-5
    for f in names:
        assert orc.rel_err(got[f].to_host_cell_major(), want[f].to_host_cell_major()) < tol, f
    absx = g.nodes.double().cpu().numpy() + np.array(g.origin[:g.gdim])
    ref = orc.eval_block(cell, degree, absx, mesh.blocks[0].cells, ps.points, factors=("detj",))
    assert orc.rel_err(got["detj"].to_host_cell_major(), ref["detj"]) < (1e-12 if precision == "f64" else 1e-5)


@pytest.mark.parametrize("cell,degree,rdeg,dtype,prec", [
    ("Hexahedron", 2, 4, F64, "native"), ("Hexahedron", 3, 6, F64, "split"), ("Tetrahedron", 4, 5, F64, "split"),
    ("Tetrahedron", 2, 4, F32, "native"), ("Prism", 3, 6, F32, "native"), ("Triangle", 6, 8, F64, "native")])
def test_policy_matches_its_forced_choice_bitwise(cuda, cell, degree, rdeg, dtype, prec):
    """Under the policy the values are those of forcing the strategy it chose, bit for bit
    (tests/strategy.rs:138-182)."""
    mesh = high_mesh(cell, 2, degree, 2 if cell == "Triangle" else 3)
    g = tg.Geometry.from_host(mesh, dtype=dtype)
    pts, _ = tg.refcell.gauss_rule(cell, rdeg)
    ps = tg.PointSet(cell, pts, np.ones(len(pts)))
    names = ("points", "jacobian", "detj", "pinv")
    with tg.record_strategies() as rec:
        auto = tg.geometric_factors_block(g, 0, ps, names, precision=prec)
    chosen = rec[-1][1]
    with tg.with_strategy(chosen):
        forced = tg.geometric_factors_block(g, 0, ps, names, precision=prec)
        assert tg.last_kernel_family() == chosen
    for f in names:
        assert torch.equal(auto[f].chunks[0].data, forced[f].chunks[0].data), (f, chosen)


@pytest.mark.parametrize("precision", ["f32", "split"])
@pytest.mark.parametrize("cell,degree,rdeg,gd", [("Tetrahedron", 5, 6, 3), ("Tetrahedron", 3, 4, 3),
                                                 ("Triangle", 6, 8, 2), ("Triangle", 5, 6, 3),
                                                 ("Quadrilateral", 4, 5, 2)])
def test_tensor_kernel_against_the_oracle(cuda, cell, degree, rdeg, gd, precision):
    """The 3xTF32 tensor-core contraction on coordinates relative to each cell's first node against
    the oracle within the f32 tolerance (surfaces with flipped normals, an odd point count, a cell
    count that is not a multiple of 16): the mma fragment layout is the one the kernel assumes (a
    wrong one would not agree), and it stays within 4x of the FP32 cooperative kernel's error."""
    mesh = high_mesh(cell, 2, degree, gd)
    if cell == "Tetrahedron":
        mesh = mesh.first_cells(37)
    flags = np.random.default_rng(4).integers(0, 2, mesh.blocks[0].num_cells).astype(np.uint32)
    g = tg.Geometry.from_host(mesh, dtype=F32 if precision == "f32" else F64, flags=[flags])
    pts, _ = tg.refcell.gauss_rule(cell, rdeg)
    pts = pts[:-1]  # an odd number of points
    ps = tg.PointSet(cell, pts, np.ones(len(pts)))
    td = tg.refcell.tdim(cell)
    names = factors_for(gd, td)
    prec = "split" if precision == "split" else "native"
    with tg.with_strategy("tensor"):
        got = tg.geometric_factors_block(g, 0, ps, names, precision=prec)
        assert tg.last_kernel_family() == "tensor"
    with tg.with_strategy("cooperative"):
        coop = tg.geometric_factors_block(g, 0, ps, names, precision=prec)
    absx = g.nodes.double().cpu().numpy() + np.array(g.origin[:gd])
    keys = [KEYS[f] for f in names]
    want = orc.eval_block(cell, degree, absx, mesh.blocks[0].cells, pts, factors=keys, flags=flags)
    nodes = orc.node_ratio(cell, degree)
    s_val = orc.tolerance_scale(cell, degree, "Equispaced", pts, "values") * nodes
    s_der = orc.tolerance_scale(cell, degree, "Equispaced", pts) * nodes
    if precision == "f32":
        ratio = orc.origin_ratio(absx, np.array(g.origin[:gd]), want["j"])
        s_val, s_der = s_val * ratio, s_der * ratio
    cond = orc.condition_scale(want["j"], td, gd)
    scale = {"points": s_val, "jacobian": s_der, "detj": s_der, "pinv": s_der * cond, "normals": s_der * cond}
    for f in names:
        err = orc.rel_err(got[f].to_host_cell_major(), want[KEYS[f]])
        assert err < orc.TOL_F32 * scale[f], (f, err)
        base = orc.rel_err(coop[f].to_host_cell_major(), want[KEYS[f]])
        assert err < 8 * base + 1e-6, (f, err, base)  # 3xTF32 against FP32 arithmetic


def test_tensor_facet_normals(cuda):
    mesh = meshes.curved_box("Tetrahedron", 2, 4, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=F32)
    ps = tg.facet_point_set("Tetrahedron", 4)
    with tg.with_strategy("tensor"):
        got = tg.facet_normals_block(g, 0, ps).to_host_cell_major()
        assert tg.last_kernel_family() == "tensor"
    with tg.with_strategy("loops"):
        want = tg.facet_normals_block(g, 0, ps).to_host_cell_major()
    assert orc.rel_err(got, want) < 2e-5


@pytest.mark.parametrize("strategy,cell,degree,rdeg,dtype,prec", [
    ("sumfact", "Hexahedron", 2, 4, F64, "native"), ("sumfact", "Hexahedron", 2, 4, F64, "split"),
    ("sumfact", "Prism", 2, 4, F32, "native"), ("tensor", "Tetrahedron", 4, 5, F32, "native"),
    ("tensor", "Tetrahedron", 4, 5, F64, "split"), ("cooperative", "Tetrahedron", 4, 5, F64, "split")])
def test_chunked_ranges_equal_one_launch(cuda, strategy, cell, degree, rdeg, dtype, prec):
    """Chunks of at most 37 cells (32-cell ranges at block offsets, each chunk's own output) give
    the values of one launch over the block, bit for bit, for each kernel family."""
    mesh = meshes.curved_box(cell, 3, degree, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=dtype)
    pts, _ = tg.refcell.gauss_rule(cell, rdeg)
    ps = tg.PointSet(cell, pts, np.ones(len(pts)))
    names = ("points", "jacobian", "detj", "pinv")
    with tg.with_strategy(strategy):
        whole = tg.geometric_factors_block(g, 0, ps, names, precision=prec)
        assert tg.last_kernel_family() == strategy
        parts = tg.geometric_factors_block(g, 0, ps, names, precision=prec, max_chunk_cells=37)
    for f in names:
        assert np.array_equal(whole[f].to_host_cell_major(), parts[f].to_host_cell_major()), f
