"""Pyramids through the C ABI (GPU): the rational Lagrange space of degrees 1-3 (the reference's
pyramid tests stop at p = 3, tetraloma-testing/src/reference.rs:497-500) against the oracle, which
builds the Lagrange functions from an exact inverse of its own rationomial Vandermonde matrix.

Covered as for the other cells: every factor in f64, f32, split precision and double-float on
curved, jittered pyramid boxes at the reference's tolerances (scaled as reference.rs:696-754);
each evaluation strategy; facet normals of the mixed triangle/quadrilateral facets; the unit
volume of affine pyramid boxes and of the mixed tetrahedron/hexahedron/pyramid and
hexahedron/prism/pyramid boxes through batched graphs (tetraloma/tests/unit_volume.rs: 1e-12 in
f64); the adjoint; the pull-back on the affine pyramid box of tetraloma/tests/pull_back.rs:111-114.
"""

import numpy as np
import pytest
import torch

import gridcl_gb300 as tg
from gridcl_gb300 import meshes
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

F64, F32 = torch.float64, torch.float32
FACTORS = ("points", "jacobian", "detj", "pinv")
KEYS = {"points": "x", "jacobian": "j", "detj": "detj", "pinv": "k"}
CASES = [(3, 1, 3), (2, 2, 6), (2, 3, 9)]  # (n, degree, rule degree)


def scales(degree, pts, absx, origin, j, f32):
    nodes = orc.node_ratio("Pyramid", degree)
    s_val = orc.tolerance_scale("Pyramid", degree, "Equispaced", pts, "values") * nodes
    s_der = orc.tolerance_scale("Pyramid", degree, "Equispaced", pts) * nodes
    if f32:  # coordinates rounded relative to the origin
        r = orc.origin_ratio(absx, np.array(origin[:3]), j)
        s_val, s_der = s_val * r, s_der * r
    cond = orc.condition_scale(j, 3, 3)
    return {"points": s_val, "jacobian": s_der, "detj": s_der, "pinv": s_der * cond}


def check_against_oracle(g, mesh, degree, pts, got, precision, block=0):
    absx = g.nodes.double().cpu().numpy() + np.array(g.origin[:3])
    want = orc.eval_block("Pyramid", degree, absx, mesh.blocks[block].cells, pts, factors=("x", "j", "detj", "k"))
    base = orc.TOL_F64 if precision in ("f64", "df64") else orc.TOL_F32
    sc = scales(degree, pts, absx, g.origin, want["j"], precision == "f32")
    for f in got:
        err = orc.rel_err(got[f].to_host_cell_major(), want[KEYS[f]])
        assert err < base * sc[f], (f, err, base * sc[f])


@pytest.mark.parametrize("precision", ["f64", "f32", "split", "df64"])
@pytest.mark.parametrize("n,degree,rdeg", CASES)
def test_factors_match_the_oracle(cuda, n, degree, rdeg, precision):
    mesh = meshes.curved_box("Pyramid", n, degree, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=F32 if precision == "f32" else F64)
    pts, _ = tg.refcell.gauss_rule("Pyramid", rdeg)
    ps = tg.PointSet("Pyramid", pts, np.ones(len(pts)))
    prec = {"f64": "native", "f32": "native", "split": "split", "df64": "df64"}[precision]
    got = tg.geometric_factors_block(g, 0, ps, FACTORS, precision=prec)
    check_against_oracle(g, mesh, degree, pts, got, precision)
    if precision == "df64" and degree < 3:  # the P3 rule's tables exceed the staging budget
        assert tg.last_kernel_family() == "direct"  # the double-float kernel


@pytest.mark.parametrize("precision", ["f64", "split"])
@pytest.mark.parametrize("strategy", ["direct", "loops", "shared", "cooperative", "tensor", "sumfact"])
def test_every_strategy(cuda, strategy, precision):
    """Each strategy (sum factorisation has no pyramid form and runs the loops kernel) against the
    oracle on P2 pyramids."""
    mesh = meshes.curved_box("Pyramid", 2, 2, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    pts, _ = tg.refcell.gauss_rule("Pyramid", 6)
    ps = tg.PointSet("Pyramid", pts, np.ones(len(pts)))
    with tg.with_strategy(strategy):
        got = tg.geometric_factors_block(g, 0, ps, FACTORS, precision="split" if precision == "split" else "native")
        family = tg.last_kernel_family()
    if strategy in ("loops", "cooperative"):
        assert family == strategy
    elif strategy == "sumfact":
        assert family == "loops"
    elif strategy == "tensor":
        assert family == ("tensor" if precision == "split" else "loops")
    check_against_oracle(g, mesh, 2, pts, got, precision)


@pytest.mark.parametrize("precision", ["native", "df64"])
def test_facet_normals_match_the_oracle(cuda, precision):
    """The base (a quadrilateral) and the four triangles, each with its reference normal."""
    mesh = meshes.curved_box("Pyramid", 2, 2, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    ps = tg.facet_point_set("Pyramid", 3)
    got = tg.geometric_factors_block(g, 0, ps, ("facet_normals",), precision=precision)["facet_normals"]
    absx = g.nodes.cpu().numpy() + np.array(g.origin[:3])
    want = orc.eval_block("Pyramid", 2, absx, mesh.blocks[0].cells, ps.points, factors=("j", "facet_normals"),
                          ref_normals=ps.ref_normals)
    s = orc.tolerance_scale("Pyramid", 2, "Equispaced", ps.points) * orc.condition_scale(want["j"], 3, 3)
    assert orc.rel_err(got.to_host_cell_major(), want["facet_normals"]) < orc.TOL_F64 * s


@pytest.mark.parametrize("dtype", [F64, F32])
def test_unit_volume(cuda, dtype):
    """Affine pyramid boxes and the two mixed boxes (pyramid nodes affine, the others sin-mapped
    as far as the boundary allows: here all affine), p = 1..3, rule degree 3p: volume 1."""
    tol = 1e-12 if dtype == F64 else 1e-5
    for p in (1, 2, 3):
        for mesh in (meshes.cube_box("Pyramid", 2, p), meshes.mixed_box(2, p), meshes.hex_prism_pyramid_box(3, p)):
            g = tg.Geometry.from_host(mesh, dtype=dtype)
            vol = 0.0
            for b, blk in enumerate(mesh.blocks):
                ps = tg.PointSet(blk.cell, *tg.refcell.gauss_rule(blk.cell, 3 * p))
                vol += tg.measure_block(g, b, ps)
            assert abs(vol - 1.0) <= tol, (p, [b.cell for b in mesh.blocks], vol)


@pytest.mark.parametrize("precision", ["native", "df64", "split"])
def test_mixed_box_batches(cuda, precision):
    """The mixed tetrahedron/hexahedron/pyramid box, curved and jittered, P2, in one batched graph:
    every block against the oracle."""
    mesh = meshes.mixed_box(3, 2)
    x = meshes.sin_map(mesh.nodes, 0.05)
    mesh.nodes = meshes.jitter_interior(x, mesh.nodes, 0.02 / 3, 2026)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    rule = tg.QuadRule([tg.PointSet(c, *tg.refcell.gauss_rule(c, 6)) for c in ("Tetrahedron", "Hexahedron", "Pyramid")])
    batch = tg.Batch(g, rule, factors=FACTORS, precision=precision)
    batch.launch()
    torch.cuda.synchronize()
    absx = g.nodes.cpu().numpy() + np.array(g.origin[:3])
    for b, blk in enumerate(mesh.blocks):
        pts = rule.get(blk.cell).points
        want = orc.eval_block(blk.cell, 2, absx, blk.cells, pts, factors=("x", "j", "detj", "k"))
        if precision == "split":
            tol = dict.fromkeys(FACTORS, 5e-6)
        else:
            s = orc.tolerance_scale(blk.cell, 2, "Equispaced", pts) * orc.node_ratio(blk.cell, 2)
            s *= orc.origin_ratio(absx, np.array(g.origin[:3]), want["j"])
            sk = s * orc.condition_scale(want["j"], 3, 3)
            tol = {"points": orc.TOL_F64, "jacobian": orc.TOL_F64 * s, "detj": orc.TOL_F64 * s,
                   "pinv": orc.TOL_F64 * sk}
        for f in FACTORS:
            err = orc.rel_err(batch.fields[b][f].to_host_cell_major(), want[KEYS[f]])
            assert err < tol[f], (blk.cell, f, err)


def cotangents(rng, ncells, nq, dtype):
    out, host = {}, {}
    for name, length in (("points", 3), ("detj", 1), ("pinv", 9)):
        f = tg.QuadField.uninit(ncells, nq, length, 16, dtype)
        f.chunks[0].data.copy_(torch.from_numpy(rng.standard_normal(f.chunks[0].data.numel())).to(dtype))
        out[name] = f
        host[name] = f.to_host_cell_major().astype(np.float64)
    return out, host


@pytest.mark.parametrize("n,degree,rdeg", CASES)
def test_adjoint_matches_the_oracle(cuda, n, degree, rdeg):
    mesh = meshes.curved_box("Pyramid", n, degree, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    pts, _ = tg.refcell.gauss_rule("Pyramid", rdeg)
    ps = tg.PointSet("Pyramid", pts, np.ones(len(pts)))
    nc = mesh.blocks[0].num_cells
    ct, host = cotangents(np.random.default_rng(7), nc, len(pts), F64)
    absx = g.nodes.cpu().numpy() + np.array(g.origin[:3])
    want = orc.vjp("Pyramid", degree, absx, mesh.blocks[0].cells, pts, host["points"], host["detj"][..., 0],
                   host["pinv"])
    got, _ = tg.vjp_block(g, 0, ps, ct)
    assert orc.rel_err(got.cpu().numpy(), want) < 1e-11
    ct32 = {k: tg.QuadField([tg.geometry.QuadChunk(0, nc, v.chunks[0].data.float())], nc, len(pts), v.length, 16)
            for k, v in ct.items()}
    h32 = {k: v.to_host_cell_major().astype(np.float64) for k, v in ct32.items()}
    want32 = orc.vjp("Pyramid", degree, absx, mesh.blocks[0].cells, pts, h32["points"], h32["detj"][..., 0],
                     h32["pinv"])
    got32, _ = tg.vjp_block(g, 0, ps, ct32, precision="split")
    assert orc.rel_err(got32.cpu().numpy(), want32) < 2e-5


def affine(x):
    """The affine map of the reference's pull-back test."""
    return np.column_stack([x[:, 0] + 0.3 * x[:, 1] + 1.5, x[:, 1] - 0.25, 1.2 * x[:, 2] + 0.7])


@pytest.mark.parametrize("dtype", [F64, F32])
@pytest.mark.parametrize("degree", [1, 2, 3])
def test_pull_back_recovers_gauss_points(cuda, degree, dtype):
    mesh = meshes.cube_box("Pyramid", 2, degree)
    mesh.nodes = affine(mesh.nodes)
    g = tg.Geometry.from_host(mesh, dtype=dtype)
    pts, _ = tg.refcell.gauss_rule("Pyramid", 2 * degree)
    x = tg.physical_points_block(g, 0, tg.PointSet("Pyramid", pts, np.ones(len(pts))))
    xi, step = tg.pull_back_block(g, 0, x)
    tol = 1e-13 if dtype == F64 else 1e-5
    assert step.to_host_cell_major().max() <= tol
    assert np.abs(xi.to_host_cell_major() - pts[None]).max() < (1e-12 if dtype == F64 else 2e-5)


def test_pull_back_matches_the_oracle_on_curved_pyramids(cuda):
    """Seeded reference points inside and beyond curved P2 pyramids, mapped forward by the
    oracle: the converged points agree with the oracle's iterates to 1e-11."""
    mesh = meshes.curved_box("Pyramid", 2, 2, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    rng = np.random.default_rng(5)
    ref = rng.uniform(-0.2, 1.0, size=(12, 3)) * np.array([1.0, 1.0, 0.8])
    absx = g.nodes.cpu().numpy() + np.array(g.origin[:3])
    cells = mesh.blocks[0].cells
    x = orc.eval_block("Pyramid", 2, absx, cells, ref, factors=("x",))["x"]
    nc, nq = x.shape[:2]
    data = np.zeros((-(-nc // 16) * 16, nq, 3))
    data[:nc] = x
    data[nc:] = x[-1]
    t = data.reshape(-1, 16, nq, 3).transpose(0, 2, 3, 1).ravel()
    field = tg.QuadField([tg.geometry.QuadChunk(0, nc, torch.from_numpy(t).cuda())], nc, nq, 3, 16)
    xi, step = tg.pull_back_block(g, 0, field)
    want_xi, want_step = orc.pull_back("Pyramid", 2, absx, cells, x)
    got_xi, got_step = xi.to_host_cell_major(), step.to_host_cell_major()[..., 0]
    conv = (got_step <= 1e-13) & (want_step <= 1e-13)
    assert conv.mean() > 0.5
    assert np.abs(got_xi[conv] - want_xi[conv]).max() < 1e-11
