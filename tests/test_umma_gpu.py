"""The tcgen05 tensor-core kernel (strategy "tensor" on volume cells of 21 to 88 nodes in 3D)
through the C ABI (GPU): against the oracle at the f32 tolerance for f32 meshes and split
precision (scaled as tetraloma-testing/src/reference.rs:696-754), on tetrahedra P4-P6, Q3
hexahedra at a non-tensor rule and P4 prisms; facet normals; ranges that are not whole tiles;
more tiles than CTAs; the FP64 recompute of split precision; its bounded waits running out."""

import ctypes

import numpy as np
import pytest
import torch

import gridcl_gb300 as tg
from gridcl_gb300 import meshes
from gridcl_gb300._lib import lib
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

F64, F32 = torch.float64, torch.float32
FACTORS = ("points", "jacobian", "detj", "pinv")
KEYS = {"points": "x", "jacobian": "j", "detj": "detj", "pinv": "k"}
DEVICE_TIMEOUT = 6

CASES = [
    # (cell, n, degree, rule degree)
    ("Tetrahedron", 3, 4, 8),
    ("Tetrahedron", 2, 5, 10),
    ("Tetrahedron", 2, 6, 12),
    ("Hexahedron", 2, 3, 5),
    ("Prism", 2, 4, 6),
]


def run(mesh, cell, pts, precision, names=FACTORS, **kw):
    g = tg.Geometry.from_host(mesh, dtype=F32 if precision == "f32" else F64)
    ps = tg.PointSet(cell, pts, np.ones(len(pts)))
    with tg.with_strategy("tensor"):
        got = tg.geometric_factors_block(g, 0, ps, names, precision="split" if precision == "split" else "native", **kw)
        family = tg.last_kernel_family()
    return g, got, family


def check(g, mesh, cell, degree, pts, got, precision, names=FACTORS):
    absx = g.nodes.double().cpu().numpy() + np.array(g.origin[:3])
    want = orc.eval_block(cell, degree, absx, mesh.blocks[0].cells, pts, factors=[KEYS[f] for f in names])
    nodes = orc.node_ratio(cell, degree)
    s_val = orc.tolerance_scale(cell, degree, "Equispaced", pts, "values") * nodes
    s_der = orc.tolerance_scale(cell, degree, "Equispaced", pts) * nodes
    if precision == "f32":
        r = orc.origin_ratio(absx, np.array(g.origin[:3]), want["j"])
        s_val, s_der = s_val * r, s_der * r
    cond = orc.condition_scale(want["j"], 3, 3)
    scale = {"points": s_val, "jacobian": s_der, "detj": s_der, "pinv": s_der * cond}
    errs = {}
    for f in names:
        errs[f] = orc.rel_err(got[f].to_host_cell_major(), want[KEYS[f]])
        assert errs[f] < orc.TOL_F32 * scale[f], (f, errs[f], orc.TOL_F32 * scale[f])
    return errs


@pytest.mark.parametrize("precision", ["f32", "split"])
@pytest.mark.parametrize("cell,n,degree,rdeg", CASES)
def test_matches_the_oracle(cuda, cell, n, degree, rdeg, precision):
    mesh = meshes.curved_box(cell, n, degree, jitter=0.02)
    pts, _ = tg.refcell.gauss_rule(cell, rdeg)
    pts = pts[np.random.default_rng(1).permutation(len(pts))]  # no tensor structure
    g, got, family = run(mesh, cell, pts, precision)
    assert family == "tensor"
    check(g, mesh, cell, degree, pts, got, precision)


@pytest.mark.parametrize("precision", ["f32", "split"])
def test_many_tiles_match_the_oracle(cuda, precision):
    """6 x 16^3 P4 tetrahedra (384 tiles of 64 cells: more tiles than CTAs, so CTAs run several),
    125 points, against the oracle."""
    mesh = meshes.curved_box("Tetrahedron", 16, 4, jitter=0.02)
    pts, _ = tg.refcell.gauss_rule("Tetrahedron", 8)
    g, got, family = run(mesh, "Tetrahedron", pts, precision)
    assert family == "tensor"
    check(g, mesh, "Tetrahedron", 4, pts, got, precision)


@pytest.mark.parametrize("precision", ["f32", "split"])
def test_fewer_cells_than_a_tile(cuda, precision):
    """6 P5 tetrahedra (one tile of 64 mostly padding, its 27 chunks in work-item groups) against
    the oracle."""
    mesh = meshes.curved_box("Tetrahedron", 1, 5, jitter=0.0)
    pts, _ = tg.refcell.gauss_rule("Tetrahedron", 10)
    g, got, family = run(mesh, "Tetrahedron", pts, precision)
    assert family == "tensor"
    check(g, mesh, "Tetrahedron", 5, pts, got, precision)


def test_ranges_and_facet_normals(cuda):
    """Chunks of 48 cells (tiles of 64 cut short, outputs at 16-cell boundaries) give the fields
    of one launch; facet normals of a facet rule against the oracle."""
    mesh = meshes.curved_box("Tetrahedron", 3, 4, jitter=0.02)  # 162 cells
    pts, _ = tg.refcell.gauss_rule("Tetrahedron", 6)
    g, one, _ = run(mesh, "Tetrahedron", pts, "split")
    _, many, family = run(mesh, "Tetrahedron", pts, "split", max_chunk_cells=48)
    assert family == "tensor"
    for f in FACTORS:
        assert np.array_equal(one[f].to_host_cell_major(), many[f].to_host_cell_major()), f
    ps = tg.facet_point_set("Tetrahedron", 5)
    with tg.with_strategy("tensor"):
        fn = tg.geometric_factors_block(g, 0, ps, ("jacobian", "facet_normals"), precision="split")
        assert tg.last_kernel_family() == "tensor"
    absx = g.nodes.cpu().numpy() + np.array(g.origin[:3])
    want = orc.eval_block("Tetrahedron", 4, absx, mesh.blocks[0].cells, ps.points, factors=("j", "facet_normals"),
                          ref_normals=ps.ref_normals)
    s = orc.tolerance_scale("Tetrahedron", 4, "Equispaced", ps.points) * orc.condition_scale(want["j"], 3, 3)
    assert orc.rel_err(fn["facet_normals"].to_host_cell_major(), want["facet_normals"]) < orc.TOL_F32 * s


def test_split_recomputes_ill_conditioned_points_in_f64(cuda):
    """A condition limit below every point's condition number sends each point through the FP64
    recompute: J, det J and K then match the oracle at the f64 level (1e-12 scaled)."""
    mesh = meshes.curved_box("Tetrahedron", 2, 4, jitter=0.02)
    pts, _ = tg.refcell.gauss_rule("Tetrahedron", 6)
    g, got, family = run(mesh, "Tetrahedron", pts, "split", cond_limit=0.5)
    assert family == "tensor"
    absx = g.nodes.cpu().numpy() + np.array(g.origin[:3])
    want = orc.eval_block("Tetrahedron", 4, absx, mesh.blocks[0].cells, pts, factors=("j", "detj", "k"))
    for f in ("jacobian", "detj", "pinv"):
        # The recompute's f64 results are rounded to the f32 fields.
        assert orc.rel_err(got[f].to_host_cell_major(), want[KEYS[f]]) < 1e-6, f


def test_bounded_waits_run_out(cuda):
    """The tables' test hook leaves the chunk copies unissued: the waits run out, nothing is
    written, the status reports the timeout, and the next launch is correct."""
    mesh = meshes.curved_box("Tetrahedron", 2, 4, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    pts, _ = tg.refcell.gauss_rule("Tetrahedron", 6)
    ps = tg.PointSet("Tetrahedron", pts, np.ones(len(pts)))
    tables = ps.tables(g.blocks[0].element, 3, tg.geometry.SPLIT32)
    with tg.with_strategy("tensor"):
        fields = tg.geometric_factors_block(g, 0, ps, FACTORS, precision="split")
        for f in fields.values():
            f.chunks[0].data.fill_(float("nan"))
        stream = torch.cuda.current_stream().cuda_stream
        assert lib().tlg_tables_set_wait(tables.handle, 16, 0) == 0
        tg.geometric_factors_block(g, 0, ps, FACTORS, precision="split", out=fields)
        assert tg.last_kernel_family() == "tensor"
        assert lib().tlg_tables_device_status(tables.handle, ctypes.c_void_p(stream)) == DEVICE_TIMEOUT
        for f in fields.values():
            assert torch.isnan(f.chunks[0].data).all()
        assert lib().tlg_tables_set_wait(tables.handle, 0, 1) == 0
        tg.geometric_factors_block(g, 0, ps, FACTORS, precision="split", out=fields)
        assert lib().tlg_tables_device_status(tables.handle, ctypes.c_void_p(stream)) == 0
    check(g, mesh, "Tetrahedron", 4, pts, fields, "split")
