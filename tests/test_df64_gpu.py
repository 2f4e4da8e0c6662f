"""The double-float evaluation (``precision="df64"``: f64 meshes and fields, arithmetic on the FP32
pipe in pairs of f32) against the oracle, through the C ABI (GPU).

It is held to the reference's f64 tolerance (1e-12 relative, tetraloma-testing/src/lib.rs:130,
scaled as reference.rs:696-754 like the f64 tests), and, on the benchmark's kind of mesh (curved,
jittered), to 3e-13 unscaled: its own error budget is about 2^-48 per operation, and the oracle's
own rounding (f64 sums of absolute coordinates, as the reference computes them) is of the order
of 1e-13 on cells of 1/64 of the box.
"""

import numpy as np
import pytest
import torch

import gridcl_gb300 as tg
from gridcl_gb300 import meshes
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

F64 = torch.float64
FACTORS = ("points", "jacobian", "detj", "pinv")
ORC = {"points": "x", "jacobian": "j", "detj": "detj", "pinv": "k", "normals": "normals"}


def oracle_factors(mesh, geom, cell, degree, pts, factors, flags=None, ref_normals=None, block=0):
    stored = geom.nodes.double().cpu().numpy()
    absx = stored + np.array(geom.origin[: geom.gdim])
    return orc.eval_block(cell, degree, absx, mesh.blocks[block].cells, pts, factors=factors,
                          flags=flags, ref_normals=ref_normals), absx


def scale_for(cell, degree, pts, absx, origin, j, td, gd, conditioned=False):
    s = orc.tolerance_scale(cell, degree, "Equispaced", pts) * orc.node_ratio(cell, degree)
    s *= orc.origin_ratio(absx, np.array(origin[:gd]), j)
    if conditioned:
        s *= orc.condition_scale(j, td, gd)
    return s


VOLUME = [
    ("Tetrahedron", 4, 1, 4),
    ("Tetrahedron", 4, 2, 4),
    ("Tetrahedron", 3, 3, 6),
    ("Hexahedron", 3, 1, 2),
    ("Hexahedron", 3, 2, 4),
    ("Prism", 3, 1, 2),
    ("Prism", 3, 2, 4),
]


@pytest.mark.parametrize("cell,n,degree,rdeg", VOLUME)
def test_volume_factors_match_the_oracle(cuda, cell, n, degree, rdeg):
    mesh = meshes.curved_box(cell, n, degree, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    pts, _ = tg.refcell.gauss_rule(cell, rdeg)
    ps = tg.PointSet(cell, pts, np.ones(len(pts)))
    got = tg.geometric_factors_block(g, 0, ps, FACTORS, precision="df64")
    torch.cuda.synchronize()
    want, absx = oracle_factors(mesh, g, cell, degree, pts, ("x", "j", "detj", "k"))
    sj = scale_for(cell, degree, pts, absx, g.origin, want["j"], 3, 3)
    sk = scale_for(cell, degree, pts, absx, g.origin, want["j"], 3, 3, conditioned=True)
    errs = {f: orc.rel_err(got[f].to_host_cell_major(), want[ORC[f]]) for f in FACTORS}
    assert errs["points"] < orc.TOL_F64
    assert errs["jacobian"] < orc.TOL_F64 * sj
    assert errs["detj"] < orc.TOL_F64 * sj
    assert errs["pinv"] < orc.TOL_F64 * sk
    # The double-float budget on these meshes, unscaled.
    assert max(errs.values()) < 3e-13, errs


@pytest.mark.parametrize("degree", [1, 2, 4])
def test_surface_factors_and_normals_match_the_oracle(cuda, degree):
    mesh = meshes.perturbed_radius(meshes.sphere(1, degree), 0.02)
    flags = (np.arange(mesh.blocks[0].num_cells) % 3 == 0).astype(np.uint32)
    g = tg.Geometry.from_host(mesh, dtype=F64, flags=[flags])
    pts, _ = tg.refcell.gauss_rule("Triangle", 2 * degree)
    ps = tg.PointSet("Triangle", pts, np.ones(len(pts)))
    names = ("points", "jacobian", "detj", "pinv", "normals")
    got = tg.geometric_factors_block(g, 0, ps, names, precision="df64")
    torch.cuda.synchronize()
    want, absx = oracle_factors(mesh, g, "Triangle", degree, pts, ("x", "j", "detj", "k", "normals"), flags=flags)
    sj = scale_for("Triangle", degree, pts, absx, g.origin, want["j"], 2, 3)
    sk = scale_for("Triangle", degree, pts, absx, g.origin, want["j"], 2, 3, conditioned=True)
    assert orc.rel_err(got["points"].to_host_cell_major(), want["x"]) < orc.TOL_F64
    assert orc.rel_err(got["jacobian"].to_host_cell_major(), want["j"]) < orc.TOL_F64 * sj
    assert orc.rel_err(got["detj"].to_host_cell_major(), want["detj"]) < orc.TOL_F64 * sj
    assert orc.rel_err(got["pinv"].to_host_cell_major(), want["k"]) < orc.TOL_F64 * sk
    n = got["normals"].to_host_cell_major()
    assert orc.rel_err(n, want["normals"]) < orc.TOL_F64 * sk
    assert np.allclose(np.linalg.norm(n, axis=2), 1.0, atol=1e-13)


@pytest.mark.parametrize("cell,degree", [("Triangle", 2), ("Quadrilateral", 2), ("Interval", 2)])
def test_planar_and_curve_factors_match_the_oracle(cuda, cell, degree):
    if cell == "Interval":
        # A curve in 3D: P2 intervals along a helix.
        n = 64
        t = np.linspace(0.0, 1.0, 2 * n + 1)
        nodes = np.stack([np.cos(3 * t), np.sin(3 * t), 0.3 * t], axis=1)
        cells = np.stack([2 * np.arange(n), 2 * np.arange(n) + 2, 2 * np.arange(n) + 1], axis=1).astype(np.uint32)
        mesh = meshes.HostMesh(3, nodes, [meshes.HostBlock("Interval", 2, cells)])
        td, gd = 1, 3
        names, onames = FACTORS, ("x", "j", "detj", "k")
    else:
        mesh = meshes.square_box(cell, 4, degree)
        rng = np.random.default_rng(5)
        mesh.nodes = mesh.nodes + 0.01 * rng.uniform(-1, 1, mesh.nodes.shape)
        td, gd = 2, 2
        names, onames = FACTORS, ("x", "j", "detj", "k")
    g = tg.Geometry.from_host(mesh, dtype=F64)
    pts, _ = tg.refcell.gauss_rule(cell, 2 * degree)
    ps = tg.PointSet(cell, pts, np.ones(len(pts)))
    got = tg.geometric_factors_block(g, 0, ps, names, precision="df64")
    torch.cuda.synchronize()
    want, absx = oracle_factors(mesh, g, cell, degree, pts, onames)
    sk = scale_for(cell, degree, pts, absx, g.origin, want["j"], td, gd, conditioned=True)
    for f in names:
        assert orc.rel_err(got[f].to_host_cell_major(), want[ORC[f]]) < orc.TOL_F64 * sk, f


def test_facet_normals_match_the_oracle(cuda):
    mesh = meshes.curved_box("Tetrahedron", 2, 2, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    ps = tg.facet_point_set("Tetrahedron", 3)
    got = tg.geometric_factors_block(g, 0, ps, ("facet_normals",), precision="df64")["facet_normals"]
    torch.cuda.synchronize()
    want, absx = oracle_factors(mesh, g, "Tetrahedron", 2, ps.points, ("j", "facet_normals"),
                                ref_normals=ps.ref_normals)
    s = scale_for("Tetrahedron", 2, ps.points, absx, g.origin, want["j"], 3, 3, conditioned=True)
    assert orc.rel_err(got.to_host_cell_major(), want["facet_normals"]) < orc.TOL_F64 * s


def test_df64_runs_the_double_float_kernel_and_matches_fp64(cuda):
    """The policy runs the double-float kernel (recorded as DIRECT); its fields are within the
    double-float budget of the plain FP64 kernel's, which ran on the same tables' f64 sections
    under the loops strategy."""
    mesh = meshes.curved_box("Tetrahedron", 4, 2, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    pts, _ = tg.refcell.collapsed_rule("Tetrahedron", (4, 3, 2))
    ps = tg.PointSet("Tetrahedron", pts, np.ones(len(pts)))
    got = tg.geometric_factors_block(g, 0, ps, FACTORS, precision="df64")
    assert tg.last_kernel_family() == "direct"
    with tg.with_strategy("loops"):
        f64 = tg.geometric_factors_block(g, 0, ps, FACTORS, precision="df64")
        assert tg.last_kernel_family() == "loops"
        plain = tg.geometric_factors_block(g, 0, ps, FACTORS)
    for f in FACTORS:
        assert torch.equal(f64[f].chunks[0].data, plain[f].chunks[0].data), f
        a, b = got[f].chunks[0].data, plain[f].chunks[0].data
        assert float((a - b).abs().max() / b.abs().max()) < 3e-13, f


def test_padding_lanes_and_chunks(cuda):
    """Ranges that are not whole tiles and several chunks give the fields of one launch."""
    mesh = meshes.curved_box("Tetrahedron", 3, 2, jitter=0.02)  # 162 cells
    g = tg.Geometry.from_host(mesh, dtype=F64)
    pts, _ = tg.refcell.gauss_rule("Tetrahedron", 4)
    ps = tg.PointSet("Tetrahedron", pts, np.ones(len(pts)))
    one = tg.geometric_factors_block(g, 0, ps, FACTORS, precision="df64")
    many = tg.geometric_factors_block(g, 0, ps, FACTORS, precision="df64", max_chunk_cells=48)
    for f in FACTORS:
        assert np.array_equal(one[f].to_host_cell_major(), many[f].to_host_cell_major()), f
