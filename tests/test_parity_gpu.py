"""Parity of the CUDA path with the oracle, through the C ABI (GPU).

Tolerances are the reference's (tetraloma-testing/src/lib.rs:127-130): 1e-12 relative in f64
and 1e-5 in f32, scaled as in reference.rs:696-754 by the element's amplification ratio, the
node ratio, the origin ratio R (coordinates are summed relative to the origin) and, for K and
the normals, the condition number of J. The E-vector gather is compared bit for bit.
"""

import numpy as np
import pytest
import torch

import gridcl_gb300 as tg
from gridcl_gb300 import meshes
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

F64, F32 = torch.float64, torch.float32


def oracle_factors(mesh, geom, cell, degree, pts, factors, flags=None, ref_normals=None):
    """The oracle at the node coordinates the grid stores: F(x - origin) widened plus origin."""
    stored = geom.nodes.double().cpu().numpy()
    absx = stored + np.array(geom.origin[: geom.gdim])
    return orc.eval_block(cell, degree, absx, mesh.blocks[0].cells, pts, factors=factors,
                          flags=flags, ref_normals=ref_normals), absx


def scale_for(cell, degree, pts, absx, origin, j, td, gd, conditioned=False):
    s = orc.tolerance_scale(cell, degree, "Equispaced", pts) * orc.node_ratio(cell, degree)
    s *= orc.origin_ratio(absx, np.array(origin[:gd]), j)
    if conditioned:
        s *= orc.condition_scale(j, td, gd)
    return s


CASES = [
    # (cell, n, degree, rule degree)
    ("Tetrahedron", 3, 1, 4),
    ("Tetrahedron", 3, 2, 4),
    ("Tetrahedron", 2, 3, 6),
    ("Hexahedron", 2, 1, 2),
    ("Hexahedron", 2, 2, 4),
    ("Prism", 2, 1, 2),
    ("Prism", 2, 2, 4),
]


@pytest.mark.parametrize("dtype", [F64, F32])
@pytest.mark.parametrize("cell,n,degree,rdeg", CASES)
def test_volume_factors_match_the_oracle(cuda, cell, n, degree, rdeg, dtype):
    mesh = meshes.curved_box(cell, n, degree, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=dtype)
    pts, _ = tg.refcell.gauss_rule(cell, rdeg)
    ps = tg.PointSet(cell, pts, np.ones(len(pts)))
    got = tg.geometric_factors_block(g, 0, ps, ("points", "jacobian", "detj", "pinv"))
    torch.cuda.synchronize()
    want, absx = oracle_factors(mesh, g, cell, degree, pts, ("x", "j", "detj", "k"))
    tol = orc.TOL_F64 if dtype == F64 else orc.TOL_F32
    sj = scale_for(cell, degree, pts, absx, g.origin, want["j"], 3, 3)
    sk = scale_for(cell, degree, pts, absx, g.origin, want["j"], 3, 3, conditioned=True)
    assert orc.rel_err(got["points"].to_host_cell_major(), want["x"]) < tol
    assert orc.rel_err(got["jacobian"].to_host_cell_major(), want["j"]) < tol * sj
    assert orc.rel_err(got["detj"].to_host_cell_major(), want["detj"]) < tol * sj
    assert orc.rel_err(got["pinv"].to_host_cell_major(), want["k"]) < tol * sk


@pytest.mark.parametrize("dtype", [F64, F32])
@pytest.mark.parametrize("degree", [1, 2, 4])
def test_surface_factors_and_normals_match_the_oracle(cuda, degree, dtype):
    mesh = meshes.perturbed_radius(meshes.sphere(1, degree), 0.02)
    flags = (np.arange(mesh.blocks[0].num_cells) % 3 == 0).astype(np.uint32)
    g = tg.Geometry.from_host(mesh, dtype=dtype, flags=[flags])
    pts, _ = tg.refcell.gauss_rule("Triangle", 2 * degree)
    ps = tg.PointSet("Triangle", pts, np.ones(len(pts)))
    got = tg.geometric_factors_block(g, 0, ps, ("points", "jacobian", "detj", "pinv", "normals"))
    torch.cuda.synchronize()
    want, absx = oracle_factors(mesh, g, "Triangle", degree, pts, ("x", "j", "detj", "k", "normals"),
                                flags=flags)
    tol = orc.TOL_F64 if dtype == F64 else orc.TOL_F32
    sj = scale_for("Triangle", degree, pts, absx, g.origin, want["j"], 2, 3)
    sk = scale_for("Triangle", degree, pts, absx, g.origin, want["j"], 2, 3, conditioned=True)
    assert orc.rel_err(got["points"].to_host_cell_major(), want["x"]) < tol
    assert orc.rel_err(got["jacobian"].to_host_cell_major(), want["j"]) < tol * sj
    assert orc.rel_err(got["detj"].to_host_cell_major(), want["detj"]) < tol * sj
    assert orc.rel_err(got["pinv"].to_host_cell_major(), want["k"]) < tol * sk
    n = got["normals"].to_host_cell_major()
    assert orc.rel_err(n, want["normals"]) < tol * sk
    assert np.allclose(np.linalg.norm(n, axis=2), 1.0, atol=10 * tol)


@pytest.mark.parametrize("dtype", [F64, F32])
def test_facet_normals_match_the_oracle(cuda, dtype):
    mesh = meshes.curved_box("Tetrahedron", 2, 2, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=dtype)
    ps = tg.facet_point_set("Tetrahedron", 3)
    got = tg.facet_normals_block(g, 0, ps).to_host_cell_major()
    torch.cuda.synchronize()
    want, absx = oracle_factors(mesh, g, "Tetrahedron", 2, ps.points, ("j", "facet_normals"),
                                ref_normals=ps.ref_normals)
    tol = orc.TOL_F64 if dtype == F64 else orc.TOL_F32
    s = scale_for("Tetrahedron", 2, ps.points, absx, g.origin, want["j"], 3, 3, conditioned=True)
    assert orc.rel_err(got, want["facet_normals"]) < tol * s


@pytest.mark.parametrize("dtype", [F64, F32])
def test_evector_is_bit_exact(cuda, dtype):
    mesh = meshes.curved_box("Tetrahedron", 3, 2, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=dtype)
    cells = mesh.blocks[0].cells
    for max_chunk in (None, 48):
        chunks = g.evector(0, max_chunk_cells=max_chunk)
        stored = g.nodes.cpu().numpy()
        for ch in chunks:
            stride = ch.data.shape[2]
            want = orc.evector(stored, cells, cells.shape[0], 10, 3, ch.first_cell,
                               -(-ch.num_cells // 16) * 16, stride)
            assert np.array_equal(ch.data.cpu().numpy().view(np.uint8), want.view(np.uint8))


def test_single_factor_launches_equal_the_fused_launch(cuda):
    mesh = meshes.curved_box("Tetrahedron", 3, 2, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    pts, _ = tg.refcell.gauss_rule("Tetrahedron", 4)
    ps = tg.PointSet("Tetrahedron", pts, np.ones(len(pts)))
    fused = tg.geometric_factors_block(g, 0, ps, ("points", "jacobian", "detj", "pinv"))
    single = {
        "points": tg.physical_points_block(g, 0, ps),
        "jacobian": tg.jacobians_block(g, 0, ps),
        "detj": tg.detj_block(g, 0, ps),
        "pinv": tg.pseudo_inverse_block(g, 0, ps),
    }
    for k in single:
        assert torch.equal(fused[k].chunks[0].data, single[k].chunks[0].data), k


def test_invariance_to_tile_chunks_and_repeats(cuda):
    """high_order_invariance.rs, quad_field_chunks.rs, determinism.rs: results are identical for
    tile widths 1 and 16, 1 and 7 chunks, and two runs."""
    mesh = meshes.curved_box("Hexahedron", 3, 2, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    pts, _ = tg.refcell.gauss_rule("Hexahedron", 4)
    ps = tg.PointSet("Hexahedron", pts, np.ones(len(pts)))
    base = tg.geometric_factors_block(g, 0, ps, ("points", "detj", "pinv"))
    again = tg.geometric_factors_block(g, 0, ps, ("points", "detj", "pinv"))
    tile1 = tg.geometric_factors_block(g, 0, ps, ("points", "detj", "pinv"), tile=1)
    chunks = tg.geometric_factors_block(g, 0, ps, ("points", "detj", "pinv"), tile=1, max_chunk_cells=4)
    assert len(chunks["detj"].chunks) == 7
    for k in base:
        ref = base[k].to_host_cell_major()
        assert np.array_equal(ref, again[k].to_host_cell_major())
        assert np.array_equal(ref, tile1[k].to_host_cell_major())
        assert np.array_equal(ref, chunks[k].to_host_cell_major())


def test_padding_lanes_repeat_the_last_cell(cuda):
    mesh = meshes.cube_box("Tetrahedron", 1, 1)  # 6 cells: one partial tile
    g = tg.Geometry.from_host(mesh, dtype=F64)
    pts, _ = tg.refcell.gauss_rule("Tetrahedron", 2)
    ps = tg.PointSet("Tetrahedron", pts, np.ones(len(pts)))
    f = tg.detj_block(g, 0, ps)
    raw = f.chunks[0].data.cpu().numpy().reshape(1, len(pts), 1, 16)
    assert np.array_equal(raw[0, :, 0, 6:], np.repeat(raw[0, :, 0, 5:6], 10, axis=1))


def test_clamped_node_indices_read_the_last_node(cuda):
    mesh = meshes.cube_box("Tetrahedron", 1, 1)
    bad = mesh.blocks[0].cells.copy()
    bad[2, 1] = 1000  # past the last node: the kernel reads the last node
    clamped = bad.copy()
    clamped[2, 1] = mesh.num_nodes - 1
    ga = tg.Geometry.from_host(meshes.HostMesh(3, mesh.nodes, [meshes.HostBlock("Tetrahedron", 1, bad)]))
    gb = tg.Geometry.from_host(meshes.HostMesh(3, mesh.nodes, [meshes.HostBlock("Tetrahedron", 1, clamped)]))
    pts, _ = tg.refcell.gauss_rule("Tetrahedron", 2)
    ps = tg.PointSet("Tetrahedron", pts, np.ones(len(pts)))
    a = tg.jacobians_block(ga, 0, ps).to_host_cell_major()
    b = tg.jacobians_block(gb, 0, ps).to_host_cell_major()
    assert np.array_equal(a, b)


def test_empty_block_and_empty_point_set_launch_nothing(cuda):
    mesh = meshes.cube_box("Tetrahedron", 1, 1)
    empty = meshes.HostMesh(3, mesh.nodes, [meshes.HostBlock("Tetrahedron", 1, np.zeros((0, 4), np.uint32))])
    g = tg.Geometry.from_host(empty)
    pts, _ = tg.refcell.gauss_rule("Tetrahedron", 2)
    ps = tg.PointSet("Tetrahedron", pts, np.ones(len(pts)))
    f = tg.detj_block(g, 0, ps)
    assert f.num_cells == 0 and f.to_host_cell_major().shape == (0, len(pts), 1)
    g2 = tg.Geometry.from_host(mesh)
    e = tg.detj_block(g2, 0, tg.PointSet("Tetrahedron", np.zeros((0, 3)), np.zeros(0)))
    assert e.to_host_cell_major().shape == (6, 0, 1)


def test_known_answers_on_the_gpu(cuda):
    """det J = 1/4, J = I/2, K = 2I on 2 x 2 quadrilaterals; unit volume of the cube."""
    m = meshes.square_box("Quadrilateral", 2, 1)
    g = tg.Geometry.from_host(m, dtype=F64)
    pts, w = tg.refcell.gauss_rule("Quadrilateral", 2)
    ps = tg.PointSet("Quadrilateral", pts, w)
    f = tg.geometric_factors_block(g, 0, ps, ("jacobian", "detj", "pinv"))
    assert np.allclose(f["detj"].to_host_cell_major(), 0.25, atol=1e-15)
    assert np.allclose(f["jacobian"].to_host_cell_major(), [0.5, 0, 0, 0.5], atol=1e-15)
    assert np.allclose(f["pinv"].to_host_cell_major(), [2, 0, 0, 2], atol=1e-14)
    for cell in ("Tetrahedron", "Hexahedron", "Prism"):
        m = meshes.cube_box(cell, 3, 1)
        g = tg.Geometry.from_host(m, dtype=F64)
        pts, w = tg.refcell.gauss_rule(cell, 2)
        d = tg.detj_block(g, 0, tg.PointSet(cell, pts, w)).to_host_cell_major()[..., 0]
        assert abs(float((d * w).sum()) - 1.0) < 1e-12


def test_argument_errors(cuda):
    mesh = meshes.cube_box("Tetrahedron", 1, 1)
    g = tg.Geometry.from_host(mesh)
    pts, _ = tg.refcell.gauss_rule("Tetrahedron", 2)
    ps = tg.PointSet("Tetrahedron", pts, np.ones(len(pts)))
    with pytest.raises(tg.GridError) as e:
        tg.normals_block(g, 0, ps)
    assert e.value.kind == "InvalidArgument"
    with pytest.raises(tg.GridError):
        tg.geometric_factors_block(g, 0, ps, ("detj",), tile=3)
    with pytest.raises(tg.GridError) as e:
        tg.Geometry([tg.GeometryBlock(tg.CoordinateElement("Tetrahedron", 2), g.blocks[0].dofmap)],
                    g.nodes, g.origin)
    assert e.value.kind == "LengthMismatch"


@pytest.mark.parametrize("dtype", [F64, F32])
def test_measure_matches_the_oracle_and_the_unit_volume(cuda, dtype):
    """unit_volume.rs: the unit cube's volume to 1e-12 in f64; the sum tree against the oracle's
    f64 sum of the same det J."""
    for cell in ("Tetrahedron", "Hexahedron"):
        mesh = meshes.curved_box(cell, 4, 2, jitter=0.0, amplitude=0.0)
        g = tg.Geometry.from_host(mesh, dtype=dtype)
        pts, w = tg.refcell.gauss_rule(cell, 4)
        ps = tg.PointSet(cell, pts, w)
        vol = tg.measure_block(g, 0, ps)
        tol = 1e-12 if dtype == F64 else 1e-5
        assert abs(vol - 1.0) < tol
    mesh = meshes.curved_box("Tetrahedron", 5, 2, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=dtype)
    pts, w = tg.refcell.gauss_rule("Tetrahedron", 4)
    ps = tg.PointSet("Tetrahedron", pts, w)
    want, _ = oracle_factors(mesh, g, "Tetrahedron", 2, pts, ("detj",))
    ref = orc.measure(want["detj"][..., 0], w)
    got = tg.measure_block(g, 0, ps)
    assert abs(got - ref) / abs(ref) < (1e-13 if dtype == F64 else 1e-5)
    assert got == tg.measure_block(g, 0, ps)  # deterministic
