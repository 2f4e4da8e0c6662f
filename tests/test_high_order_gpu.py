"""Elements without compiled kernels, and tabulations beyond the shared-memory budget: the loops
kernels (tables staged, or read from global memory) in f64 and f32, and the split-precision
loops kernel, against the oracle (GPU).

Tolerances as in the parity tests (the reference's 1e-12 / 1e-5 scaled by the element's
amplification, node and origin ratios and, for K and normals, the condition of J); split
precision within the reference's f32 tolerance scaled the same way (the condition capped at
the FP64 recompute limit)."""

import numpy as np
import pytest
import torch

import gridcl_gb300 as tg
from gridcl_gb300 import meshes
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

F64, F32 = torch.float64, torch.float32
SPLIT_TOL = {"points": 2e-7, "jacobian": 2e-6, "detj": 4e-6, "pinv": 4e-6, "normals": 4e-6}
KEYS = {"points": "x", "jacobian": "j", "detj": "detj", "pinv": "k", "normals": "normals"}

CASES = [
    # (cell, n, degree, rule degree): K, points, f64 table bytes
    ("Hexahedron", 2, 4, 8),   # 125 nodes, 125 points, 500 KB: global tables
    ("Tetrahedron", 2, 5, 8),  # 56 nodes, 125 points, 224 KB: global tables; no paired kernel
    ("Tetrahedron", 2, 4, 6),  # 35 nodes, 64 points: staged loops kernels
    ("Prism", 2, 3, 6),        # 40 nodes, 64 points: staged loops kernels
    ("Tetrahedron", 1, 8, 16), # 165 nodes, 729 points, 3.8 MB: global tables
    ("Hexahedron", 1, 6, 12),  # 343 nodes, 343 points, 3.8 MB: global tables
]


def box(cell, n, degree):
    return meshes.curved_box(cell, n, degree, jitter=0.02)


def oracle(mesh, g, cell, degree, pts, factors, flags=None):
    absx = g.nodes.double().cpu().numpy() + np.array(g.origin[: g.gdim])
    return orc.eval_block(cell, degree, absx, mesh.blocks[0].cells, pts, factors=factors, flags=flags), absx


def scale_for(cell, degree, pts, absx, origin, j, td, gd, conditioned=False):
    s = orc.tolerance_scale(cell, degree, "Equispaced", pts) * orc.node_ratio(cell, degree)
    s *= orc.origin_ratio(absx, np.array(origin[:gd]), j)
    if conditioned:
        s *= orc.condition_scale(j, td, gd)
    return s


@pytest.mark.parametrize("dtype", [F64, F32])
@pytest.mark.parametrize("cell,n,degree,rdeg", CASES)
def test_high_order_factors_match_the_oracle(cuda, cell, n, degree, rdeg, dtype):
    mesh = box(cell, n, degree)
    g = tg.Geometry.from_host(mesh, dtype=dtype)
    pts, _ = tg.refcell.gauss_rule(cell, rdeg)
    ps = tg.PointSet(cell, pts, np.ones(len(pts)))
    got = tg.geometric_factors_block(g, 0, ps, ("points", "jacobian", "detj", "pinv"))
    want, absx = oracle(mesh, g, cell, degree, pts, ("x", "j", "detj", "k"))
    tol = orc.TOL_F64 if dtype == F64 else orc.TOL_F32
    sj = scale_for(cell, degree, pts, absx, g.origin, want["j"], 3, 3)
    sk = scale_for(cell, degree, pts, absx, g.origin, want["j"], 3, 3, conditioned=True)
    assert orc.rel_err(got["points"].to_host_cell_major(), want["x"]) < tol * sj
    assert orc.rel_err(got["jacobian"].to_host_cell_major(), want["j"]) < tol * sj
    assert orc.rel_err(got["detj"].to_host_cell_major(), want["detj"]) < tol * sj
    assert orc.rel_err(got["pinv"].to_host_cell_major(), want["k"]) < tol * sk


@pytest.mark.parametrize("cell,n,degree,rdeg", CASES)
def test_high_order_split_matches_the_oracle(cuda, cell, n, degree, rdeg):
    mesh = box(cell, n, degree)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    pts, _ = tg.refcell.gauss_rule(cell, rdeg)
    ps = tg.PointSet(cell, pts, np.ones(len(pts)))
    count = torch.zeros(1, dtype=torch.int64, device="cuda")
    got = tg.geometric_factors_block(g, 0, ps, ("points", "jacobian", "detj", "pinv"),
                                     precision="split", recomputed=count)
    want, _ = oracle(mesh, g, cell, degree, pts, ("x", "j", "detj", "k"))
    # The reference's own f32 tolerance (1e-5) with its scales: split precision is at least as
    # accurate as the reference evaluated in f32 (K with the condition number of J, capped at the
    # FP64 recompute limit).
    nodes = orc.node_ratio(cell, degree)
    scale = {"points": orc.tolerance_scale(cell, degree, "Equispaced", pts, "values") * nodes,
             "jacobian": orc.tolerance_scale(cell, degree, "Equispaced", pts) * nodes}
    scale["detj"] = scale["jacobian"]
    scale["pinv"] = scale["jacobian"] * min(orc.condition_scale(want["j"], 3, 3), 256.0)
    for f, field in got.items():
        assert field.chunks[0].data.dtype == F32
        err = orc.rel_err(field.to_host_cell_major(), want[KEYS[f]])
        assert err < orc.TOL_F32 * scale[f], (f, err, scale[f])
    assert int(count.item()) <= len(pts) * mesh.blocks[0].num_cells // 100


def test_high_order_split_surface_with_normals(cuda):
    """P5 triangles on a perturbed sphere (no paired kernel): area element, K and signed unit
    normals in split precision."""
    mesh = meshes.perturbed_radius(meshes.sphere(1, 5), 0.02)
    flags = (np.arange(mesh.blocks[0].num_cells) % 3 == 0).astype(np.uint32)
    g = tg.Geometry.from_host(mesh, dtype=F64, flags=[flags])
    pts, _ = tg.refcell.gauss_rule("Triangle", 10)
    ps = tg.PointSet("Triangle", pts, np.ones(len(pts)))
    names = ("points", "jacobian", "detj", "pinv", "normals")
    got = tg.geometric_factors_block(g, 0, ps, names, precision="split")
    want, absx = oracle(mesh, g, "Triangle", 5, pts, ("x", "j", "detj", "k", "normals"), flags=flags)
    scale = orc.tolerance_scale("Triangle", 5, "Equispaced", pts) * orc.condition_scale(want["j"], 2, 3)
    for f in names:
        err = orc.rel_err(got[f].to_host_cell_major(), want[KEYS[f]])
        assert err < SPLIT_TOL[f] * scale, (f, err, scale)
    n = got["normals"].to_host_cell_major()
    assert np.allclose(np.linalg.norm(n, axis=2), 1.0, atol=1e-5)


def test_split_loops_and_paired_kernels_agree(cuda):
    """The split loops kernel runs the paired kernel's arithmetic one point at a time: on an
    element that has both (P2 tetrahedra), a tabulation too large to stage sends the same mesh
    to the loops kernel, whose fields equal the paired kernel's bit for bit."""
    mesh = box("Tetrahedron", 3, 2)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    small, _ = tg.refcell.gauss_rule("Tetrahedron", 4)
    # 27 copies of the 27 points: 729 points, 729 x 10 x (4 f32 + 3 f32 pairs + 3 f64) bytes.
    big = np.tile(small, (27, 1))
    names = ("points", "jacobian", "detj", "pinv")
    a = tg.geometric_factors_block(g, 0, tg.PointSet("Tetrahedron", small, np.ones(len(small))), names,
                                   precision="split")
    b = tg.geometric_factors_block(g, 0, tg.PointSet("Tetrahedron", big, np.ones(len(big))), names,
                                   precision="split")
    nq = len(small)
    for f in names:
        fa = a[f].to_host_cell_major()
        fb = b[f].to_host_cell_major()
        for r in range(3):
            assert np.array_equal(fb[:, r * nq:(r + 1) * nq], fa), (f, r)
