"""Pull-back (Newton physical -> reference) through the C ABI against the oracle and known
answers (GPU): Gauss points come back from their images in f64 and f32, points of every cell
type and of a surface match the oracle's iterates, points outside their cell stay in the clamp
box without converging, and the iteration count semantics (pull_back.rs:27-60)."""

import numpy as np
import pytest
import torch

import gridcl_gb300 as tg
from gridcl_gb300 import meshes
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

F64, F32 = torch.float64, torch.float32


def quad_or_tri(cell, n, degree):
    m = meshes.square_box(cell, n, degree)
    m.nodes = meshes.jitter_interior(m.nodes, m.nodes, 0.02 / n, 2026)
    return m


CELLS = [
    ("Tetrahedron", 1), ("Tetrahedron", 2), ("Tetrahedron", 3), ("Hexahedron", 1), ("Hexahedron", 2),
    ("Prism", 1), ("Prism", 2), ("Pyramid", 2), ("Pyramid", 3), ("Triangle", 2), ("Quadrilateral", 3),
]


def inside(cell, xi, eps=1e-9):
    """Whether reference points `[..., td]` lie in the reference cell (up to eps)."""
    x = [xi[..., d] for d in range(xi.shape[-1])]
    lo = np.all(xi >= -eps, axis=-1)
    if cell in ("Interval", "Quadrilateral", "Hexahedron"):
        return lo & np.all(xi <= 1 + eps, axis=-1)
    if cell in ("Triangle", "Tetrahedron"):
        return lo & (xi.sum(axis=-1) <= 1 + eps)
    if cell == "Prism":
        return lo & (x[0] + x[1] <= 1 + eps) & (x[2] <= 1 + eps)
    if cell == "Pyramid":
        return lo & (x[0] + x[2] <= 1 + eps) & (x[1] + x[2] <= 1 + eps)
    raise ValueError(cell)


def mesh_for(cell, degree, n=2):
    if cell in ("Triangle", "Quadrilateral"):
        return quad_or_tri(cell, n, degree)
    return meshes.curved_box(cell, n, degree, jitter=0.02)


def field_of(values, tile, dtype):
    """A tiled QuadField from cell-major values [cell][q][len]."""
    nc, nq, ln = values.shape
    nt = -(-nc // tile)
    padded = np.zeros((nt * tile, nq, ln))
    padded[:nc] = values
    padded[nc:] = values[-1] if nc else 0
    data = padded.reshape(nt, tile, nq, ln).transpose(0, 2, 3, 1).ravel()
    ch = tg.geometry.QuadChunk(0, nc, torch.from_numpy(data).to(dtype).cuda())
    return tg.QuadField([ch], nc, nq, ln, tile)


@pytest.mark.parametrize("dtype", [F64, F32])
@pytest.mark.parametrize("cell,degree", CELLS)
def test_gauss_points_come_back(cuda, cell, degree, dtype):
    mesh = mesh_for(cell, degree)
    g = tg.Geometry.from_host(mesh, dtype=dtype)
    pts, _ = tg.refcell.gauss_rule(cell, 2 * degree)
    ps = tg.PointSet(cell, pts, np.ones(len(pts)))
    x = tg.physical_points_block(g, 0, ps)
    xi, step = tg.pull_back_block(g, 0, x)
    got = xi.to_host_cell_major()
    tol = 1e-13 if dtype == F64 else 1e-5
    conv = step.to_host_cell_major()[..., 0] <= tol
    # Newton from the centroid can leave strongly curved cells for points near a vertex (the
    # reference's algorithm, and the oracle's, flag those as not converged), and near the apex of
    # a curved P3 pyramid it can converge to the map's second preimage beyond the apex (the
    # oracle finds the same one); every point converged inside the reference cell is the Gauss
    # point.
    conv_in = conv & inside(cell, got, 1e-6)
    assert conv_in.mean() > 0.99
    assert np.abs(got - pts[None])[conv_in].max() < (1e-11 if dtype == F64 else 2e-5)


@pytest.mark.parametrize("cell,degree", CELLS)
def test_pull_back_matches_the_oracle(cuda, cell, degree):
    """Seeded reference points inside and beyond the cells, mapped forward by the oracle: the
    converged points agree to 1e-11 with the oracle's, and so do the convergence flags away from
    the threshold."""
    mesh = mesh_for(cell, degree)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    td = tg.refcell.tdim(cell)
    rng = np.random.default_rng(5)
    ref = rng.uniform(-0.3, 1.3, size=(12, td))
    absx = g.nodes.cpu().numpy() + np.array(g.origin[: g.gdim])
    cells = mesh.blocks[0].cells
    x = orc.eval_block(cell, degree, absx, cells, ref, factors=("x",))["x"]
    xi, step = tg.pull_back_block(g, 0, field_of(x, 16, F64))
    want_xi, want_step = orc.pull_back(cell, degree, absx, cells, x)
    got_xi, got_step = xi.to_host_cell_major(), step.to_host_cell_major()[..., 0]
    conv = (got_step <= 1e-13) & (want_step <= 1e-13)
    assert conv.any()
    assert np.abs(got_xi[conv] - want_xi[conv]).max() < 1e-11
    clear = (np.minimum(got_step, want_step) > 1e-11) | (np.maximum(got_step, want_step) <= 1e-13)
    assert np.array_equal((got_step <= 1e-13)[clear], (want_step <= 1e-13)[clear])
    assert np.all(got_xi >= float(np.float32(-0.1))) and np.all(got_xi <= float(np.float32(1.1)))


def test_surface_pull_back(cuda):
    """Gauss-Newton on a curved P2 triangle surface: the images of Gauss points come back."""
    mesh = meshes.perturbed_radius(meshes.sphere(1, 2), 0.02)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    pts, _ = tg.refcell.gauss_rule("Triangle", 4)
    x = tg.physical_points_block(g, 0, tg.PointSet("Triangle", pts, np.ones(len(pts))))
    xi, step = tg.pull_back_block(g, 0, x)
    assert np.abs(xi.to_host_cell_major() - pts[None]).max() < 1e-11
    assert step.to_host_cell_major().max() <= 1e-13


def test_iteration_semantics(cuda):
    """No iterations leave the centroid and the largest finite step; an affine cell converges
    after one step (the second step is zero); a tolerance of 1e-3 freezes earlier."""
    mesh = meshes.cube_box("Tetrahedron", 2, 1)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    pts, _ = tg.refcell.gauss_rule("Tetrahedron", 2)
    x = tg.physical_points_block(g, 0, tg.PointSet("Tetrahedron", pts, np.ones(len(pts))))
    xi0, step0 = tg.pull_back_block(g, 0, x, max_iterations=0)
    assert np.all(xi0.to_host_cell_major() == 0.25)
    assert np.all(step0.to_host_cell_major() == np.finfo(np.float64).max)
    xi2, step2 = tg.pull_back_block(g, 0, x, max_iterations=2)
    assert np.abs(xi2.to_host_cell_major() - pts[None]).max() < 1e-14
    assert step2.to_host_cell_major().max() <= 1e-13
    mesh = meshes.curved_box("Hexahedron", 2, 2, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    pts, _ = tg.refcell.gauss_rule("Hexahedron", 4)
    x = tg.physical_points_block(g, 0, tg.PointSet("Hexahedron", pts, np.ones(len(pts))))
    _, loose = tg.pull_back_block(g, 0, x, tolerance=1e-3)
    _, tight = tg.pull_back_block(g, 0, x)
    loose, tight = loose.to_host_cell_major(), tight.to_host_cell_major()
    assert loose.max() <= 1e-3 and np.all(loose >= tight) and loose.max() > 1e3 * tight.max()


def test_pull_back_errors(cuda):
    mesh = meshes.curved_box("Tetrahedron", 1, 2, jitter=0.0)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    pts, _ = tg.refcell.gauss_rule("Tetrahedron", 2)
    x = tg.physical_points_block(g, 0, tg.PointSet("Tetrahedron", pts, np.ones(len(pts))))
    with pytest.raises(tg.GridError):
        tg.pull_back_block(g, 0, x, max_iterations=-1)
    wrong = tg.QuadField(x.chunks, x.num_cells + 1, x.num_points, x.length, x.tile)
    with pytest.raises(tg.GridError):
        tg.pull_back_block(g, 0, wrong)


@pytest.mark.parametrize("cell,degree", CELLS)
def test_split_pull_back_matches_f64(cuda, cell, degree):
    """Mixed precision (FP32 iteration, FP64-residual refinement): on Gauss points and on seeded
    points inside and beyond the cells, the points that converge in f64 converge here too, to
    the same reference point within 1e-12, with steps of at most the f64 tolerance."""
    mesh = mesh_for(cell, degree)
    g = tg.Geometry.from_host(mesh, dtype=F64)
    td = tg.refcell.tdim(cell)
    pts, _ = tg.refcell.gauss_rule(cell, 2 * degree)
    ref = np.concatenate([pts, np.random.default_rng(8).uniform(-0.3, 1.3, size=(8, td))])
    absx = g.nodes.cpu().numpy() + np.array(g.origin[: g.gdim])
    x = orc.eval_block(cell, degree, absx, mesh.blocks[0].cells, ref, factors=("x",))["x"]
    field = field_of(x, 16, F64)
    xi64, st64 = tg.pull_back_block(g, 0, field)
    xis, sts = tg.pull_back_block(g, 0, field, precision="split")
    xi64, st64 = xi64.to_host_cell_major(), st64.to_host_cell_major()[..., 0]
    xis, sts = xis.to_host_cell_major(), sts.to_host_cell_major()[..., 0]
    # Both converged, the f64 one inside the reference cell (near a curved P3 pyramid's apex the
    # iteration can reach the map's second preimage beyond it, and the two precisions need not
    # reach the same one).
    both = (st64 <= 1e-13) & (sts <= 1e-13) & inside(cell, xi64) & inside(cell, xis)
    assert both.any()
    assert np.abs(xis[both] - xi64[both]).max() < 1e-12
    # Points converged in f64 well inside the box converge in mixed precision too.
    in_box = (st64 <= 1e-13) & np.all((xi64 > 0.0) & (xi64 < 1.0), axis=2)
    assert np.all(sts[in_box] <= 1e-13)


def test_split_pull_back_needs_f64(cuda):
    mesh = meshes.curved_box("Tetrahedron", 1, 2, jitter=0.0)
    g = tg.Geometry.from_host(mesh, dtype=F32)
    pts, _ = tg.refcell.gauss_rule("Tetrahedron", 2)
    x = tg.physical_points_block(g, 0, tg.PointSet("Tetrahedron", pts, np.ones(len(pts))))
    with pytest.raises(tg.GridError):
        tg.pull_back_block(g, 0, x, precision="split")
