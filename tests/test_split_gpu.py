"""Split precision (f64 mesh, FP32 arithmetic on cell-shifted coordinates, f32 fields, FP64
recompute at flagged points) against the f64 oracle, with the error stated per output (GPU)."""

import numpy as np
import pytest
import torch

import gridcl_gb300 as tg
from gridcl_gb300 import meshes
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

# Per-output relative error bounds of the split path against the f64 oracle (max abs error
# over the block / max abs value, reference.rs:805-817), for well-conditioned curved cells.
SPLIT_TOL = {"points": 2e-7, "jacobian": 2e-6, "detj": 4e-6, "pinv": 4e-6, "normals": 4e-6}


def oracle(mesh, g, cell, degree, pts, factors, flags=None):
    absx = g.nodes.cpu().numpy() + np.array(g.origin[: g.gdim])
    return orc.eval_block(cell, degree, absx, mesh.blocks[0].cells, pts, factors=factors, flags=flags)


KEYS = {"points": "x", "jacobian": "j", "detj": "detj", "pinv": "k", "normals": "normals"}


@pytest.mark.parametrize("cell,n,degree,rdeg", [("Tetrahedron", 4, 2, 4), ("Tetrahedron", 3, 1, 4),
                                                ("Hexahedron", 3, 2, 4), ("Prism", 3, 2, 4),
                                                ("Tetrahedron", 2, 3, 6)])
def test_split_volume_errors_are_stated_per_output(cuda, cell, n, degree, rdeg):
    mesh = meshes.curved_box(cell, n, degree, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    pts, _ = tg.refcell.gauss_rule(cell, rdeg)
    ps = tg.PointSet(cell, pts, np.ones(len(pts)))
    count = torch.zeros(1, dtype=torch.int64, device="cuda")
    got = tg.geometric_factors_block(g, 0, ps, ("points", "jacobian", "detj", "pinv"),
                                     precision="split", recomputed=count)
    want = oracle(mesh, g, cell, degree, pts, ("x", "j", "detj", "k"))
    for f, field in got.items():
        assert field.chunks[0].data.dtype == torch.float32
        err = orc.rel_err(field.to_host_cell_major(), want[KEYS[f]])
        assert err < SPLIT_TOL[f], (f, err)
    assert int(count.item()) == 0  # no point of these meshes is near-degenerate


def test_split_is_more_accurate_than_plain_f32(cuda):
    """Shifting by the cell's first node in f64 before rounding keeps J's rounding relative to
    the cell size; plain f32 rounds coordinates relative to their distance from the origin."""
    mesh = meshes.curved_box("Tetrahedron", 16, 2, jitter=0.02)
    pts, _ = tg.refcell.gauss_rule("Tetrahedron", 4)
    ps = tg.PointSet("Tetrahedron", pts, np.ones(len(pts)))
    g64 = tg.Geometry.from_host(mesh, dtype=torch.float64)
    g32 = tg.Geometry.from_host(mesh, dtype=torch.float32)
    want = oracle(mesh, g64, "Tetrahedron", 2, pts, ("j", "detj"))
    split = tg.geometric_factors_block(g64, 0, ps, ("jacobian", "detj"), precision="split")
    plain = tg.geometric_factors_block(g32, 0, ps, ("jacobian", "detj"))
    for f in ("jacobian", "detj"):
        es = orc.rel_err(split[f].to_host_cell_major(), want[KEYS[f]])
        ep = orc.rel_err(plain[f].to_host_cell_major(), want[KEYS[f]])
        assert es < ep / 3, (f, es, ep)


def test_near_degenerate_points_are_recomputed_in_f64(cuda):
    """A sliver tetrahedron (height 1e-6) next to a regular one: its points exceed the condition
    limit and get det J and K from FP64; their det J is then exact to f32 rounding."""
    nodes = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.3, 0.3, 1e-6],
                      [0.0, 0.0, 1.0]]) + 100.0
    cells = np.array([[0, 1, 2, 3], [0, 1, 2, 4]], dtype=np.uint32)
    mesh = meshes.HostMesh(3, nodes, [meshes.HostBlock("Tetrahedron", 1, cells)])
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    pts, _ = tg.refcell.gauss_rule("Tetrahedron", 2)
    ps = tg.PointSet("Tetrahedron", pts, np.ones(len(pts)))
    count = torch.zeros(1, dtype=torch.int64, device="cuda")
    got = tg.geometric_factors_block(g, 0, ps, ("detj", "pinv"), precision="split", recomputed=count)
    want = oracle(mesh, g, "Tetrahedron", 1, pts, ("detj", "j"))
    assert int(count.item()) == len(pts)  # every point of the sliver, none of the other cell
    d = got["detj"].to_host_cell_major()[..., 0]
    assert np.all(np.abs(d[0] - want["detj"][0, :, 0]) <= 2e-7 * np.abs(want["detj"][0, :, 0]))
    # K by a pivoted LU inverse of the f64 J: the normal-equations route of the host reference
    # (reference.rs:197-235) squares the condition number (1e12 here) and is not an oracle for K
    # of a sliver.
    jm = want["j"][0].reshape(-1, 3, 3)  # [q][d][g] = J(g, d)
    kref = np.linalg.inv(np.transpose(jm, (0, 2, 1)))  # [q][t][g]
    kref = np.transpose(kref, (0, 2, 1)).reshape(-1, 9)  # K(t, g) at g * 3 + t
    k = got["pinv"].to_host_cell_major()
    assert orc.rel_err(k[0], kref) < 1e-6


@pytest.mark.parametrize("degree", [2, 4])
def test_split_surface_errors(cuda, degree):
    mesh = meshes.perturbed_radius(meshes.sphere(2, degree), 0.02)
    flags = (np.arange(mesh.blocks[0].num_cells) % 2).astype(np.uint32)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64, flags=[flags])
    pts, _ = tg.refcell.gauss_rule("Triangle", 2 * degree)
    ps = tg.PointSet("Triangle", pts, np.ones(len(pts)))
    got = tg.geometric_factors_block(g, 0, ps, ("points", "jacobian", "detj", "pinv", "normals"),
                                     precision="split")
    want = oracle(mesh, g, "Triangle", degree, pts, ("x", "j", "detj", "k", "normals"), flags=flags)
    for f, field in got.items():
        err = orc.rel_err(field.to_host_cell_major(), want[KEYS[f]])
        assert err < SPLIT_TOL[f], (f, err)


def test_split_is_deterministic_and_matches_per_factor_launches(cuda):
    mesh = meshes.curved_box("Hexahedron", 3, 2, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    pts, _ = tg.refcell.gauss_rule("Hexahedron", 4)
    ps = tg.PointSet("Hexahedron", pts, np.ones(len(pts)))
    a = tg.geometric_factors_block(g, 0, ps, ("points", "detj", "pinv"), precision="split")
    b = tg.geometric_factors_block(g, 0, ps, ("points", "detj", "pinv"), precision="split")
    c = tg.geometric_factors_block(g, 0, ps, ("detj",), precision="split")
    for k in a:
        assert torch.equal(a[k].chunks[0].data, b[k].chunks[0].data)
    assert torch.equal(a["detj"].chunks[0].data, c["detj"].chunks[0].data)


def test_split_rejects_f32_meshes(cuda):
    mesh = meshes.cube_box("Tetrahedron", 1, 1)
    g = tg.Geometry.from_host(mesh, dtype=torch.float32)
    pts, _ = tg.refcell.gauss_rule("Tetrahedron", 2)
    with pytest.raises(tg.GridError):
        tg.geometric_factors_block(g, 0, tg.PointSet("Tetrahedron", pts, np.ones(len(pts))),
                                   ("detj",), precision="split")


def test_integer_conversions_match_the_instructions(cuda):
    """The split kernels round f64 -> f32 and widen f32 -> f64 with integer operations; over
    random bit patterns (NaN, infinities, subnormals), exact ties, and the edges of the f32
    normal range, both match the conversion instructions bit for bit."""
    from gridcl_gb300._lib import check, lib
    from gridcl_gb300.geometry import current_stream_handle

    rng = np.random.default_rng(17)
    parts = [rng.integers(0, 2**63, 1 << 20, dtype=np.int64).view(np.float64)]
    f = rng.standard_normal(1 << 18).astype(np.float32) * np.float32(2.0) ** rng.integers(-126, 127, 1 << 18)
    nxt = np.nextafter(f, np.float32(np.inf), dtype=np.float32)
    ties = 0.5 * (f.astype(np.float64) + nxt.astype(np.float64))  # exact halfway points
    parts += [ties, np.nextafter(ties, np.inf), np.nextafter(ties, -np.inf), f.astype(np.float64)]
    fmax = float(np.finfo(np.float32).max)
    tiny = float(np.finfo(np.float32).tiny)
    edges = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, fmax, -fmax, fmax * (1 + 2.0**-25),
                      fmax * (1 + 2.0**-24), tiny, -tiny, tiny * (1 - 2.0**-30), tiny * 0.5,
                      2.0**-149, 2.0**-150, 2.0**-151, 1.0, 1.0 + 2.0**-24, 1.0 + 3 * 2.0**-24])
    parts.append(np.concatenate([edges, -edges]))
    x = torch.from_numpy(np.concatenate(parts)).cuda()
    bad = torch.zeros(2, dtype=torch.int64, device="cuda")
    check(lib().tlg_selftest_conversions(x.data_ptr(), x.numel(), bad.data_ptr(), current_stream_handle()))
    assert bad.tolist() == [0, 0]


def test_measure_of_a_split_field(cuda):
    """measure_block sums a split-precision (f32) det J field in f32, blocking or not."""
    mesh = meshes.curved_box("Tetrahedron", 4, 2, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    pts, w = tg.refcell.gauss_rule("Tetrahedron", 4)
    ps = tg.PointSet("Tetrahedron", pts, w)
    f = tg.geometric_factors_block(g, 0, ps, ("detj",), precision="split")
    dev = tg.measure_block(g, 0, ps, detj=f["detj"], sync=False)
    assert dev.dtype == torch.float32 and dev.is_cuda
    blocking = tg.measure_block(g, 0, ps, detj=f["detj"])
    assert float(dev.item()) == blocking
    plain = tg.measure_block(g, 0, ps)  # the f64 path
    assert abs(blocking - plain) < 1e-6 * abs(plain)
    assert abs(plain - 1.0) < 1e-12  # the curved map keeps the unit cube's boundary


@pytest.mark.parametrize("ncells", [1, 64, 65, 4097, 262145])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_fused_measure_equals_two_steps(cuda, ncells, dtype):
    """tlg_measure (level 1 of the tree straight from det J, the caller's workspace) gives the bits
    of tlg_measure_cell_sums followed by tlg_sum, and measure_block over one chunk equals it over
    several chunks."""
    from gridcl_gb300._lib import check, lib
    from gridcl_gb300.geometry import current_stream_handle

    rng = np.random.default_rng(ncells)
    nq = 7
    f = tg.QuadField.uninit(ncells, nq, 1, 16, dtype)
    f.chunks[0].data.copy_(torch.from_numpy(rng.random(f.chunks[0].data.numel())))
    w = torch.from_numpy(rng.random(nq)).to(dtype).cuda()
    es = 8 if dtype == torch.float64 else 4
    s = current_stream_handle()
    nbytes = int(lib().tlg_measure_workspace_bytes(es, ncells))
    work = torch.empty(max(nbytes, es), dtype=torch.uint8, device="cuda")
    fused = torch.empty(1, dtype=dtype, device="cuda")
    check(lib().tlg_measure(f.chunks[0].data.data_ptr(), es, ncells, nq, 16, w.data_ptr(), work.data_ptr(),
                            nbytes, fused.data_ptr(), s))
    sums = torch.empty(ncells, dtype=dtype, device="cuda")
    check(lib().tlg_measure_cell_sums(f.chunks[0].data.data_ptr(), es, ncells, nq, 16, w.data_ptr(),
                                      sums.data_ptr(), s))
    tb = int(lib().tlg_sum_workspace_bytes(es, ncells))
    tw = torch.empty(max(tb, es), dtype=torch.uint8, device="cuda")
    two = torch.empty(1, dtype=dtype, device="cuda")
    check(lib().tlg_sum(sums.data_ptr(), es, ncells, tw.data_ptr(), tb, two.data_ptr(), s))
    assert torch.equal(fused, two)
    if nbytes > 0:
        with pytest.raises(tg.GridError):
            check(lib().tlg_measure(f.chunks[0].data.data_ptr(), es, ncells, nq, 16, w.data_ptr(),
                                    work.data_ptr(), nbytes - 1, fused.data_ptr(), s))
