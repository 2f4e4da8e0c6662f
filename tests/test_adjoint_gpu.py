"""Adjoint (node cotangents through the device CSR) against the f64 oracle and central finite
differences; the CSR against a stable host sort (GPU)."""

import numpy as np
import pytest
import torch

import gridcl_gb300 as tg
from gridcl_gb300 import meshes
from oracle import oracle as orc

pytestmark = pytest.mark.gpu


def stable_csr(dofmap, num_nodes):
    keys = np.minimum(dofmap.ravel().astype(np.int64), num_nodes - 1)
    order = np.argsort(keys, kind="stable")
    counts = np.bincount(keys, minlength=num_nodes)
    offsets = np.concatenate([[0], np.cumsum(counts)])
    return offsets, order


@pytest.mark.parametrize("cell,n,p", [("Tetrahedron", 3, 2), ("Hexahedron", 24, 2), ("Prism", 2, 1)])
def test_csr_is_the_stable_sort(cuda, cell, n, p):
    mesh = meshes.cube_box(cell, n, p)
    g = tg.Geometry.from_host(mesh)
    inc = tg.node_incidence(g, 0)
    offsets, entries = stable_csr(mesh.blocks[0].cells, mesh.num_nodes)
    assert np.array_equal(inc.offsets.cpu().numpy().view(np.uint32), offsets)
    assert np.array_equal(inc.entries.cpu().numpy().view(np.uint32)[: entries.size], entries)


def test_csr_with_unused_and_clamped_nodes(cuda):
    nodes = np.random.default_rng(1).random((40, 3))
    cells = np.array([[3, 5, 7, 9], [9, 3, 12, 77], [1, 2, 3, 4], [30, 31, 32, 39]], dtype=np.uint32)
    mesh = meshes.HostMesh(3, nodes, [meshes.HostBlock("Tetrahedron", 1, cells)])
    g = tg.Geometry.from_host(mesh)
    inc = tg.node_incidence(g, 0)
    offsets, entries = stable_csr(cells, 40)
    assert np.array_equal(inc.offsets.cpu().numpy().view(np.uint32), offsets)
    assert np.array_equal(inc.entries.cpu().numpy().view(np.uint32), entries)


def cotangent_fields(rng, ncells, nq, dtype, gd=3):
    """Seeded standard-normal cotangents as tile-16 fields, with their cell-major copies."""
    out, host = {}, {}
    for name, length in (("points", gd), ("detj", 1), ("pinv", gd * gd)):
        f = tg.QuadField.uninit(ncells, nq, length, 16, dtype)
        vals = rng.standard_normal(f.chunks[0].data.numel())
        f.chunks[0].data.copy_(torch.from_numpy(vals).to(dtype))
        out[name] = f
        host[name] = f.to_host_cell_major().astype(np.float64)
    return out, host


@pytest.mark.parametrize("cell,n,degree,rdeg", [("Tetrahedron", 3, 2, 4), ("Hexahedron", 3, 2, 4),
                                                ("Tetrahedron", 2, 3, 6), ("Prism", 2, 2, 4),
                                                ("Hexahedron", 2, 1, 3), ("Quadrilateral", 4, 2, 3),
                                                ("Triangle", 5, 3, 4)])
def test_vjp_matches_the_oracle(cuda, cell, n, degree, rdeg):
    mesh = jittered_box(cell, n, degree)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    pts, _ = tg.refcell.gauss_rule(cell, rdeg)
    ps = tg.PointSet(cell, pts, np.ones(len(pts)))
    ncells = mesh.blocks[0].num_cells
    rng = np.random.default_rng(7)
    ct64, host = cotangent_fields(rng, ncells, len(pts), torch.float64, g.gdim)
    absx = g.nodes.cpu().numpy() + np.array(g.origin[: g.gdim])
    want = orc.vjp(cell, degree, absx, mesh.blocks[0].cells, pts, host["points"],
                   host["detj"][..., 0], host["pinv"])
    got, _ = tg.vjp_block(g, 0, ps, ct64)
    assert orc.rel_err(got.cpu().numpy(), want) < 1e-11
    again, _ = tg.vjp_block(g, 0, ps, ct64)
    assert torch.equal(got, again)  # deterministic
    # Split precision: f32 cotangents (the same values rounded), FP32 arithmetic.
    ct32 = {k: tg.QuadField([tg.geometry.QuadChunk(0, ncells, v.chunks[0].data.float())], ncells,
                            len(pts), v.length, 16) for k, v in ct64.items()}
    host32 = {k: v.to_host_cell_major().astype(np.float64) for k, v in ct32.items()}
    want32 = orc.vjp(cell, degree, absx, mesh.blocks[0].cells, pts, host32["points"],
                     host32["detj"][..., 0], host32["pinv"])
    got32, _ = tg.vjp_block(g, 0, ps, ct32, precision="split")
    assert orc.rel_err(got32.cpu().numpy(), want32) < 2e-5


def jittered_box(cell, n, degree):
    """The curved unit cube, or for 2D cells the unit square with interior nodes jittered."""
    if cell in ("Quadrilateral", "Triangle"):
        m = meshes.square_box(cell, n, degree)
        m.nodes = meshes.jitter_interior(m.nodes, m.nodes, 0.02 / n, 2026)
        return m
    return meshes.curved_box(cell, n, degree, jitter=0.02)


@pytest.mark.parametrize("precision", ["native", "split"])
@pytest.mark.parametrize("cell,n,degree,rdeg", [("Hexahedron", 3, 2, 4), ("Tetrahedron", 3, 3, 5),
                                                ("Quadrilateral", 5, 2, 3), ("Triangle", 4, 1, 2)])
def test_fused_forward_matches_the_forward_kernels(cuda, precision, cell, n, degree, rdeg):
    """The fused forward sums J over the four lanes of a cell (a butterfly), the forward kernels
    over the nodes in order: equal to rounding, and both within tolerance of the oracle."""
    mesh = jittered_box(cell, n, degree)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    pts, _ = tg.refcell.gauss_rule(cell, rdeg)
    ps = tg.PointSet(cell, pts, np.ones(len(pts)))
    dt = torch.float64 if precision == "native" else torch.float32
    ct, _ = cotangent_fields(np.random.default_rng(3), mesh.blocks[0].num_cells, len(pts), dt, g.gdim)
    names = ("points", "jacobian", "detj", "pinv")
    _, fused = tg.vjp_block(g, 0, ps, ct, precision=precision, forward=names)
    plain = tg.geometric_factors_block(g, 0, ps, names, precision=precision)
    absx = g.nodes.cpu().numpy() + np.array(g.origin[: g.gdim])
    want = orc.eval_block(cell, degree, absx, mesh.blocks[0].cells, pts)
    tight = 1e-14 if precision == "native" else 2e-6
    loose = 1e-12 if precision == "native" else 1e-5
    for k, o in zip(names, ("x", "j", "detj", "k")):
        f = fused[k].to_host_cell_major()
        assert orc.rel_err(f, plain[k].to_host_cell_major()) < tight, k
        assert orc.rel_err(f, want[o]) < loose, k


def test_vjp_against_central_differences(cuda):
    """Central differences (step 1e-6) of L = sum(xbar . x + dbar det J + kbar : K), evaluated by
    the f64 forward kernels, at 12 seeded node coordinates."""
    mesh = meshes.curved_box("Tetrahedron", 2, 2, jitter=0.02)
    pts, _ = tg.refcell.gauss_rule("Tetrahedron", 4)
    ps = tg.PointSet("Tetrahedron", pts, np.ones(len(pts)))
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    ct, host = cotangent_fields(np.random.default_rng(11), mesh.blocks[0].num_cells, len(pts),
                                torch.float64)
    grad, _ = tg.vjp_block(g, 0, ps, ct)
    grad = grad.cpu().numpy()

    def functional(nodes_rel):
        gg = tg.Geometry(g.blocks, torch.from_numpy(nodes_rel).cuda(), g.origin)
        f = tg.geometric_factors_block(gg, 0, ps, ("points", "detj", "pinv"))
        return sum(float((f[k].to_host_cell_major() * host[k]).sum()) for k in ("points", "detj", "pinv"))

    base = g.nodes.cpu().numpy()
    rng = np.random.default_rng(5)
    h = 1e-6
    for n in rng.choice(mesh.num_nodes, 4, replace=False):
        for c in range(3):
            xp, xm = base.copy(), base.copy()
            xp[n, c] += h
            xm[n, c] -= h
            fd = (functional(xp) - functional(xm)) / (2 * h)
            assert abs(fd - grad[n, c]) <= 1e-6 * max(1.0, abs(grad[n, c])), (n, c, fd, grad[n, c])


def test_fd_check_on_seeded_nodes(cuda):
    """The product's local central-difference check (f64 forward kernels) agrees with the f64
    adjoint at seeded nodes of a curved Q2 hexahedral box."""
    mesh = meshes.curved_box("Hexahedron", 4, 2, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    pts, _ = tg.refcell.gauss_rule("Hexahedron", 4)
    ps = tg.PointSet("Hexahedron", pts, np.ones(len(pts)))
    ct, host = cotangent_fields(np.random.default_rng(2), mesh.blocks[0].num_cells, len(pts), torch.float64)
    grad, _ = tg.vjp_block(g, 0, ps, ct)
    sample = np.random.default_rng(9).choice(mesh.num_nodes, 40, replace=False)
    res = tg.fd_check(g, 0, ps, {"points": host["points"], "detj": host["detj"][..., 0],
                                 "pinv": host["pinv"]}, grad.cpu().numpy(), sample)
    assert res["max_rel_err"] < 1e-6, res


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_gather_sums_rows_in_f64(cuda, dtype):
    """tlg_vjp_gather on seeded rows spanning 60 decades, with zeros, negative zeros and
    subnormals: f64 rows summed in f64, f32 rows as a TwoSum pair rounded to f64, both within
    n 2^-46 of the exact sum relative to the sum of magnitudes."""
    from gridcl_gb300._lib import check, lib
    from gridcl_gb300.geometry import current_stream_handle

    mesh = meshes.cube_box("Hexahedron", 4, 2)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    inc = tg.node_incidence(g, 0)
    cells = mesh.blocks[0].cells
    ncells, k = cells.shape
    rng = np.random.default_rng(4)
    vals = rng.standard_normal((ncells, k, 4)) * 10.0 ** rng.integers(-30, 30, size=(ncells, k, 4))
    flat = vals.reshape(-1, 4)
    flat[rng.choice(flat.shape[0], 40, replace=False), :3] = 0.0
    flat[rng.choice(flat.shape[0], 40, replace=False), :3] = -0.0
    flat[rng.choice(flat.shape[0], 40, replace=False), :3] = 3e-41  # subnormal in f32
    vals[..., 3] = 0.0
    vals = vals.astype(dtype)
    local = torch.from_numpy(vals).cuda()
    grad = torch.empty((mesh.num_nodes, 3), dtype=torch.float64, device="cuda")
    check(lib().tlg_vjp_gather(inc.offsets.data_ptr(), inc.entries.data_ptr(), mesh.num_nodes, 3,
                               local.data_ptr(), np.dtype(dtype).itemsize, grad.data_ptr(),
                               current_stream_handle()))
    got = grad.cpu().numpy()
    v64 = vals.reshape(-1, 4)[:, :3].astype(np.float64)
    want = np.zeros((mesh.num_nodes, 3))
    mag = np.zeros((mesh.num_nodes, 3))
    np.add.at(want, cells.ravel(), v64)
    np.add.at(mag, cells.ravel(), np.abs(v64))
    assert np.all(np.abs(got - want) <= 8 * 2.0 ** -46 * mag)


@pytest.mark.parametrize("precision", ["native", "split"])
@pytest.mark.parametrize("n,degree,rdeg", [(3, 2, 4), (5, 2, 5), (4, 1, 2), (3, 1, 4), (2, 2, 3)])
def test_sumfact_adjoint_matches_node_rows(cuda, n, degree, rdeg, precision):
    """Hexahedra at tensor rules: the sum-factorised adjoint (one cell per thread, transposed
    contraction row by row and plane by plane) against the node-row kernel and the oracle, with the
    fused forward; cell counts that are not multiples of the 32-cell warp runs."""
    mesh = meshes.curved_box("Hexahedron", n, degree, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    pts, _ = tg.refcell.gauss_rule("Hexahedron", rdeg)
    ps = tg.PointSet("Hexahedron", pts, np.ones(len(pts)))
    ncells = mesh.blocks[0].num_cells
    dt = torch.float64 if precision == "native" else torch.float32
    ct, host = cotangent_fields(np.random.default_rng(13), ncells, len(pts), dt)
    names = ("points", "jacobian", "detj", "pinv")
    with tg.with_strategy("sumfact"):
        got, fused = tg.vjp_block(g, 0, ps, ct, precision=precision, forward=names)
        assert tg.last_kernel_family() == "sumfact"
    with tg.with_strategy("direct"):
        rows, plain = tg.vjp_block(g, 0, ps, ct, precision=precision, forward=names)
        assert tg.last_kernel_family() == "direct"
    absx = g.nodes.cpu().numpy() + np.array(g.origin[:3])
    want = orc.vjp("Hexahedron", degree, absx, mesh.blocks[0].cells, pts, host["points"],
                   host["detj"][..., 0], host["pinv"])
    tol = 1e-11 if precision == "native" else 2e-5
    assert orc.rel_err(got.cpu().numpy(), want) < tol
    assert orc.rel_err(got.cpu().numpy(), rows.cpu().numpy()) < tol
    fwd = orc.eval_block("Hexahedron", degree, absx, mesh.blocks[0].cells, pts)
    for k, o in zip(names, ("x", "j", "detj", "k")):
        f = fused[k].to_host_cell_major()
        assert orc.rel_err(f, plain[k].to_host_cell_major()) < (1e-13 if precision == "native" else 2e-6), k
        assert orc.rel_err(f, fwd[o]) < (1e-12 if precision == "native" else 1e-5), k


@pytest.mark.parametrize("missing", ["points", "detj", "pinv"])
def test_sumfact_adjoint_with_missing_cotangents(cuda, missing):
    """A missing cotangent field counts as zero, in both kernel families."""
    mesh = meshes.curved_box("Hexahedron", 3, 2, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    pts, _ = tg.refcell.gauss_rule("Hexahedron", 4)
    ps = tg.PointSet("Hexahedron", pts, np.ones(len(pts)))
    ct, host = cotangent_fields(np.random.default_rng(17), mesh.blocks[0].num_cells, len(pts), torch.float64)
    del ct[missing]
    host[missing] = np.zeros_like(host[missing])
    with tg.with_strategy("sumfact"):
        got, _ = tg.vjp_block(g, 0, ps, ct)
    absx = g.nodes.cpu().numpy() + np.array(g.origin[:3])
    want = orc.vjp("Hexahedron", 2, absx, mesh.blocks[0].cells, pts, host["points"],
                   host["detj"][..., 0], host["pinv"])
    assert orc.rel_err(got.cpu().numpy(), want) < 1e-11


@pytest.mark.parametrize("cell,degree,rdeg,family", [("Hexahedron", 2, 4, "sumfact"), ("Hexahedron", 1, 2, "sumfact"),
                                                     ("Prism", 2, 4, "direct"), ("Tetrahedron", 2, 4, "direct")])
def test_adjoint_auto_policy(cuda, cell, degree, rdeg, family):
    mesh = meshes.curved_box(cell, 2, degree, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    pts, _ = tg.refcell.gauss_rule(cell, rdeg)
    ps = tg.PointSet(cell, pts, np.ones(len(pts)))
    ct, _ = cotangent_fields(np.random.default_rng(1), mesh.blocks[0].num_cells, len(pts), torch.float32)
    with tg.with_strategy("auto"):
        tg.vjp_block(g, 0, ps, ct, precision="split")
        assert tg.last_kernel_family() == family


def curve(n, degree, gd):
    """n curved intervals of degree `degree` on a closed curve in the plane (gd 2) or on a helix
    turn (gd 3, open)."""
    nodes, cells = [], []
    per = degree
    total = n * per + (1 if gd == 3 else 0)
    for c in range(n):
        last = (c + 1) * per if gd == 3 else ((c + 1) * per) % (n * per)
        cells.append([c * per, last] + [c * per + i for i in range(1, degree)])
    for i in range(total):
        t = 2 * np.pi * i / (n * per)
        r = 1 + 0.05 * np.sin(3 * t)
        nodes.append([r * np.cos(t), r * np.sin(t)] + ([0.3 * t] if gd == 3 else []))
    return meshes.HostMesh(gd, np.array(nodes), [meshes.HostBlock("Interval", degree, np.array(cells, dtype=np.uint32))])


def surface_case(kind):
    if kind == "sphere":
        return meshes.perturbed_radius(meshes.sphere(1, 2), 0.05), "Triangle", 2, 4
    if kind == "sphere3":
        return meshes.perturbed_radius(meshes.sphere(1, 3), 0.05), "Triangle", 3, 5
    if kind == "quads":
        m = meshes.square_box("Quadrilateral", 3, 2)
        x = meshes.jitter_interior(m.nodes, m.nodes, 0.02 / 3, 2026)
        z = 0.1 * np.sin(2 * np.pi * x[:, 0]) * np.sin(2 * np.pi * x[:, 1])
        return meshes.HostMesh(3, np.column_stack([x, z]), m.blocks), "Quadrilateral", 2, 4
    if kind == "circle":
        return curve(9, 3, 2), "Interval", 3, 5
    return curve(8, 2, 3), "Interval", 2, 4


@pytest.mark.parametrize("kind", ["sphere", "sphere3", "quads", "circle", "helix"])
def test_surface_adjoint_matches_the_oracle(cuda, kind):
    """Below codimension 0: cotangents on x, the area element, the pseudo-inverse and (TD + 1 = GD)
    the unit normals, with seeded flipped cells, against the oracle's adjoint (itself checked
    against central differences); f64 within 1e-11, split precision (f32 cotangents) within 2e-5."""
    mesh, cell, degree, rdeg = surface_case(kind)
    ncells = mesh.blocks[0].num_cells
    flags = np.random.default_rng(3).integers(0, 2, ncells).astype(np.uint32)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64, flags=[flags])
    pts, _ = tg.refcell.gauss_rule(cell, rdeg)
    ps = tg.PointSet(cell, pts, np.ones(len(pts)))
    td, gd = tg.refcell.tdim(cell), g.gdim
    rng = np.random.default_rng(17)
    ct, host = cotangent_fields(rng, ncells, len(pts), torch.float64, gd)
    if td + 1 == gd:
        f = tg.QuadField.uninit(ncells, len(pts), gd, 16, torch.float64)
        f.chunks[0].data.copy_(torch.from_numpy(rng.standard_normal(f.chunks[0].data.numel())))
        ct["normals"] = f
        host["normals"] = f.to_host_cell_major()
    pinv_len = td * gd
    if ct["pinv"].length != pinv_len:  # cotangent_fields makes gd * gd components
        f = tg.QuadField.uninit(ncells, len(pts), pinv_len, 16, torch.float64)
        f.chunks[0].data.copy_(torch.from_numpy(rng.standard_normal(f.chunks[0].data.numel())))
        ct["pinv"] = f
        host["pinv"] = f.to_host_cell_major()
    absx = g.nodes.cpu().numpy() + np.array(g.origin[:gd])
    want = orc.vjp(cell, degree, absx, mesh.blocks[0].cells, pts, host["points"], host["detj"][..., 0],
                   host["pinv"], nbar=host.get("normals"), flags=flags)
    got, _ = tg.vjp_block(g, 0, ps, ct)
    assert orc.rel_err(got.cpu().numpy(), want) < 1e-11
    ct32 = {k: tg.QuadField([tg.geometry.QuadChunk(0, ncells, v.chunks[0].data.float())], ncells, len(pts),
                            v.length, 16) for k, v in ct.items()}
    host32 = {k: v.to_host_cell_major().astype(np.float64) for k, v in ct32.items()}
    want32 = orc.vjp(cell, degree, absx, mesh.blocks[0].cells, pts, host32["points"], host32["detj"][..., 0],
                     host32["pinv"], nbar=host32.get("normals"), flags=flags)
    got32, _ = tg.vjp_block(g, 0, ps, ct32, precision="split")
    assert orc.rel_err(got32.cpu().numpy(), want32) < 2e-5


@pytest.mark.parametrize("precision", ["native", "split"])
def test_surface_fused_forward(cuda, precision):
    """The surface adjoint's fused forward (x, J, area element, K, normals) equals the forward
    kernels' to rounding."""
    mesh, cell, degree, rdeg = surface_case("sphere")
    flags = np.random.default_rng(3).integers(0, 2, mesh.blocks[0].num_cells).astype(np.uint32)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64, flags=[flags])
    pts, _ = tg.refcell.gauss_rule(cell, rdeg)
    ps = tg.PointSet(cell, pts, np.ones(len(pts)))
    dt = torch.float64 if precision == "native" else torch.float32
    ct, _ = cotangent_fields(np.random.default_rng(3), mesh.blocks[0].num_cells, len(pts), dt, 3)
    del ct["pinv"]
    names = ("points", "jacobian", "detj", "pinv", "normals")
    _, fused = tg.vjp_block(g, 0, ps, ct, precision=precision, forward=names)
    plain = tg.geometric_factors_block(g, 0, ps, names, precision=precision)
    tol = 1e-13 if precision == "native" else 2e-6
    for k in names:
        assert orc.rel_err(fused[k].to_host_cell_major(), plain[k].to_host_cell_major()) < tol, k


def test_surface_adjoint_fd_check(cuda):
    mesh, cell, degree, rdeg = surface_case("sphere")
    flags = np.random.default_rng(5).integers(0, 2, mesh.blocks[0].num_cells).astype(np.uint32)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64, flags=[flags])
    pts, _ = tg.refcell.gauss_rule(cell, rdeg)
    ps = tg.PointSet(cell, pts, np.ones(len(pts)))
    rng = np.random.default_rng(8)
    nc, nq = mesh.blocks[0].num_cells, len(pts)
    host = {"detj": rng.standard_normal((nc, nq)), "normals": rng.standard_normal((nc, nq, 3)),
            "pinv": rng.standard_normal((nc, nq, 6))}
    ct = {}
    for name, v in host.items():
        ln = 1 if name == "detj" else v.shape[-1]
        f = tg.QuadField.uninit(nc, nq, ln, 16, torch.float64)
        vals = v.reshape(nc, nq, ln)
        pad = np.zeros((-(-nc // 16) * 16, nq, ln))
        pad[:nc] = vals
        pad[nc:] = vals[-1]
        f.chunks[0].data.copy_(torch.from_numpy(pad.reshape(-1, 16, nq, ln).transpose(0, 2, 3, 1).ravel()))
        ct[name] = f
    grad, _ = tg.vjp_block(g, 0, ps, ct)
    sample = np.random.default_rng(9).choice(mesh.num_nodes, 12, replace=False)
    res = tg.fd_check(g, 0, ps, host, grad.cpu().numpy(), sample)
    assert res["max_rel_err"] < 1e-6, res


@pytest.mark.parametrize("precision", ["native", "split"])
def test_adjoint_batch_equals_the_blocks(cuda, precision):
    """The hybrid mesh's fused forward + adjoint in one graph launch: the node cotangents are the
    per-block adjoints' summed in block order, bit for bit, and the forward fields those of the
    per-block fused passes."""
    mesh = meshes.hybrid_box(300, 120, 60)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    rule = tg.QuadRule([tg.PointSet("Hexahedron", *tg.refcell.gauss_rule("Hexahedron", 4)),
                        tg.PointSet("Prism", *tg.refcell.collapsed_rule("Prism", (3, 1, 7))),
                        tg.PointSet("Tetrahedron", *tg.refcell.collapsed_rule("Tetrahedron", (4, 3, 2)))])
    dt = torch.float64 if precision == "native" else torch.float32
    rng = np.random.default_rng(31)
    cts = []
    for blk in g.blocks:
        ct, _ = cotangent_fields(rng, blk.num_cells, len(rule.get(blk.element.cell)), dt)
        cts.append(ct)
    names = ("points", "jacobian", "detj", "pinv")
    batch = tg.AdjointBatch(g, rule, cts, precision=precision, forward=names, two_pass=False)
    batch.grad.fill_(float("nan"))  # the first block's sums overwrite every node
    batch.launch()
    batch.launch()  # a second launch replays the graph
    want = torch.zeros_like(batch.grad)
    for b, blk in enumerate(g.blocks):
        grad, fields = tg.vjp_block(g, b, rule.get(blk.element.cell), cts[b], precision=precision, forward=names)
        want += grad
        for k in names:
            assert torch.equal(fields[k].chunks[0].data, batch.fields[b][k].chunks[0].data), (b, k)
    assert torch.equal(batch.grad, want)


@pytest.mark.parametrize("precision", ["native", "split"])
def test_adjoint_batch_with_more_blocks_than_a_gather_pass(cuda, precision):
    """11 blocks (slices of one P2 tetrahedron mesh, sharing nodes): the node sums run as a pass of
    eight blocks writing the gradient and a pass of three adding onto it; the gradient equals the
    per-block adjoints summed in block order, bit for bit."""
    base = meshes.curved_box("Tetrahedron", 3, 2, jitter=0.02)
    parts = np.array_split(base.blocks[0].cells, 11)
    mesh = meshes.HostMesh(3, base.nodes, [meshes.HostBlock("Tetrahedron", 2, np.ascontiguousarray(c)) for c in parts])
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    ps = tg.PointSet("Tetrahedron", *tg.refcell.gauss_rule("Tetrahedron", 4))
    dt = torch.float64 if precision == "native" else torch.float32
    rng = np.random.default_rng(47)
    cts = [cotangent_fields(rng, blk.num_cells, len(ps), dt)[0] for blk in g.blocks]
    batch = tg.AdjointBatch(g, tg.QuadRule([ps]), cts, precision=precision)
    batch.grad.fill_(float("nan"))
    batch.launch()
    want = torch.zeros_like(batch.grad)
    for b in range(len(g.blocks)):
        grad, _ = tg.vjp_block(g, b, ps, cts[b], precision=precision)
        want += grad
    assert torch.equal(batch.grad, want)


@pytest.mark.parametrize("precision", ["native", "split"])
def test_adjoint_batch_on_the_mixed_box(cuda, precision):
    """The tetrahedron/hexahedron/pyramid box (P2, sin-mapped and jittered) in one adjoint graph:
    the node cotangents equal the per-block adjoints summed in block order, bit for bit, and the
    FP64 ones match the oracle's restated adjoint."""
    mesh = meshes.mixed_box(3, 2)
    x = meshes.sin_map(mesh.nodes, 0.05)
    mesh.nodes = meshes.jitter_interior(x, mesh.nodes, 0.02 / 3, 2026)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    rule = tg.QuadRule([tg.PointSet(c, *tg.refcell.gauss_rule(c, 4)) for c in ("Tetrahedron", "Hexahedron", "Pyramid")])
    dt = torch.float64 if precision == "native" else torch.float32
    rng = np.random.default_rng(37)
    cts, hosts = [], []
    for blk in g.blocks:
        ct, host = cotangent_fields(rng, blk.num_cells, len(rule.get(blk.element.cell)), dt)
        cts.append(ct)
        hosts.append(host)
    batch = tg.AdjointBatch(g, rule, cts, precision=precision)
    batch.launch()
    want = torch.zeros_like(batch.grad)
    absx = g.nodes.cpu().numpy() + np.array(g.origin[:3])
    oracle = np.zeros(want.shape)
    for b, blk in enumerate(g.blocks):
        pts = rule.get(blk.element.cell)
        grad, _ = tg.vjp_block(g, b, pts, cts[b], precision=precision)
        want += grad
        h = hosts[b]
        oracle += orc.vjp(blk.element.cell, 2, absx, mesh.blocks[b].cells, pts.points, h["points"],
                          h["detj"][..., 0], h["pinv"])
    assert torch.equal(batch.grad, want)
    assert orc.rel_err(batch.grad.cpu().numpy(), oracle) < (1e-11 if precision == "native" else 2e-5)


@pytest.mark.parametrize("precision", ["native", "split"])
def test_two_pass_adjoint_batch(cuda, precision):
    """two_pass: the hexahedra's forward fields from the policy's kernel, then the adjoint from det
    J and K read back (tlg_vjp_block_from_fields); the prisms and tetrahedra fused. The node
    cotangents against the one-pass batch (the forward kernels differ only in rounding) and the
    oracle; the forward fields those of tlg_eval_block."""
    mesh = meshes.hybrid_box(300, 120, 60)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    rule = tg.QuadRule([tg.PointSet("Hexahedron", *tg.refcell.gauss_rule("Hexahedron", 4)),
                        tg.PointSet("Prism", *tg.refcell.collapsed_rule("Prism", (3, 1, 7))),
                        tg.PointSet("Tetrahedron", *tg.refcell.collapsed_rule("Tetrahedron", (4, 3, 2)))])
    dt = torch.float64 if precision == "native" else torch.float32
    rng = np.random.default_rng(41)
    cts, hosts = [], []
    for blk in g.blocks:
        ct, host = cotangent_fields(rng, blk.num_cells, len(rule.get(blk.element.cell)), dt)
        cts.append(ct)
        hosts.append(host)
    names = ("points", "jacobian", "detj", "pinv")
    one = tg.AdjointBatch(g, rule, cts, precision=precision, forward=names, two_pass=False)
    one.launch()
    two = tg.AdjointBatch(g, rule, cts, precision=precision, forward=names, two_pass=True)
    two.launch()
    two.launch()
    # The default: two passes in split precision with det J and K among the forward fields.
    assert tg.AdjointBatch(g, rule, cts, precision=precision, forward=names).two_pass == (precision == "split")
    assert not tg.AdjointBatch(g, rule, cts, precision=precision, forward=("points",)).two_pass
    tol = 1e-12 if precision == "native" else 2e-5
    assert orc.rel_err(two.grad.cpu().numpy(), one.grad.cpu().numpy()) < tol
    absx = g.nodes.cpu().numpy() + np.array(g.origin[:3])
    want = np.zeros(two.grad.shape)
    for b, blk in enumerate(g.blocks):
        h = hosts[b]
        pts = rule.get(blk.element.cell).points
        want += orc.vjp(blk.element.cell, blk.element.degree, absx, mesh.blocks[b].cells, pts, h["points"],
                        h["detj"][..., 0], h["pinv"])
    assert orc.rel_err(two.grad.cpu().numpy(), want) < (1e-11 if precision == "native" else 2e-5)
    fwd = tg.geometric_factors_block(g, 0, rule.get("Hexahedron"), names,
                                     precision="split" if precision == "split" else "native")
    for k in names:
        assert torch.equal(two.fields[0][k].chunks[0].data, fwd[k].chunks[0].data), k


@pytest.mark.parametrize("precision", ["native", "split"])
@pytest.mark.parametrize("degree,counts,missing", [(2, (3, 3, 3), None), (2, (2, 3, 4), "points"),
                                                   (2, (3, 3, 3), "pinv"), (1, (2, 2, 2), None),
                                                   (1, (3, 2, 2), "detj"), (2, (5, 5, 5), None)])
def test_two_pass_adjoint_on_hexahedra(cuda, precision, degree, counts, missing):
    """The adjoint from det J and K read back on 27 hexahedra (a whole tile of 16 and a partial
    one), cube and anisotropic tensor rules, a missing cotangent counted as zero: against the
    oracle and the fused one-pass batch. vjp_sumfact_tile_kernel, except FP64 at 125 points, whose
    tile does not fit in shared memory (vjp_sumfact_bwd_kernel, one thread per cell)."""
    mesh = meshes.curved_box("Hexahedron", 3, degree, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    ps = tg.PointSet("Hexahedron", *tg.refcell.collapsed_rule("Hexahedron", counts))
    dt = torch.float64 if precision == "native" else torch.float32
    ct, host = cotangent_fields(np.random.default_rng(43), mesh.blocks[0].num_cells, len(ps), dt)
    if missing:
        del ct[missing]
        host[missing] = np.zeros_like(host[missing])
    names = ("detj", "pinv")
    two = tg.AdjointBatch(g, tg.QuadRule([ps]), [ct], precision=precision, forward=names, two_pass=True)
    two.launch()
    one = tg.AdjointBatch(g, tg.QuadRule([ps]), [ct], precision=precision, forward=names, two_pass=False)
    one.launch()
    absx = g.nodes.cpu().numpy() + np.array(g.origin[:3])
    want = orc.vjp("Hexahedron", degree, absx, mesh.blocks[0].cells, ps.points, host["points"],
                   host["detj"][..., 0], host["pinv"])
    tol = 1e-11 if precision == "native" else 2e-5
    assert orc.rel_err(two.grad.cpu().numpy(), want) < tol
    assert orc.rel_err(two.grad.cpu().numpy(), one.grad.cpu().numpy()) < tol


@pytest.mark.parametrize("precision", ["native", "split"])
@pytest.mark.parametrize("cell,degree,rdeg,missing", [("Tetrahedron", 2, 4, None), ("Tetrahedron", 3, 6, "points"),
                                                      ("Prism", 2, 4, None), ("Pyramid", 2, 4, "pinv"),
                                                      ("Hexahedron", 2, 4, None), ("Tetrahedron", 1, 3, "detj")])
def test_two_pass_adjoint_on_volume_cells(cuda, precision, cell, degree, rdeg, missing):
    """The adjoint from det J and K read back through the node rows (vjp_tile_kernel): tetrahedra,
    prisms, pyramids and hexahedra at a rule in no tensor order, odd and even point counts, a
    missing cotangent counted as zero; against the oracle and the fused one-pass batch."""
    mesh = meshes.curved_box(cell, 2, degree, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    pts, w = tg.refcell.gauss_rule(cell, rdeg)
    order = np.random.default_rng(5).permutation(len(pts))
    ps = tg.PointSet(cell, pts[order], w[order])
    dt = torch.float64 if precision == "native" else torch.float32
    ct, host = cotangent_fields(np.random.default_rng(53), mesh.blocks[0].num_cells, len(ps), dt)
    if missing:
        del ct[missing]
        host[missing] = np.zeros_like(host[missing])
    names = ("detj", "pinv")
    two = tg.AdjointBatch(g, tg.QuadRule([ps]), [ct], precision=precision, forward=names, two_pass=True)
    two.launch()
    one = tg.AdjointBatch(g, tg.QuadRule([ps]), [ct], precision=precision, forward=names, two_pass=False)
    one.launch()
    absx = g.nodes.cpu().numpy() + np.array(g.origin[:3])
    want = orc.vjp(cell, degree, absx, mesh.blocks[0].cells, ps.points, host["points"], host["detj"][..., 0],
                   host["pinv"])
    tol = 1e-11 if precision == "native" else 2e-5
    assert orc.rel_err(two.grad.cpu().numpy(), want) < tol
    assert orc.rel_err(two.grad.cpu().numpy(), one.grad.cpu().numpy()) < tol


def test_adjoint_batch_with_double_float_forward(cuda):
    """precision="df64": each block's forward fields from the double-float kernels (bit for bit
    the fields of tlg_eval_block with df64 tables, and within 1e-12 of the oracle's f64 values),
    its adjoint the split-precision one (bit for bit the node cotangents of the split batch)."""
    mesh = meshes.hybrid_box(300, 120, 60)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    rule = tg.QuadRule([tg.PointSet("Hexahedron", *tg.refcell.gauss_rule("Hexahedron", 4)),
                        tg.PointSet("Prism", *tg.refcell.collapsed_rule("Prism", (3, 1, 7))),
                        tg.PointSet("Tetrahedron", *tg.refcell.collapsed_rule("Tetrahedron", (4, 3, 2)))])
    rng = np.random.default_rng(37)
    cts = []
    for blk in g.blocks:
        ct, _ = cotangent_fields(rng, blk.num_cells, len(rule.get(blk.element.cell)), torch.float32)
        cts.append(ct)
    names = ("points", "jacobian", "detj", "pinv")
    batch = tg.AdjointBatch(g, rule, cts, precision="df64", forward=names)
    batch.launch()
    split = tg.AdjointBatch(g, rule, cts, precision="split")
    split.launch()
    torch.cuda.synchronize()
    assert torch.equal(batch.grad, split.grad)
    absx = g.nodes.cpu().numpy() + np.array(g.origin[:3])
    for b, blk in enumerate(g.blocks):
        ps = rule.get(blk.element.cell)
        want = tg.geometric_factors_block(g, b, ps, names, precision="df64")
        oracle = orc.eval_block(blk.element.cell, blk.element.degree, absx, mesh.blocks[b].cells, ps.points)
        for k, ok in zip(names, ("x", "j", "detj", "k")):
            got = batch.fields[b][k]
            assert got.chunks[0].data.dtype == torch.float64
            assert torch.equal(got.chunks[0].data, want[k].chunks[0].data), (b, k)
            assert orc.rel_err(got.to_host_cell_major(), oracle[ok]) < 1e-12, (b, k)


def test_csr_with_long_runs_of_unused_nodes(cuda):
    """Offsets across long runs of nodes without entries (a block's nodes in the middle of a large
    node array, as in a mesh of several blocks) against the host's stable sort."""
    rng = np.random.default_rng(6)
    nodes = rng.random((20_000, 3))
    cells = rng.integers(7_000, 7_300, size=(500, 4)).astype(np.uint32)
    cells[::97, 0] = 19_999
    mesh = meshes.HostMesh(3, nodes, [meshes.HostBlock("Tetrahedron", 1, cells)])
    g = tg.Geometry.from_host(mesh)
    inc = tg.node_incidence(g, 0)
    offsets, entries = stable_csr(cells, 20_000)
    assert np.array_equal(inc.offsets.cpu().numpy().view(np.uint32), offsets)
    assert np.array_equal(inc.entries.cpu().numpy().view(np.uint32)[: entries.size], entries)


@pytest.mark.parametrize("precision", ["native", "split"])
@pytest.mark.parametrize("cell,n,degree,rdeg", [("Tetrahedron", 2, 4, 5), ("Hexahedron", 2, 3, 5),
                                                ("Triangle", 3, 5, 6), ("Quadrilateral", 2, 4, 5)])
def test_runtime_k_adjoint_for_elements_without_node_row_kernels(cuda, cell, n, degree, rdeg, precision):
    """Codimension-0 elements without a compiled node-row kernel (P4 tetrahedra, Q3 hexahedra at a
    shuffled rule, P5 triangles, Q4 quadrilaterals) run the adjoint with K at run time, against the
    oracle."""
    mesh = jittered_box(cell, n, degree)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    pts, _ = tg.refcell.gauss_rule(cell, rdeg)
    pts = pts[np.random.default_rng(2).permutation(len(pts))]
    ps = tg.PointSet(cell, pts, np.ones(len(pts)))
    ncells = mesh.blocks[0].num_cells
    dt = torch.float64 if precision == "native" else torch.float32
    ct, host = cotangent_fields(np.random.default_rng(23), ncells, len(pts), dt, g.gdim)
    absx = g.nodes.cpu().numpy() + np.array(g.origin[: g.gdim])
    want = orc.vjp(cell, degree, absx, mesh.blocks[0].cells, pts, host["points"], host["detj"][..., 0],
                   host["pinv"])
    names = ("points", "detj", "pinv")
    got, fused = tg.vjp_block(g, 0, ps, ct, precision=precision, forward=names)
    assert tg.last_kernel_family() == "loops"
    assert orc.rel_err(got.cpu().numpy(), want) < (1e-11 if precision == "native" else 5e-5)
    plain = tg.geometric_factors_block(g, 0, ps, names, precision=precision)
    for k in names:  # the forward kernels sum in another order (cooperative or paired kernels)
        assert orc.rel_err(fused[k].to_host_cell_major(), plain[k].to_host_cell_major()) < (
            1e-13 if precision == "native" else 1e-5), k


def test_split_node_sums_are_within_their_stated_bound(cuda):
    """The node sums of f32 contribution rows (tlg_vjp_gather with local_dtype 4) are FP32 TwoSum
    pairs, each addition's rounding error kept in the low part, rounded once to f64. Against the
    f64 sums of the same rows the error stays within n^2 2^-48 sum |rows| per node and component (n
    its entries: the low part's own roundings), bounded here by 2^-40 sum |rows| — far below the
    2^-24 of FP32 sums and of the f32 contributions themselves."""
    rng = np.random.default_rng(41)
    ncells, k, nn = 20_000, 10, 9_000
    cells = rng.integers(0, nn, size=(ncells, k)).astype(np.uint32)
    mesh = meshes.HostMesh(3, rng.random((nn, 3)), [meshes.HostBlock("Tetrahedron", 2, cells)])
    g = tg.Geometry.from_host(mesh)
    inc = tg.node_incidence(g, 0)
    # Rows of widely different magnitudes and signs (cancellation within a node's sum).
    rows = (rng.standard_normal((ncells, k, 4)) * 10.0 ** rng.integers(-6, 3, size=(ncells, k, 1))).astype(np.float32)
    rows[..., 3] = 0.0
    local = torch.from_numpy(rows).cuda()
    grad = torch.empty((nn, 3), dtype=torch.float64, device="cuda")
    st = tg._lib.lib().tlg_vjp_gather(inc.offsets.data_ptr(), inc.entries.data_ptr(), nn, 3, local.data_ptr(), 4,
                                      grad.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert st == 0
    exact = np.zeros((nn, 3))
    mag = np.zeros((nn, 3))
    r64 = rows[..., :3].astype(np.float64)
    np.add.at(exact, cells.astype(np.int64).ravel(), r64.reshape(-1, 3))
    np.add.at(mag, cells.astype(np.int64).ravel(), np.abs(r64).reshape(-1, 3))
    err = np.abs(grad.cpu().numpy() - exact)
    count = np.bincount(cells.astype(np.int64).ravel(), minlength=nn).astype(np.float64)[:, None]
    assert np.all(err <= count ** 2 * 2.0 ** -48 * mag + 1e-300)
    assert np.all(err <= 2.0 ** -40 * mag + 1e-300)
