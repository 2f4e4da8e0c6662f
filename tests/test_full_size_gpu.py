"""Parity at the benchmark workloads' full sizes (GPU), against the oracle.

Where the oracle evaluates every value in seconds (the 3,072-cell P1 box, the Q2 adjoint's node
cotangents) every value is compared; elsewhere a seeded sample of cells (65,536, or 16,384 per
block of the hybrid mesh), as the reference's bench checks sampled cells against its host f64
evaluation (tetraloma-bench/src/families/degree.rs:1-25). Tolerances: the reference's 1e-12
(f64) and 1e-5 (f32), scaled as reference.rs:696-754 (amplification, node and origin ratios,
condition number for K and normals); split precision (FP32 arithmetic on an f64 mesh) against its
stated bounds, 5e-6 on the volume meshes and 1e-4 on the strongly distorted sphere.
"""

import numpy as np
import pytest
import torch

import gridcl_gb300 as tg
from gridcl_gb300 import meshes
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

FACTORS = ("points", "jacobian", "detj", "pinv")
ORC = {"points": "x", "jacobian": "j", "detj": "detj", "pinv": "k", "normals": "normals"}
SPLIT_VOLUME, SPLIT_SPHERE = 5e-6, 1e-4


def sample_cells(num_cells, count=65536, seed=2026):
    if num_cells <= count:
        return np.arange(num_cells)
    return np.sort(np.random.default_rng(seed).choice(num_cells, count, replace=False))


def field_at(field, cells):
    """A one-chunk QuadField's values at `cells`, gathered on the device from the tiled layout."""
    t, q, length = field.tile, field.num_points, field.length
    data = field.chunks[0].data
    c = torch.from_numpy(np.asarray(cells, dtype=np.int64)).to(data.device)
    qq = torch.arange(q, device=data.device)
    kk = torch.arange(length, device=data.device)
    idx = (((c // t)[:, None, None] * q + qq[None, :, None]) * length + kk[None, None, :]) * t + (c % t)[:, None, None]
    return data[idx].double().cpu().numpy()


def oracle_at(mesh, g, block, pts, cells, factors=("x", "j", "detj", "k")):
    blk = mesh.blocks[block]
    absx = g.nodes.double().cpu().numpy() + np.array(g.origin[: g.gdim])
    return orc.eval_block(blk.cell, blk.degree, absx, blk.cells[cells], pts, factors=factors), absx


def tolerances(blk, pts, absx, origin, j, td, gd, dtype_bytes):
    base = orc.TOL_F64 if dtype_bytes == 8 else orc.TOL_F32
    s = orc.tolerance_scale(blk.cell, blk.degree, "Equispaced", pts) * orc.node_ratio(blk.cell, blk.degree)
    s *= orc.origin_ratio(absx, np.array(origin[:gd]), j)
    sk = s * orc.condition_scale(j, td, gd)
    # Below codimension 0 the oracle's area element is the reference's sqrt(a c - b^2)
    # (tetraloma-geometry/src/layout.rs:198-213), whose own rounding grows with the condition
    # number: it takes K's scale there.
    sd = sk if td < gd else s
    return {"points": base, "jacobian": base * s, "detj": base * sd, "pinv": base * sk, "normals": base * sk}


def check(fields, want, cells, tol):
    errs = {f: orc.rel_err(field_at(fields[f], cells), want[ORC[f]]) for f in fields}
    bad = {f: (e, tol[f]) for f, e in errs.items() if not e < tol[f]}
    assert not bad, bad
    return errs


def test_p1_box_every_value(cuda):
    """3,072 P1 tetrahedra (8^3 x 6, interior nodes jittered by 0.1 h), 14 points: every value of
    the FP64 and double-float paths."""
    mesh = meshes.curved_box("Tetrahedron", 8, 1, jitter=0.1, amplitude=0.0)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    pts, w = tg.refcell.collapsed_rule("Tetrahedron", (7, 2, 1))
    ps = tg.PointSet("Tetrahedron", pts, w)
    cells = np.arange(mesh.blocks[0].num_cells)
    want, absx = oracle_at(mesh, g, 0, pts, cells)
    tol = tolerances(mesh.blocks[0], pts, absx, g.origin, want["j"], 3, 3, 8)
    for prec in ("native", "df64"):
        check(tg.geometric_factors_block(g, 0, ps, FACTORS, precision=prec), want, cells, tol)


def test_p2_box_full_size(cuda):
    """1,572,864 curved P2 tetrahedra, 24 points: FP64 and double-float at the f64 tolerance (and
    the double-float path within 5e-13 unscaled), split precision within its bound, an f32 mesh at
    the f32 tolerance."""
    mesh = meshes.curved_box("Tetrahedron", 64, 2, jitter=0.02, seed=2026)
    pts, w = tg.refcell.collapsed_rule("Tetrahedron", (4, 3, 2))
    ps = tg.PointSet("Tetrahedron", pts, w)
    cells = sample_cells(mesh.blocks[0].num_cells)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    want, absx = oracle_at(mesh, g, 0, pts, cells)
    tol = tolerances(mesh.blocks[0], pts, absx, g.origin, want["j"], 3, 3, 8)
    check(tg.geometric_factors_block(g, 0, ps, FACTORS), want, cells, tol)
    errs = check(tg.geometric_factors_block(g, 0, ps, FACTORS, precision="df64"), want, cells, tol)
    assert max(errs.values()) < 5e-13, errs
    split = tg.geometric_factors_block(g, 0, ps, FACTORS, precision="split")
    check(split, want, cells, dict.fromkeys(FACTORS, SPLIT_VOLUME))
    del g, split
    torch.cuda.empty_cache()
    g32 = tg.Geometry.from_host(mesh, dtype=torch.float32)
    want32, absx32 = oracle_at(mesh, g32, 0, pts, cells)
    tol32 = tolerances(mesh.blocks[0], pts, absx32, g32.origin, want32["j"], 3, 3, 4)
    check(tg.geometric_factors_block(g32, 0, ps, FACTORS), want32, cells, tol32)


def test_hybrid_blocks_full_size(cuda):
    """The hybrid mesh (2,000,000 Q2 hexahedra, 300,000 P2 prisms, 50,000 P3 tetrahedra) evaluated
    by the batched graphs, 16,384 sampled cells per block."""
    mesh = meshes.hybrid_box(2_000_000, 300_000, 50_000)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    rule = tg.QuadRule([tg.PointSet("Hexahedron", *tg.refcell.gauss_rule("Hexahedron", 4)),
                        tg.PointSet("Prism", *tg.refcell.collapsed_rule("Prism", (3, 1, 7))),
                        tg.PointSet("Tetrahedron", *tg.refcell.collapsed_rule("Tetrahedron", (4, 3, 2)))])
    samples, wants, tols = [], [], []
    for b, blk in enumerate(mesh.blocks):
        pts = rule.get(blk.cell).points
        cells = sample_cells(blk.num_cells, 16384, seed=7 + b)
        want, absx = oracle_at(mesh, g, b, pts, cells)
        samples.append(cells)
        wants.append(want)
        tols.append(tolerances(blk, pts, absx, g.origin, want["j"], 3, 3, 8))
    for prec in ("native", "df64", "split"):
        batch = tg.Batch(g, rule, factors=FACTORS, precision=prec)
        batch.launch()
        torch.cuda.synchronize()
        for b in range(len(mesh.blocks)):
            tol = dict.fromkeys(FACTORS, SPLIT_VOLUME) if prec == "split" else tols[b]
            check(batch.fields[b], wants[b], samples[b], tol)
        del batch
        torch.cuda.empty_cache()


def test_sphere_full_size(cuda):
    """4,194,304 degree-4 triangles of the perturbed sphere, 28 points, with normals."""
    mesh = meshes.perturbed_radius(meshes.sphere(9, 4, max_cells=4_194_304), 0.02)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    pts, w = tg.refcell.collapsed_rule("Triangle", (7, 4))
    ps = tg.PointSet("Triangle", pts, w)
    names = ("points", "jacobian", "detj", "pinv", "normals")
    cells = sample_cells(mesh.blocks[0].num_cells)
    want, absx = oracle_at(mesh, g, 0, pts, cells, factors=("x", "j", "detj", "k", "normals"))
    tol = tolerances(mesh.blocks[0], pts, absx, g.origin, want["j"], 2, 3, 8)
    for prec in ("native", "df64", "split"):
        fields = tg.geometric_factors_block(g, 0, ps, names, precision=prec)
        check(fields, want, cells, dict.fromkeys(names, SPLIT_SPHERE) if prec == "split" else tol)
        del fields
        torch.cuda.empty_cache()


def test_q2_adjoint_full_size(cuda):
    """128^3 Q2 hexahedra, 27 points, seeded standard-normal cotangents on det J and K: the FP64
    adjoint's node cotangents against the oracle's (every node, 1e-12 relative), the double-float
    forward + split adjoint's within 1e-5 (its FP32 contributions), the double-float forward
    fields against the oracle on 65,536 sampled cells, and central differences (step 1e-6) of the
    FP64 functional at 1,000 seeded nodes."""
    mesh = meshes.curved_box("Hexahedron", 128, 2, jitter=0.02, seed=2026)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    pts, w = tg.refcell.gauss_rule("Hexahedron", 4)
    ps = tg.PointSet("Hexahedron", pts, w)
    nc, nq = mesh.blocks[0].num_cells, len(ps)
    gen = torch.Generator(device="cuda").manual_seed(2026)
    ct64 = {}
    for name, length in (("detj", 1), ("pinv", 9)):
        f = tg.QuadField.uninit(nc, nq, length, 16, torch.float64)
        f.chunks[0].data.normal_(generator=gen)
        ct64[name] = f
    grad64, _ = tg.vjp_block(g, 0, ps, ct64)
    host = {k: v.to_host_cell_major() for k, v in ct64.items()}
    absx = g.nodes.cpu().numpy() + np.array(g.origin[:3])
    want = orc.vjp("Hexahedron", 2, absx, mesh.blocks[0].cells, pts, None, host["detj"][..., 0], host["pinv"])
    g64 = grad64.cpu().numpy()
    assert orc.rel_err(g64, want) < 1e-12
    ct32 = {k: tg.QuadField([tg.geometry.QuadChunk(0, nc, v.chunks[0].data.float())], nc, nq, v.length, 16)
            for k, v in ct64.items()}
    del host
    batch = tg.AdjointBatch(g, tg.QuadRule([ps]), [ct32], precision="df64", forward=FACTORS)
    batch.launch()
    torch.cuda.synchronize()
    assert orc.rel_err(batch.grad.cpu().numpy(), g64) < 1e-5
    cells = sample_cells(nc)
    fwd, absx_s = oracle_at(mesh, g, 0, pts, cells)
    tol = tolerances(mesh.blocks[0], pts, absx_s, g.origin, fwd["j"], 3, 3, 8)
    check(batch.fields[0], fwd, cells, tol)
    del batch
    torch.cuda.empty_cache()
    sample = np.random.default_rng(2026).choice(mesh.num_nodes, 1000, replace=False)
    hostc = {k: v.to_host_cell_major() for k, v in ct64.items()}
    fd = tg.fd_check(g, 0, ps, {"detj": hostc["detj"][..., 0], "pinv": hostc["pinv"]}, g64, sample)
    assert fd["max_rel_err"] < 1e-4, fd
