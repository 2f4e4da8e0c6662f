"""Per-cell measure summed by the evaluation (tlg_outputs::cell_measure) against the per-cell sums
the measure takes over the det J field it wrote (measure.rs:15-41): the same bits for the paired
kernels that sum as they evaluate, for every other strategy (a launch after the evaluation), for
ranges of several chunks and for points recomputed in FP64 (GPU)."""

import numpy as np
import pytest
import torch

import gridcl_gb300 as tg
from gridcl_gb300 import meshes
from gridcl_gb300._lib import check, lib
from gridcl_gb300.geometry import current_stream_handle

pytestmark = pytest.mark.gpu


def sums_over(detj: tg.QuadField, weights: torch.Tensor, num_cells: int) -> torch.Tensor:
    """tlg_measure_cell_sums over each chunk of a det J field: the reference's per-cell sums."""
    es = detj.chunks[0].data.element_size()
    out = torch.empty(num_cells, dtype=detj.chunks[0].data.dtype, device="cuda")
    for ch in detj.chunks:
        check(lib().tlg_measure_cell_sums(ch.data.data_ptr(), es, ch.num_cells, detj.num_points, detj.tile,
                                          weights.data_ptr(), out.data_ptr() + ch.first_cell * es,
                                          current_stream_handle()))
    return out


def rule(cell, degree):
    pts, w = tg.refcell.gauss_rule(cell, degree)
    return tg.PointSet(cell, pts, w)


CASES = [("Tetrahedron", 12, 2, 4, "split"), ("Tetrahedron", 12, 2, 4, "native32"),
         ("Tetrahedron", 8, 2, 4, "native64"), ("Tetrahedron", 6, 3, 6, "split"),
         ("Hexahedron", 8, 2, 4, "split"), ("Prism", 6, 2, 4, "split"), ("Tetrahedron", 10, 1, 3, "split")]


@pytest.mark.parametrize("cell,n,degree,rdeg,mode", CASES)
@pytest.mark.parametrize("strategy", ["auto", "direct", "loops", "shared", "sumfact", "cooperative", "tensor"])
def test_cell_measure_equals_sums_over_the_field(cuda, cell, n, degree, rdeg, mode, strategy):
    mesh = meshes.curved_box(cell, n, degree, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=torch.float32 if mode == "native32" else torch.float64)
    ps = rule(cell, rdeg)
    precision = "split" if mode == "split" else "native"
    dt = torch.float64 if mode == "native64" else torch.float32
    nc = g.blocks[0].num_cells
    cm = torch.full((nc,), float("nan"), dtype=dt, device="cuda")
    with tg.with_strategy(strategy):
        f = tg.geometric_factors_block(g, 0, ps, ("points", "jacobian", "detj", "pinv"), precision=precision,
                                       cell_measure=cm)
    want = sums_over(f["detj"], ps.weights_device(dt, "cuda"), nc)
    assert torch.equal(cm, want)
    assert tg.measure_block(g, 0, ps, cell_sums=cm) == tg.measure_block(g, 0, ps, detj=f["detj"])


def test_cell_measure_of_chunked_fields(cuda):
    mesh = meshes.curved_box("Tetrahedron", 10, 2, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    ps = rule("Tetrahedron", 4)
    nc = g.blocks[0].num_cells
    one = torch.empty(nc, dtype=torch.float32, device="cuda")
    tg.geometric_factors_block(g, 0, ps, ("detj",), precision="split", cell_measure=one)
    many = torch.full((nc,), float("nan"), dtype=torch.float32, device="cuda")
    f = tg.geometric_factors_block(g, 0, ps, ("detj", "pinv"), precision="split", max_chunk_cells=1000,
                                   cell_measure=many)
    assert len(f["detj"].chunks) > 1
    assert torch.equal(one, many)


def test_cell_measure_reads_back_recomputed_points(cuda):
    """A sliver tetrahedron's points are recomputed in FP64 after the FP32 pass: its cell measure
    sums the det J values as stored, not the FP32 ones."""
    nodes = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.3, 0.3, 1e-6],
                      [0.0, 0.0, 1.0]]) + 100.0
    cells = np.array([[0, 1, 2, 3], [0, 1, 2, 4]], dtype=np.uint32)
    mesh = meshes.HostMesh(3, nodes, [meshes.HostBlock("Tetrahedron", 1, cells)])
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    ps = rule("Tetrahedron", 2)
    count = torch.zeros(1, dtype=torch.int64, device="cuda")
    cm = torch.empty(2, dtype=torch.float32, device="cuda")
    f = tg.geometric_factors_block(g, 0, ps, ("detj", "pinv"), precision="split", recomputed=count,
                                   cell_measure=cm)
    assert int(count.item()) == len(ps)
    assert torch.equal(cm, sums_over(f["detj"], ps.weights_device(torch.float32, "cuda"), 2))
    assert abs(cm[0].item() - 1e-6 / 6) < 1e-12


def test_cell_measure_in_a_batch(cuda):
    """Batches carry cell_measure into their graph branches: a hybrid mesh (sum-factorised
    hexahedra and prisms, paired tetrahedra) in one launch, each block's sums as its own
    evaluation writes them."""
    mesh = meshes.hybrid_box(4, 4, 4)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    qrule = tg.QuadRule.for_grid(g, 4)
    batch = tg.Batch(g, qrule, factors=("jacobian", "detj"), precision="split", cell_measure=True)
    batch.tune()
    batch.launch()
    total = 0.0
    for b, blk in enumerate(g.blocks):
        ps = qrule.get(blk.element.cell)
        want = sums_over(batch.fields[b]["detj"], ps.weights_device(torch.float32, "cuda"), blk.num_cells)
        assert torch.equal(batch.cell_measure[b][: blk.num_cells], want), blk.element.cell
        total += tg.measure_block(g, b, ps, detj=batch.fields[b]["detj"])
    assert batch.measure() == total


def test_cell_measure_needs_det_j_and_weights(cuda):
    mesh = meshes.curved_box("Tetrahedron", 4, 2, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    ps = rule("Tetrahedron", 4)
    nc = g.blocks[0].num_cells
    with pytest.raises(tg.GridError):
        tg.geometric_factors_block(g, 0, ps, ("pinv",), precision="split",
                                   cell_measure=torch.empty(nc, dtype=torch.float32, device="cuda"))
    with pytest.raises(tg.GridError):
        tg.geometric_factors_block(g, 0, ps, ("detj",), precision="split",
                                   cell_measure=torch.empty(nc, dtype=torch.float64, device="cuda"))
    for bad in (torch.empty(nc - 1, dtype=torch.float32, device="cuda"), torch.empty(nc, dtype=torch.float32),
                torch.empty(nc, dtype=torch.int32, device="cuda")):
        with pytest.raises(tg.GridError):
            tg.measure_block(g, 0, ps, cell_sums=bad)
    f = tg.geometric_factors_block(g, 0, ps, ("detj",), precision="split")
    tables = ps.tables(g.blocks[0].element, 3, tg.geometry.SPLIT32)
    o = tg._lib.TlgOutputs()
    o.first_cell, o.num_cells, o.out_first_cell, o.tile = 0, nc, 0, 16
    o.detj = f["detj"].chunks[0].data.data_ptr()
    cm = torch.empty(nc, dtype=torch.float32, device="cuda")
    o.cell_measure = cm.data_ptr()  # no weights
    import ctypes
    desc = g.block_desc(0)
    with pytest.raises(tg.GridError):
        check(lib().tlg_eval_block(tables.handle, ctypes.byref(desc), ctypes.byref(o), current_stream_handle()))
