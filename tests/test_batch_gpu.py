"""Batched evaluation of a hybrid mesh (one CUDA graph launch) against per-block launches (GPU)."""

import numpy as np
import pytest
import torch

import gridcl_gb300 as tg
from gridcl_gb300 import meshes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["native", "split"])
def test_batch_equals_per_block_launches(cuda, precision):
    mesh = meshes.hybrid_box(300, 200, 100)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    rule = tg.QuadRule.for_grid(g, 4)
    batch = tg.Batch(g, rule, precision=precision)
    batch.launch()
    for b in range(len(g.blocks)):
        want = tg.geometric_factors_block(g, b, rule.get(g.blocks[b].element.cell),
                                          precision=precision)
        for k, f in want.items():
            assert torch.equal(batch.fields[b][k].chunks[0].data, f.chunks[0].data), (b, k)
    grids = batch.tune()
    assert len(grids) == 3
    tuning = batch.tuning()
    batch.launch()
    batch.launch()  # graph replay
    # Each block as a launch of its own under the strategy the tuner chose for it.
    for b in range(len(g.blocks)):
        name = tuning["strategies"][b]
        with tg.with_strategy("auto" if name == "caller" else name):
            want = tg.geometric_factors_block(g, b, rule.get(g.blocks[b].element.cell), precision=precision)
        for k, f in want.items():
            assert torch.equal(batch.fields[b][k].chunks[0].data, f.chunks[0].data), (b, k, name)


def test_tuner_keeps_the_callers_strategy(cuda):
    """Under a scoped strategy the tuner times grids only: every block keeps the caller's."""
    mesh = meshes.hybrid_box(200, 100, 50)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    rule = tg.QuadRule.for_grid(g, 4)
    batch = tg.Batch(g, rule, precision="split")
    with tg.with_strategy("loops"):
        batch.tune()
        assert batch.tuning()["strategies"] == ["caller"] * 3
        batch.launch()
        for b in range(len(g.blocks)):
            want = tg.geometric_factors_block(g, b, rule.get(g.blocks[b].element.cell), precision="split")
            for k, f in want.items():
                assert torch.equal(batch.fields[b][k].chunks[0].data, f.chunks[0].data), (b, k)


def test_graph_replay_reads_the_current_nodes(cuda):
    mesh = meshes.hybrid_box(100, 50, 40)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    rule = tg.QuadRule.for_grid(g, 2)
    batch = tg.Batch(g, rule, factors=("detj",))
    batch.launch()
    before = batch.fields[0]["detj"].chunks[0].data.clone()
    g.nodes.mul_(2.0)  # scale the mesh in place: det J grows by 8
    batch.launch()
    after = batch.fields[0]["detj"].chunks[0].data
    assert torch.allclose(after, 8.0 * before, rtol=1e-14, atol=0)
