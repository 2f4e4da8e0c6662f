"""The allocation-free measure entry point against the allocating one (GPU).

`tlg_measure_static` serves callers that cannot call cudaMalloc: programs whose device memory
belongs to another allocator (a caching allocator, or a pool that reserves the free memory up
front), where an extra allocation can fail and a free synchronises the device. It keeps its
sum-tree levels in a fixed array inside the library. This file is collected last so that a run
that stops at the first failure has already run every other test; it also passes alone in a
fresh process.
"""

import ctypes

import numpy as np
import pytest
import torch

import gridcl_gb300 as tg
from gridcl_gb300 import meshes
from gridcl_gb300._lib import lib
from gridcl_gb300.geometry import current_stream_handle

pytestmark = pytest.mark.gpu


def allocating_measure(detj, es, nq, w, dtype):
    """tlg_measure_cell_sums + tlg_sum with caller-allocated scratch (the existing path)."""
    ch = detj.chunks[0]
    stream = current_stream_handle()
    sums = torch.empty(ch.num_cells, dtype=dtype, device="cuda")
    assert lib().tlg_measure_cell_sums(ch.data.data_ptr(), es, ch.num_cells, nq, detj.tile,
                                       w.data_ptr(), sums.data_ptr(), stream) == 0
    nbytes = int(lib().tlg_sum_workspace_bytes(es, ch.num_cells))
    work = torch.empty(max(nbytes, es), dtype=torch.uint8, device="cuda")
    out = torch.empty(1, dtype=dtype, device="cuda")
    assert lib().tlg_sum(sums.data_ptr(), es, ch.num_cells, work.data_ptr(), nbytes,
                         out.data_ptr(), stream) == 0
    return float(out.item())


@pytest.mark.parametrize("dtype,es,tol", [(torch.float64, 8, 1e-13), (torch.float32, 4, 1e-5)])
@pytest.mark.parametrize("n", [1, 7])
def test_static_measure_matches_the_allocating_measure(cuda, dtype, es, tol, n):
    mesh = meshes.curved_box("Tetrahedron", n, 2, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=dtype)
    pts, w = tg.refcell.gauss_rule("Tetrahedron", 4)
    ps = tg.PointSet("Tetrahedron", pts, w)
    detj = tg.detj_block(g, 0, ps)
    wd = ps.weights_device(dtype)
    want = allocating_measure(detj, es, len(pts), wd, dtype)
    ch = detj.chunks[0]
    result = torch.full((1,), -1.0, dtype=dtype, device="cuda")
    got = []
    for _ in range(2):  # two calls in a row share the fixed scratch
        st = lib().tlg_measure_static(ch.data.data_ptr(), es, ch.num_cells, len(pts), detj.tile,
                                      wd.data_ptr(), result.data_ptr(), current_stream_handle())
        assert st == 0, lib().tlg_last_error()
        got.append(float(result.item()))
    for v in got:
        assert abs(v - want) <= tol * abs(want), (v, want)
        # The same per-cell order and 64-value fold as the allocating path: the same bits.
        assert v == want
    assert got[0] == got[1]


def test_static_measure_rejects_more_cells_than_its_scratch_holds(cuda):
    limit = int(lib().tlg_measure_static_max_cells())
    assert limit == 1 << 24
    result = torch.empty(1, dtype=torch.float64, device="cuda")
    w = torch.ones(1, dtype=torch.float64, device="cuda")
    st = lib().tlg_measure_static(ctypes.c_void_p(result.data_ptr()), 8, limit + 1, 1, 16,
                                  w.data_ptr(), result.data_ptr(), current_stream_handle())
    assert st == 7  # TLG_ERR_ALLOCATION_TOO_LARGE
    assert b"exceed" in lib().tlg_last_error()
