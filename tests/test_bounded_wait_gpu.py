"""The table copy's bounded wait runs out without a fault (GPU).

Every evaluation kernel stages its tables into shared memory with one bulk copy and waits for it
on an mbarrier with a bounded number of polls. The tables' test hook (tlg_tables_set_wait) leaves
the copy unissued and shortens the wait, so the wait runs out with nothing in flight: the kernel
records the timeout, computes nothing, and the context stays usable for the next launch.
"""

import ctypes

import numpy as np
import pytest
import torch

import gridcl_gb300 as tg
from gridcl_gb300 import meshes
from gridcl_gb300._lib import lib
from oracle import oracle as orc

pytestmark = pytest.mark.gpu

FACTORS = ("points", "jacobian", "detj", "pinv")
DEVICE_TIMEOUT = 6


@pytest.mark.parametrize("precision", ["native", "df64", "split"])
def test_wait_runs_out_and_the_context_stays_usable(cuda, precision):
    mesh = meshes.curved_box("Tetrahedron", 3, 2, jitter=0.02)
    g = tg.Geometry.from_host(mesh, dtype=torch.float64)
    pts, w = tg.refcell.collapsed_rule("Tetrahedron", (4, 3, 2))
    ps = tg.PointSet("Tetrahedron", pts, w)
    code = {"native": torch.float64, "df64": tg.geometry.DF64, "split": tg.geometry.SPLIT32}[precision]
    tables = ps.tables(g.blocks[0].element, 3, code)
    fields = tg.geometric_factors_block(g, 0, ps, FACTORS, precision=precision)
    for f in fields.values():
        f.chunks[0].data.fill_(float("nan"))
    stream = torch.cuda.current_stream().cuda_stream
    assert lib().tlg_tables_set_wait(tables.handle, 16, 0) == 0
    tg.geometric_factors_block(g, 0, ps, FACTORS, precision=precision, out=fields)
    assert lib().tlg_tables_device_status(tables.handle, ctypes.c_void_p(stream)) == DEVICE_TIMEOUT
    # No CTA computed from tables that never arrived.
    for f in fields.values():
        assert torch.isnan(f.chunks[0].data).all()
    # The status was cleared; the default wait evaluates again on the same context.
    assert lib().tlg_tables_set_wait(tables.handle, 0, 1) == 0
    tg.geometric_factors_block(g, 0, ps, FACTORS, precision=precision, out=fields)
    assert lib().tlg_tables_device_status(tables.handle, ctypes.c_void_p(stream)) == 0
    absx = g.nodes.cpu().numpy() + np.array(g.origin[:3])
    want = orc.eval_block("Tetrahedron", 2, absx, mesh.blocks[0].cells, pts)
    tol = 1e-5 if precision == "split" else 1e-11
    for f, o in zip(FACTORS, ("x", "j", "detj", "k")):
        assert orc.rel_err(fields[f].to_host_cell_major(), want[o]) < tol, f
