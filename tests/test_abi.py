"""The C-ABI library loads on a CPU-only host and exports every entry point the header
declares; argument checks run before any device call (CPU)."""

import ctypes
import pathlib
import re

import numpy as np

from gridcl_gb300 import _lib
from gridcl_gb300._lib import TlgBlock, TlgOutputs, lib

HEADER = pathlib.Path(__file__).resolve().parents[1] / "include" / "tlgeom.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(tlg_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported():
    names = declared_functions()
    assert len(names) >= 14
    handle = ctypes.CDLL(str(_lib.LIB_PATH))
    for n in names:
        assert hasattr(handle, n), n
    assert sorted(n for n, _, _ in _lib.SIGNATURES) == names


def test_abi_version():
    assert lib().tlg_abi_version() == 1


def test_argument_errors_before_device_work():
    L = lib()
    assert L.tlg_eval_block(None, None, None, None) == 1
    assert L.tlg_tables_set_wait(None, 16, 0) == 1
    assert L.tlg_vjp_batch_set_forward(None, None) == 1
    b = TlgBlock()
    o = TlgOutputs()
    assert L.tlg_evector(ctypes.byref(b), 4, 0, 0, 16, None, None) == 1
    h = ctypes.c_void_p()
    pts = np.zeros((1, 3))
    p = pts.ctypes.data_as(ctypes.c_void_p)
    # gdim below tdim, unknown dtype, GLL nodes on pyramids, degree 0: all rejected on the host
    assert L.tlg_tables_create(4, 1, 0, 2, 8, p, 1, None, ctypes.byref(h)) == 1
    assert L.tlg_tables_create(4, 1, 0, 3, 2, p, 1, None, ctypes.byref(h)) == 1
    assert L.tlg_tables_create(7, 2, 1, 3, 8, p, 1, None, ctypes.byref(h)) == 1
    assert L.tlg_tables_create(4, 0, 0, 3, 8, p, 1, None, ctypes.byref(h)) == 1
    assert b"degree" in L.tlg_last_error()
    assert h.value is None
    del o


def test_refcell_entry_points_report_capacity():
    L = lib()
    out = np.zeros(3)
    assert L.tlg_lagrange_points(4, 2, 0, out.ctypes.data_as(ctypes.c_void_p), 3) == 2
    assert L.tlg_num_lagrange_nodes(4, 2) == 10
    assert L.tlg_num_lagrange_nodes(99, 2) == -1


def tree_elems(n: int) -> int:
    total = 0
    while n > 1:
        n = (n + 63) // 64
        total += n
    return total


def test_measure_workspace_sizes_and_checks_on_the_host():
    """tlg_measure's workspace: the tree over ceil(n / 64) level-1 sums (none at one level-1 value);
    too small a workspace and bad arguments are refused before any device work."""
    L = lib()
    for n in (0, 1, 64, 65, 4096, 4097, 1_572_864, 16_777_217):
        l1 = (n + 63) // 64
        want = (l1 + tree_elems(l1)) if l1 > 1 else 0
        assert L.tlg_measure_workspace_bytes(4, n) == 4 * want, n
        assert L.tlg_measure_workspace_bytes(8, n) == 8 * want, n
    assert L.tlg_measure_workspace_bytes(2, 10) == -1
    assert L.tlg_measure_workspace_bytes(4, -1) == -1
    assert L.tlg_measure_workspace_bytes(4, 1_572_864) == 99_868
    host = np.zeros(16)  # stands in for device pointers: nothing is dereferenced on these paths
    p = host.ctypes.data_as(ctypes.c_void_p)
    need = L.tlg_measure_workspace_bytes(4, 10_000)
    assert L.tlg_measure(p, 4, 10_000, 24, 16, p, p, need - 1, p, None) == 2
    assert b"needed" in L.tlg_last_error()
    assert L.tlg_measure(p, 4, 10_000, 24, 32, p, p, need, p, None) == 1  # tile 32
    assert L.tlg_measure(p, 3, 10_000, 24, 16, p, p, need, p, None) == 1  # dtype
    assert L.tlg_measure(None, 4, 10_000, 24, 16, p, p, need, p, None) == 1
    assert L.tlg_measure(p, 4, 10_000, 24, 16, p, p, need, None, None) == 1
