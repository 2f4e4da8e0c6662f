"""ctypes binding of the in-tree CUDA library ``libtlgeom.so`` (the C ABI of
``include/tlgeom.h``).

The library is the only compute path: if it is missing or cannot be loaded, :func:`lib`
raises, and nothing falls back to host code. Build it with ``python -m gridcl_gb300.build``.
"""

from __future__ import annotations

import ctypes
import pathlib

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "libtlgeom.so"

TLG_OK = 0
STATUS_NAMES = {
    1: "InvalidArgument",
    2: "LengthMismatch",
    3: "TooLarge",
    4: "Unsupported",
    5: "Server",
    6: "DeviceTimeout",
    7: "AllocationTooLarge",
}

CELL_IDS = {"Point": 0, "Interval": 1, "Triangle": 2, "Quadrilateral": 3, "Tetrahedron": 4,
            "Hexahedron": 5, "Prism": 6, "Pyramid": 7}
FAMILY_IDS = {"Equispaced": 0, "Gll": 1}


class GridError(RuntimeError):
    """A failed call into the library; mirrors tetraloma-device's ``GridError``
    (tetraloma-device/src/error.rs:80-105). ``kind`` is the variant name."""

    def __init__(self, status: int, message: str):
        self.status = status
        self.kind = STATUS_NAMES.get(status, f"Status{status}")
        super().__init__(f"{self.kind}: {message}")


class TlgBlock(ctypes.Structure):
    _fields_ = [
        ("dtype", ctypes.c_int),
        ("gdim", ctypes.c_int),
        ("num_cells", ctypes.c_int64),
        ("num_nodes", ctypes.c_int64),
        ("nodes", ctypes.c_void_p),
        ("dofmap", ctypes.c_void_p),
        ("flags", ctypes.c_void_p),
        ("num_flags", ctypes.c_int64),
        ("origin", ctypes.c_double * 3),
    ]


class TlgOutputs(ctypes.Structure):
    _fields_ = [
        ("first_cell", ctypes.c_int64),
        ("num_cells", ctypes.c_int64),
        ("out_first_cell", ctypes.c_int64),
        ("tile", ctypes.c_int),
        ("points", ctypes.c_void_p),
        ("jacobian", ctypes.c_void_p),
        ("detj", ctypes.c_void_p),
        ("pinv", ctypes.c_void_p),
        ("normals", ctypes.c_void_p),
        ("facet_normals", ctypes.c_void_p),
        ("cond_limit", ctypes.c_double),
        ("recomputed", ctypes.c_void_p),
        ("weights", ctypes.c_void_p),
        ("cell_measure", ctypes.c_void_p),
    ]


class TlgCotangents(ctypes.Structure):
    _fields_ = [("points", ctypes.c_void_p), ("detj", ctypes.c_void_p), ("pinv", ctypes.c_void_p),
                ("normals", ctypes.c_void_p)]


# (name, restype, argtypes) of every entry point declared in include/tlgeom.h.
_P = ctypes.c_void_p
_I = ctypes.c_int
_L = ctypes.c_int64
SIGNATURES = [
    ("tlg_last_error", ctypes.c_char_p, []),
    ("tlg_abi_version", _I, []),
    ("tlg_num_lagrange_nodes", _L, [_I, _I]),
    ("tlg_lagrange_points", _I, [_I, _I, _I, _P, _L]),
    ("tlg_collapsed_rule", _I, [_I, _P, _P, _P, _L, _P]),
    ("tlg_tabulate", _I, [_I, _I, _I, _P, _L, _I, _P, _L]),
    ("tlg_reference_facet_normals", _I, [_I, _P, _L]),
    ("tlg_tables_create", _I, [_I, _I, _I, _I, _I, _P, _L, _P, _P]),
    ("tlg_tables_destroy", _I, [_P]),
    ("tlg_tables_num_points", _L, [_P]),
    ("tlg_tables_device_status", _I, [_P, _P]),
    ("tlg_tables_nodes_per_cell", _L, [_P]),
    ("tlg_tables_set_wait", _I, [_P, _L, _I]),
    ("tlg_eval_block", _I, [_P, ctypes.POINTER(TlgBlock), ctypes.POINTER(TlgOutputs), _P]),
    ("tlg_batch_create", _I, [_P, ctypes.POINTER(TlgBlock), ctypes.POINTER(TlgOutputs), _I, _P]),
    ("tlg_batch_destroy", _I, [_P]),
    ("tlg_batch_tune", _I, [_P, _P, _P]),
    ("tlg_batch_tuning", _I, [_P, _P, _P, _P]),
    ("tlg_batch_launch", _I, [_P, _P]),
    ("tlg_evector", _I, [ctypes.POINTER(TlgBlock), _I, _L, _L, _L, _P, _P]),
    ("tlg_csr_workspace_bytes", _L, [_L, _I]),
    ("tlg_csr_build", _I, [_P, _L, _I, _L, _P, _L, _P, _P, _P]),
    ("tlg_vjp_block", _I, [_P, ctypes.POINTER(TlgBlock), ctypes.POINTER(TlgOutputs),
                           ctypes.POINTER(TlgCotangents), _P, _L, _P]),
    ("tlg_vjp_gather", _I, [_P, _P, _L, _I, _P, _I, _P, _P]),
    ("tlg_measure_workspace_bytes", _L, [_I, _L]),
    ("tlg_measure", _I, [_P, _I, _L, _L, _I, _P, _P, _L, _P, _P]),
    ("tlg_vjp_gather_add", _I, [_P, _P, _L, _I, _P, _I, _P, _P]),
    ("tlg_vjp_batch_create", _I, [_P, ctypes.POINTER(TlgBlock), ctypes.POINTER(TlgOutputs),
                                  ctypes.POINTER(TlgCotangents), _P, _P, _P, _P, _L, _I, _P, _I, _P]),
    ("tlg_vjp_batch_set_forward", _I, [_P, _P]),
    ("tlg_vjp_batch_set_two_pass", _I, [_P, _I]),
    ("tlg_vjp_block_from_fields", _I, [_P, ctypes.POINTER(TlgBlock), ctypes.POINTER(TlgOutputs), ctypes.POINTER(TlgCotangents), _P, _L, _P]),
    ("tlg_vjp_batch_launch", _I, [_P, _P]),
    ("tlg_vjp_batch_destroy", _I, [_P]),
    ("tlg_measure_cell_sums", _I, [_P, _I, _L, _L, _I, _P, _P, _P]),
    ("tlg_sum_workspace_bytes", _L, [_I, _L]),
    ("tlg_sum", _I, [_P, _I, _L, _P, _L, _P, _P]),
    ("tlg_measure_static", _I, [_P, _I, _L, _L, _I, _P, _P, _P]),
    ("tlg_measure_static_max_cells", _L, []),
    ("tlg_selftest_conversions", _I, [_P, _L, _P, _P]),
    ("tlg_set_strategy", _I, [_I]),
    ("tlg_set_family_strategy", _I, [_I, _I]),
    ("tlg_get_family_override", _I, [_I]),
    ("tlg_get_family_strategy", _I, [_I, ctypes.POINTER(ctypes.c_int)]),
    ("tlg_get_strategy", _I, []),
    ("tlg_last_kernel_family", _I, []),
    ("tlg_last_launch_family", _I, []),
    ("tlg_order_cells", _I, [_I, _I, _P, _L, _I, _P, _L, _I, _P]),
    ("tlg_number_nodes", _I, [_P, _L, _I, _L, _P, _P]),
    ("tlg_hilbert_key", ctypes.c_uint64, [_P, _I, _I]),
    ("tlg_quantise", ctypes.c_uint32, [ctypes.c_double, ctypes.c_double, ctypes.c_double]),
    ("tlg_basis_create", _I, [_I, _I, _I, _P]),
    ("tlg_basis_destroy", _I, [_P]),
    ("tlg_pull_back_block", _I, [_P, ctypes.POINTER(TlgBlock), _P, _L, _L, _L, _L, _I, _I,
                                 ctypes.c_double, _I, _I, _P, _P, _P]),
]

_lib = None


def lib():
    """The loaded library; raises if it was not built (no host fallback exists)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: the CUDA path is the only implementation; build it with "
                "`python -m gridcl_gb300.build`")
        handle = ctypes.CDLL(str(LIB_PATH))
        for name, res, args in SIGNATURES:
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


def check(status: int) -> None:
    if status != TLG_OK:
        msg = lib().tlg_last_error().decode(errors="replace")
        raise GridError(status, msg)
