"""Evaluation strategies (tetraloma-geometry/src/strategy.rs:23-34, 311-407; the test hooks of
tetraloma-geometry/src/testing.rs): which kernel family evaluates a block, per kernel family
(EVector, Points, Jacobian, Normals, FacetNormals, PullBack). Precedence as in the reference:
this thread's scoped setting (:func:`with_strategy`), then the environment variable
``TLG_GEOM_STRATEGY`` (one strategy for every family, or ``Family=strategy,...``), then the
built-in policy ("policy"/"auto": sum factorisation for quadrilaterals, hexahedra and prisms at
tensor-product rules in f64 and above the degrees with paired kernels, else the paired or
unrolled kernels where compiled (the double-float ones for double-float tables), above 27 nodes
per cell the tcgen05 tensor-core kernel for f32 and split volume cells of at most 88 nodes and
the cooperative kernel otherwise, loops otherwise). "loops" reads the tables from global
memory, "shared" stages them in shared memory, "cooperative" splits each cell's node sums over
four lanes, "tensor" (an extension of the reference's five) runs the node-by-basis contraction on
the tensor cores (tcgen05 UMMAs with tensor-memory accumulators for volume cells of 21-88 nodes,
mma.sync 3xTF32 for the others). A forced strategy that does not apply runs "loops", as in the
reference. A fused launch follows its principal family: Jacobian when J, det J or K is among its
outputs, else Normals, FacetNormals, Points."""

from __future__ import annotations

import contextlib
import ctypes
import threading

from ._lib import GridError, check, lib

STRATEGIES = {"auto": 0, "direct": 1, "loops": 2, "sumfact": 3, "shared": 4, "cooperative": 5, "tensor": 6}
_ALIASES = {"policy": 0}
FAMILIES = {"EVector": 0, "Points": 1, "Jacobian": 2, "Normals": 3, "FacetNormals": 4, "PullBack": 5}
_NAMES = {v: k for k, v in STRATEGIES.items()}
_FAMILY_NAMES = {v: k for k, v in FAMILIES.items()}
_local = threading.local()


def _code(name: str | None) -> int:
    if name is None:
        return -1
    code = STRATEGIES.get(name, _ALIASES.get(name))
    if code is None:
        raise GridError(1, f"unknown strategy {name!r}: expected one of {sorted(STRATEGIES)} or 'policy'")
    return code


def _family(family: str) -> int:
    for k, v in FAMILIES.items():
        if k.lower() == family.lower():
            return v
    raise GridError(1, f"unknown kernel family {family!r}: expected one of {list(FAMILIES)}")


def set_strategy(name: str | None, family: str | None = None) -> None:
    """Sets this thread's strategy of `family` (every family when None); None clears it, returning
    to the environment and the policy."""
    if family is None:
        check(lib().tlg_set_strategy(_code(name)))
    else:
        check(lib().tlg_set_family_strategy(_family(family), _code(name)))


def get_strategy(family: str = "Jacobian") -> str:
    """The strategy in effect for `family` (setting, environment, policy)."""
    out = ctypes.c_int(0)
    check(lib().tlg_get_family_strategy(_family(family), ctypes.byref(out)))
    return _NAMES[out.value]


def last_kernel_family() -> str | None:
    """The strategy that ran in this thread's last launch ("direct", "loops", "sumfact",
    "shared", "cooperative", "tensor")."""
    return _NAMES.get(lib().tlg_last_kernel_family()) if lib().tlg_last_kernel_family() else None


def last_launch_family() -> str | None:
    """The kernel family whose strategy decided this thread's last launch."""
    return _FAMILY_NAMES.get(lib().tlg_last_launch_family())


@contextlib.contextmanager
def with_strategy(name: str, family: str | None = None):
    """Scoped override of `family` (every family when None) on this thread, restored on exit (the
    reference's ``with_strategy`` test hook, testing.rs:11-35)."""
    fams = list(FAMILIES.values()) if family is None else [_family(family)]
    saved = [lib().tlg_get_family_override(f) for f in fams]
    code = _code(name)
    for f in fams:
        check(lib().tlg_set_family_strategy(f, code))
    try:
        yield
    finally:
        for f, s in zip(fams, saved):
            check(lib().tlg_set_family_strategy(f, s))


def _note_launch() -> None:
    """Appends this thread's last launch to the innermost active :func:`record_strategies`."""
    stack = getattr(_local, "records", None)
    if stack:
        entry = (last_launch_family(), last_kernel_family())
        for rec in stack:
            rec.append(entry)


@contextlib.contextmanager
def record_strategies():
    """Collects ``(family, strategy)`` of every launch on this thread inside the block, in order
    (the reference's ``record_strategies``, testing.rs:37-43); enclosing recorders see them too."""
    if not hasattr(_local, "records"):
        _local.records = []
    rec: list = []
    _local.records.append(rec)
    try:
        yield rec
    finally:
        _local.records.remove(rec)
