"""Evaluation strategies (tetraloma-geometry/src/strategy.rs:23-34, 373-407): which kernel family
evaluates a block. Precedence as in the reference: a scoped setting (:func:`with_strategy`),
then the environment variable ``TLG_GEOM_STRATEGY``, then the built-in policy ("auto": sum
factorisation for quadrilaterals, hexahedra and prisms at tensor-product rules in f64 and above
the degrees with paired kernels, else the paired or unrolled kernels where compiled, the
cooperative kernel above 27 nodes per cell, loops otherwise). "loops" reads the tables from
global memory, "shared" stages them in shared memory, "cooperative" splits each cell's node
sums over four lanes."""

from __future__ import annotations

import contextlib

from ._lib import check, lib

STRATEGIES = {"auto": 0, "direct": 1, "loops": 2, "sumfact": 3, "shared": 4, "cooperative": 5}
_NAMES = {v: k for k, v in STRATEGIES.items()}
_stack: list = []


def set_strategy(name: str | None) -> None:
    """Overrides the strategy for the process; None returns to the environment and the policy."""
    check(lib().tlg_set_strategy(-1 if name is None else STRATEGIES[name]))


def get_strategy() -> str:
    """The strategy in effect."""
    return _NAMES[lib().tlg_get_strategy()]


def last_kernel_family() -> str | None:
    """The kernel family of this thread's last evaluation launch ("direct", "loops", "sumfact",
    "shared", "cooperative")."""
    return _NAMES.get(lib().tlg_last_kernel_family()) if lib().tlg_last_kernel_family() else None


@contextlib.contextmanager
def with_strategy(name: str):
    """Scoped override (the reference's ``with_strategy`` test hook, testing.rs:34-43)."""
    _stack.append(name)
    set_strategy(name)
    try:
        yield
    finally:
        _stack.pop()
        set_strategy(_stack[-1] if _stack else None)
