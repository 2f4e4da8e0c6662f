"""Oracle, test infrastructure only: Python front end of the C restatement (``oracle.c``) and
the numpy refcell restatement (``refcell.py``).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may
import this module, and only as the checker or as the timed CPU baseline; the product never
calls it.

- :func:`eval_block` is ``tetraloma-testing/src/reference.rs`` (``points``, ``jacobians``,
  ``detj``, ``pseudo_inverses``, ``normals``, ``facet_normals``): the stored node L-vector
  widened to f64 plus the origin, gathered through the dofmap, contracted with the f64
  tabulation.
- :func:`evector` is the E-vector gather of ``tetraloma-geometry/src/evector.rs:195-236``.
- :func:`pull_back` is the Newton pull-back of ``tetraloma-geometry/src/pull_back.rs:102-194``.
- :func:`untile` is ``QuadField::to_host_cell_major`` (``tetraloma-geometry/src/field.rs:380-408``).
- :func:`rel_err` and the tolerance scales restate ``reference.rs:579-817``.
"""

from __future__ import annotations

import ctypes
import os
import pathlib
import subprocess

import numpy as np

from . import refcell

HERE = pathlib.Path(__file__).resolve().parent
LIB = HERE / "_build" / "liborc.so"

TOL_F32 = 1e-5  # tetraloma-testing/src/lib.rs:127-130
TOL_F64 = 1e-12

_lib = None


def build() -> pathlib.Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def load():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        lib = ctypes.CDLL(str(LIB))
        p = ctypes.c_void_p
        lib.orc_eval.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_int64, p, ctypes.c_int64, p, p, p, p,
                                 p, p, p, p, p, p, ctypes.c_int]
        lib.orc_eval.restype = ctypes.c_int
        lib.orc_evector.argtypes = [p, ctypes.c_int64, ctypes.c_int, p, ctypes.c_int64,
                                    ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_int64,
                                    ctypes.c_int64, p]
        lib.orc_evector.restype = ctypes.c_int
        lib.orc_measure.argtypes = [p, p, ctypes.c_int64, ctypes.c_int]
        lib.orc_measure.restype = ctypes.c_double
        lib.orc_max_threads.restype = ctypes.c_int
        lib.orc_vjp.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int64, p,
                                ctypes.c_int64, p, p, p, p, p, p]
        lib.orc_vjp.restype = ctypes.c_int
        lib.orc_vjp2.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int64, p,
                                 ctypes.c_int64, p, p, p, ctypes.c_int64, p, p, p, p, p]
        lib.orc_vjp2.restype = ctypes.c_int
        _lib = lib
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def max_threads() -> int:
    return load().orc_max_threads()


FACTORS = ("x", "j", "detj", "k", "normals", "facet_normals")


def eval_block(cell: str, degree: int, nodes_abs: np.ndarray, dofmap: np.ndarray,
               points: np.ndarray, factors=("x", "j", "detj", "k"), flags=None,
               ref_normals=None, family: str = "Equispaced", tab=None, nthreads: int = 0):
    """The requested factors of one block, cell-major ``[cell][q][component]`` in f64.

    ``nodes_abs`` are absolute coordinates ``[node][gdim]`` (stored L-vector + origin, widened
    to f64), ``dofmap`` ``[cell][K]`` node indices, ``points`` ``[q][tdim]``.
    """
    td = refcell.tdim(cell)
    nodes_abs = np.ascontiguousarray(nodes_abs, dtype=np.float64)
    gd = nodes_abs.shape[1]
    dofmap = np.ascontiguousarray(dofmap, dtype=np.uint32)
    ncells, k = dofmap.shape
    points = np.asarray(points, dtype=np.float64).reshape(-1, td)
    nq = points.shape[0]
    if tab is None:
        tab = refcell.tabulate(cell, degree, points, 1, family)
    tab = np.ascontiguousarray(tab, dtype=np.float64)
    assert tab.shape == (1 + td, nq, k), tab.shape
    out = {}
    lens = {"x": gd, "j": td * gd, "detj": 1, "k": td * gd, "normals": gd, "facet_normals": gd}
    for f in factors:
        out[f] = np.empty((ncells, nq, lens[f]), dtype=np.float64)
    if flags is not None:
        flags = np.ascontiguousarray(flags, dtype=np.uint32)
    if ref_normals is not None:
        ref_normals = np.ascontiguousarray(ref_normals, dtype=np.float64)
    rc = load().orc_eval(td, gd, k, nq, ncells, _ptr(nodes_abs), nodes_abs.shape[0],
                         _ptr(dofmap), _ptr(tab), _ptr(flags), _ptr(ref_normals),
                         *[_ptr(out.get(f)) for f in FACTORS], nthreads)
    if rc != 0:
        raise ValueError(f"orc_eval rejected its arguments ({rc})")
    return out


def vjp(cell: str, degree: int, nodes_abs: np.ndarray, dofmap: np.ndarray, points: np.ndarray,
        xbar=None, dbar=None, kbar=None, family: str = "Equispaced", tab=None, nbar=None,
        flags=None) -> np.ndarray:
    """Node cotangents ``[node][gdim]`` (f64) of sum(xbar . x + dbar det J + kbar : K + nbar . n)
    over a block (det J the area element and n the unit normal, sign flipped by bit 0 of `flags`,
    below codimension 0); cotangents cell-major ``[cell][q][...]`` or None."""
    td = refcell.tdim(cell)
    nodes_abs = np.ascontiguousarray(nodes_abs, dtype=np.float64)
    dofmap = np.ascontiguousarray(dofmap, dtype=np.uint32)
    ncells, k = dofmap.shape
    points = np.asarray(points, dtype=np.float64).reshape(-1, td)
    if tab is None:
        tab = refcell.tabulate(cell, degree, points, 1, family)
    tab = np.ascontiguousarray(tab, dtype=np.float64)
    conv = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)
    xbar, dbar, kbar, nbar = conv(xbar), conv(dbar), conv(kbar), conv(nbar)
    fl = None if flags is None else np.ascontiguousarray(flags, dtype=np.uint32)
    grad = np.zeros_like(nodes_abs)
    gd = nodes_abs.shape[1]
    rc = load().orc_vjp2(td, gd, k, points.shape[0], ncells, _ptr(nodes_abs), nodes_abs.shape[0],
                         _ptr(dofmap), _ptr(tab), _ptr(fl), 0 if fl is None else fl.shape[0], _ptr(xbar),
                         _ptr(dbar), _ptr(kbar), _ptr(nbar), _ptr(grad))
    if rc != 0:
        raise ValueError(f"orc_vjp2 rejected its arguments ({rc})")
    return grad


CENTROID = {"Interval": (0.5,), "Triangle": (1 / 3, 1 / 3), "Quadrilateral": (0.5, 0.5),
            "Tetrahedron": (0.25, 0.25, 0.25), "Hexahedron": (0.5, 0.5, 0.5), "Prism": (1 / 3, 1 / 3, 0.5),
            "Pyramid": (0.4, 0.4, 0.2)}


def pull_back(cell: str, degree: int, nodes_abs: np.ndarray, dofmap: np.ndarray, x_abs: np.ndarray,
              tolerance: float = 1e-13, max_iterations: int = 16, family: str = "Equispaced"):
    """Reference points ``[cell][q][TD]`` and last steps ``[cell][q]`` of the physical points
    ``x_abs [cell][q][GD]`` (tetraloma-geometry/src/pull_back.rs:102-194, 566): from the vertex
    centroid rounded to f32, `max_iterations` Newton steps delta = K (y - X) with K the
    pseudo-inverse of J, iterates clamped to [-0.1, 1.1] (bounds rounded to f32), |delta|_inf
    recorded (the largest finite value when not finite), points frozen once it is at most the
    tolerance. f64, the basis from the restated tabulation at the iterates."""
    td = refcell.tdim(cell)
    nodes_abs = np.asarray(nodes_abs, dtype=np.float64)
    dofmap = np.asarray(dofmap, dtype=np.int64)
    xc = nodes_abs[np.minimum(dofmap, nodes_abs.shape[0] - 1)]  # [cell][K][GD]
    y = np.asarray(x_abs, dtype=np.float64)
    nc, nq, gd = y.shape
    big = np.finfo(np.float64).max
    lo, hi = float(np.float32(-0.1)), float(np.float32(1.1))
    start = np.array([float(np.float32(c)) for c in CENTROID[cell]])
    p = np.broadcast_to(start, (nc, nq, td)).copy()
    last = np.full((nc, nq), big)
    frozen = np.zeros((nc, nq), dtype=bool)
    for _ in range(max_iterations):
        tab = refcell.tabulate(cell, degree, p.reshape(-1, td), 1, family)
        k = tab.shape[2]
        phi = tab[0].reshape(nc, nq, k)
        dphi = tab[1:].reshape(td, nc, nq, k)
        X = np.einsum("cqk,ckg->cqg", phi, xc)
        J = np.einsum("dcqk,ckg->cqgd", dphi, xc)  # J[g][d]
        with np.errstate(all="ignore"):
            K = np.linalg.pinv(J)  # [c][q][d][g]
            delta = np.einsum("cqdg,cqg->cqd", K, y - X)
            m = np.abs(delta)
            bad = ~np.all(m <= big, axis=2)
            s_ = np.where(bad, big, np.max(np.where(np.isfinite(m), m, 0.0), axis=2))
            q_ = p + delta
            q_ = np.where(q_ < lo, lo, q_)
            q_ = np.where(q_ > hi, hi, q_)
        move = ~frozen
        p = np.where(move[..., None], q_, p)
        last = np.where(move, s_, last)
        frozen = frozen | (move & (s_ <= tolerance))
    return p, last


def evector(nodes_stored: np.ndarray, dofmap: np.ndarray, num_cells: int, k: int, gd: int,
            first_cell: int, padded: int, stride: int) -> np.ndarray:
    """One E-vector chunk ``[k][g][stride]`` gathered byte for byte from the stored nodes."""
    nodes_stored = np.ascontiguousarray(nodes_stored)
    dofmap = np.ascontiguousarray(dofmap, dtype=np.uint32)
    out = np.zeros(k * gd * stride, dtype=nodes_stored.dtype)
    rc = load().orc_evector(_ptr(nodes_stored), nodes_stored.size // gd, nodes_stored.itemsize,
                            _ptr(dofmap), num_cells, k, gd, first_cell, padded, stride, _ptr(out))
    if rc != 0:
        raise ValueError(f"orc_evector rejected its arguments ({rc})")
    return out.reshape(k, gd, stride)


def measure(detj: np.ndarray, weights: np.ndarray) -> float:
    detj = np.ascontiguousarray(detj, dtype=np.float64).reshape(detj.shape[0], -1)
    weights = np.ascontiguousarray(weights, dtype=np.float64)
    return load().orc_measure(_ptr(detj), _ptr(weights), detj.shape[0], detj.shape[1])


def untile(tiled: np.ndarray, num_cells: int, num_points: int, length: int, tile: int):
    """``QuadField::to_host_cell_major``: (c, q, k) at ((c / tile) Q LEN + q LEN + k) tile + c % tile."""
    ntiles = -(-num_cells // tile)
    a = np.asarray(tiled)[: ntiles * num_points * length * tile]
    a = a.reshape(ntiles, num_points, length, tile).transpose(0, 3, 1, 2)
    return a.reshape(ntiles * tile, num_points, length)[:num_cells]


def rel_err(got, want) -> float:
    """max |got - want| / max |want| over a quantity (reference.rs:805-817)."""
    got = np.asarray(got, dtype=np.float64).ravel()
    want = np.asarray(want, dtype=np.float64).ravel()
    assert got.shape == want.shape, (got.shape, want.shape)
    if not (np.all(np.isfinite(got)) and np.all(np.isfinite(want))):
        return float("inf")
    scale = np.abs(want).max(initial=0.0)
    err = np.abs(got - want).max(initial=0.0)
    return float(err / scale) if scale > 0 else float(err)


# ------------------------------------------------------------------------------------------
# Tolerance scales (reference.rs:496-774).

def reference_degree(cell: str) -> int:
    return 3 if cell == "Pyramid" else 4


def amplification(cell, degree, family, points, kind):
    e = refcell.LagrangeElement(cell, degree, family)
    if kind == "values":
        t = e.tabulate(points, 0)[0]
        return np.abs(t).sum(axis=1)
    t = e.tabulate(points, 1)
    return np.abs(t[1:]).sum(axis=2).max(axis=0)


def tolerance_scale(cell, degree, family, points, kind="derivatives") -> float:
    a = amplification(cell, degree, family, points, kind).max()
    a_ref = amplification(cell, reference_degree(cell), "Equispaced", points, kind).max()
    return max(a / a_ref, 1.0)


def node_ratio(cell, degree) -> float:
    n = refcell.num_lagrange_nodes(cell, degree)
    return max(n / refcell.num_lagrange_nodes(cell, reference_degree(cell)), 1.0)


def origin_ratio(coords_abs, origin, j) -> float:
    jmax = np.abs(j).max(initial=0.0)
    if jmax <= 0:
        return 1.0
    off = np.abs(np.asarray(coords_abs) - np.asarray(origin)).max(initial=0.0)
    return max(off / jmax, 1.0)


def condition_scale(j: np.ndarray, td: int, gd: int) -> float:
    """max over points of kappa_F(J) / TD, at least 1 (reference.rs:237-242,624-639)."""
    jj = j.reshape(-1, td, gd)  # [point][d][g]: column d is J(:, d)
    jm = np.transpose(jj, (0, 2, 1))  # [point][g][d]
    pinv = np.linalg.pinv(jm)
    kap = np.linalg.norm(jm, axis=(1, 2)) * np.linalg.norm(pinv, axis=(1, 2)) / td
    return float(max(kap.max(initial=1.0), 1.0))


def tolerance(dtype_bytes: int, scale: float) -> float:
    assert np.isfinite(scale)
    return scale * (TOL_F32 if dtype_bytes == 4 else TOL_F64)
