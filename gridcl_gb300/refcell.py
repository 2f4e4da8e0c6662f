"""Reference-cell functions of the product, computed by the native library (host f64):
the Lagrange node layout, collapsed Gauss rules, the Lagrange tabulation and the reference
facet normals (tetraloma-refcell/src/lib.rs:58-69)."""

from __future__ import annotations

import ctypes

import numpy as np

from ._lib import CELL_IDS, FAMILY_IDS, check, lib

TDIM = {"Point": 0, "Interval": 1, "Triangle": 2, "Quadrilateral": 2, "Tetrahedron": 3,
        "Hexahedron": 3, "Prism": 3, "Pyramid": 3}


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def tdim(cell: str) -> int:
    return TDIM[cell]


def num_lagrange_nodes(cell: str, degree: int) -> int:
    n = lib().tlg_num_lagrange_nodes(CELL_IDS[cell], degree)
    if n < 0:
        raise ValueError(f"no Lagrange element ({cell}, {degree})")
    return int(n)


def lagrange_points(cell: str, degree: int, family: str = "Equispaced") -> np.ndarray:
    """Nodes ``[k][tdim]`` in the reference's order (tetraloma-refcell/src/lagrange.rs:163-266)."""
    n = num_lagrange_nodes(cell, degree) if degree >= 1 else 0
    out = np.zeros(max(n * tdim(cell), 1))
    check(lib().tlg_lagrange_points(CELL_IDS[cell], degree, FAMILY_IDS[family], _ptr(out), out.size))
    return out[: n * tdim(cell)].reshape(n, tdim(cell))


def collapsed_rule(cell: str, counts) -> tuple[np.ndarray, np.ndarray]:
    """Collapsed Gauss-Jacobi rule with counts[d] points in direction d; equal counts
    m = degree // 2 + 1 give ``gauss_rule`` (tetraloma-refcell/src/quadrature.rs:77-128)."""
    td = tdim(cell)
    c = np.ascontiguousarray(list(counts) + [1] * (3 - len(counts)), dtype=np.int32)
    cap = int(np.prod(c[:td])) if td else 1
    pts = np.zeros(max(cap * td, 1))
    w = np.zeros(cap)
    nq = ctypes.c_int64(0)
    check(lib().tlg_collapsed_rule(CELL_IDS[cell], _ptr(c), _ptr(pts), _ptr(w), cap,
                                   ctypes.byref(nq)))
    q = nq.value
    return pts[: q * td].reshape(q, td), w[:q]


def gauss_rule(cell: str, degree: int) -> tuple[np.ndarray, np.ndarray]:
    m = degree // 2 + 1
    return collapsed_rule(cell, [m] * tdim(cell))


def tabulate(cell: str, degree: int, points, nderivs: int = 1, family: str = "Equispaced") -> np.ndarray:
    """``[deriv][q][k]`` Lagrange values and reference derivatives (tabulation.rs:266)."""
    td = tdim(cell)
    pts = np.ascontiguousarray(np.asarray(points, dtype=np.float64).reshape(-1, td))
    k = num_lagrange_nodes(cell, degree)
    rows = 1 + (td if nderivs else 0)
    out = np.zeros(max(rows * pts.shape[0] * k, 1))
    check(lib().tlg_tabulate(CELL_IDS[cell], degree, FAMILY_IDS[family], _ptr(pts), pts.shape[0],
                             nderivs, _ptr(out), out.size))
    return out[: rows * pts.shape[0] * k].reshape(rows, pts.shape[0], k)


def reference_facet_normals(cell: str) -> np.ndarray:
    td = tdim(cell)
    out = np.zeros(6 * 3)
    check(lib().tlg_reference_facet_normals(CELL_IDS[cell], _ptr(out), out.size))
    nf = {"Interval": 2, "Triangle": 3, "Quadrilateral": 4, "Tetrahedron": 4, "Hexahedron": 6,
          "Prism": 5, "Pyramid": 5}[cell]
    return out[: nf * td].reshape(nf, td)
