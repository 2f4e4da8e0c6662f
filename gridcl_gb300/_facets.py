"""Facet point maps of the reference cells (tetraloma-refcell/src/facet.rs:62-105): a point t
of facet f (dimension fd) maps to v0 + sum_k t_k (v_{k+1} - v0), with v the facet's vertex list
(simplices in order, quadrilaterals in tensor order)."""

from __future__ import annotations

import numpy as np

_VERTS = {
    "Interval": [[0.0], [1.0]],
    "Triangle": [[0, 0], [1, 0], [0, 1]],
    "Quadrilateral": [[0, 0], [1, 0], [0, 1], [1, 1]],
    "Tetrahedron": [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]],
    "Hexahedron": [[v & 1, (v >> 1) & 1, (v >> 2) & 1] for v in range(8)],
    "Prism": [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 0, 1], [0, 1, 1]],
    "Pyramid": [[0, 0, 0], [1, 0, 0], [0, 1, 0], [1, 1, 0], [0, 0, 1]],
}
# Facets (sub-entities of dimension tdim - 1) by sorted vertex lists, lexicographic.
_FACETS = {
    "Interval": [[0], [1]],
    "Triangle": [[0, 1], [0, 2], [1, 2]],
    "Quadrilateral": [[0, 1], [0, 2], [1, 3], [2, 3]],
    "Tetrahedron": [[0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 3]],
    "Hexahedron": [[0, 1, 2, 3], [0, 1, 4, 5], [0, 2, 4, 6], [1, 3, 5, 7], [2, 3, 6, 7], [4, 5, 6, 7]],
    "Prism": [[0, 1, 2], [0, 1, 3, 4], [0, 2, 3, 5], [1, 2, 4, 5], [3, 4, 5]],
    "Pyramid": [[0, 1, 2, 3], [0, 1, 4], [0, 2, 4], [1, 3, 4], [2, 3, 4]],
}


def facet_types(cell: str) -> list:
    out = []
    for f in _FACETS[cell]:
        n = len(f)
        out.append({1: "Point", 2: "Interval", 3: "Triangle", 4: "Quadrilateral"}[n])
    return out


def facet_points_to_cell(cell: str, facet: int, points) -> np.ndarray:
    verts = np.asarray(_VERTS[cell], dtype=np.float64)
    lst = _FACETS[cell][facet]
    fd = {1: 0, 2: 1, 3: 2, 4: 2}[len(lst)]
    v0 = verts[lst[0]]
    if fd == 0:
        return v0[None, :].copy()
    t = np.asarray(points, dtype=np.float64).reshape(-1, fd)
    axes = np.stack([verts[lst[k + 1]] - v0 for k in range(fd)])  # [fd][td]
    return v0[None, :] + t @ axes
