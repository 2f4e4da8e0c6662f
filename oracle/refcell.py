"""Oracle, test infrastructure only: a numpy restatement of tetraloma-refcell.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may
import this module, and only as the checker. The product computes its own tables in
``gridcl_gb300/csrc/refcell.cpp``; the two are written independently so that each checks the
other.

What is restated, and from where (paths inside the reference project):

- reference cells and sub-entity numbering: ``tetraloma-refcell/src/cell.rs:23-190``
  (pinned by ``tests/golden/refcell_tables.json``, exported from ndelement);
- Lagrange node layout, vertices, edges, faces, interior, each entity along its own vertex
  list: ``tetraloma-refcell/src/lagrange.rs:163-266`` (pinned by
  ``tests/golden/lagrange_points.json``, p = 1..4, equispaced and GLL);
- Gauss-Jacobi rules on [0, 1] with weight (1 - x)^alpha, combined into collapsed tensor rules
  with the first direction fastest: ``tetraloma-refcell/src/quadrature.rs:77-159``. The nodes
  come here from the Golub-Welsch eigenvalue method, not from the reference's Newton
  iteration, so the two constructions check each other;
- the Lagrange basis: the reference expands it in an orthonormal set and inverts the
  generalised Vandermonde matrix (``tetraloma-refcell/src/tabulation.rs:1-5,266``). The
  Lagrange functions of a node set are unique, so this module builds them directly, without a
  matrix inverse: products of 1D Lagrange polynomials on intervals, quadrilaterals and
  hexahedra, the classical equispaced barycentric products on triangles and tetrahedra, and
  their product on prisms. This is exact up to rounding at every degree.
- pyramids: the Lagrange space is rational (``tetraloma-refcell/src/polynomials/pyramid.rs:1-17``,
  spanned by x^a y^b z^c / (1 - z)^min(a,b) with a + c <= p and b + c <= p, the set of
  ``tabulation.rs:418-460``). There is no product form, so this module expands the Lagrange
  functions in the centred rationomials u^a v^b w^c / s^min(a,b), s = 1 - z, u = 2x - s,
  v = 2y - s, w = 2z - 1 (the same space: x^a = ((u + s) / 2)^a, and the powers of s and w
  are polynomials in z of no higher degree), where the reference uses an orthonormal set, and
  inverts their Vandermonde matrix at the equispaced nodes exactly, in rational arithmetic.
  At the apex (s = 0) every value and first derivative is its limit along the pyramid's axis
  u = v = 0, as the reference returns there (``pyramid.rs:12-16``).
"""

from __future__ import annotations

import fractions
import functools
import math

import numpy as np

CELLS = ("Point", "Interval", "Triangle", "Quadrilateral", "Tetrahedron", "Hexahedron",
         "Prism", "Pyramid")

_TDIM = {"Point": 0, "Interval": 1, "Triangle": 2, "Quadrilateral": 2, "Tetrahedron": 3,
         "Hexahedron": 3, "Prism": 3, "Pyramid": 3}

# tetraloma-refcell/src/cell.rs:39-75 (table A.1).
_VERTICES = {
    "Point": [[]],
    "Interval": [[0.0], [1.0]],
    "Triangle": [[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]],
    "Quadrilateral": [[0.0, 0.0], [1.0, 0.0], [0.0, 1.0], [1.0, 1.0]],
    "Tetrahedron": [[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]],
    "Hexahedron": [[float(v & 1), float((v >> 1) & 1), float((v >> 2) & 1)] for v in range(8)],
    "Prism": [[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0],
              [0.0, 0.0, 1.0], [1.0, 0.0, 1.0], [0.0, 1.0, 1.0]],
    "Pyramid": [[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [1.0, 1.0, 0.0],
                [0.0, 0.0, 1.0]],
}

# tetraloma-refcell/src/cell.rs:86-160 (tables A.2, A.3): sub-entities of each dimension by
# their sorted vertex lists, in lexicographic order. The edge and face sets are stated here;
# the order follows from sorting.
_EDGES = {
    "Interval": [(0, 1)],
    "Triangle": [(0, 1), (0, 2), (1, 2)],
    "Quadrilateral": [(0, 1), (0, 2), (1, 3), (2, 3)],
    "Tetrahedron": [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)],
    "Hexahedron": [(a, b) for a in range(8) for b in range(a + 1, 8)
                   if bin(a ^ b).count("1") == 1],
    "Prism": [(0, 1), (0, 2), (1, 2), (3, 4), (3, 5), (4, 5), (0, 3), (1, 4), (2, 5)],
    "Pyramid": [(0, 1), (0, 2), (1, 3), (2, 3), (0, 4), (1, 4), (2, 4), (3, 4)],
}
_FACES = {
    "Triangle": [(0, 1, 2)],
    "Quadrilateral": [(0, 1, 2, 3)],
    "Tetrahedron": [(0, 1, 2), (0, 1, 3), (0, 2, 3), (1, 2, 3)],
    # Each face of the cube fixes one coordinate bit.
    "Hexahedron": [tuple(v for v in range(8) if ((v >> axis) & 1) == side)
                   for axis in range(3) for side in range(2)],
    "Prism": [(0, 1, 2), (3, 4, 5), (0, 1, 3, 4), (0, 2, 3, 5), (1, 2, 4, 5)],
    "Pyramid": [(0, 1, 2, 3), (0, 1, 4), (0, 2, 4), (1, 3, 4), (2, 3, 4)],
}


def tdim(cell: str) -> int:
    return _TDIM[cell]


def vertices(cell: str) -> np.ndarray:
    return np.array(_VERTICES[cell], dtype=np.float64).reshape(len(_VERTICES[cell]), tdim(cell))


def sub_entities(cell: str, dim: int) -> list[list[int]]:
    td = tdim(cell)
    nv = len(_VERTICES[cell])
    if dim == 0:
        return [[v] for v in range(nv)]
    if dim > td:
        return []
    if dim == td:
        return [list(range(nv))]
    table = _EDGES if dim == 1 else _FACES
    return sorted(sorted(e) for e in table[cell])


def _entity_type(cell: str, entity: list[int], dim: int) -> str:
    if dim == 0:
        return "Point"
    if dim == 1:
        return "Interval"
    if dim == tdim(cell):
        return cell
    return "Triangle" if len(entity) == 3 else "Quadrilateral"


def sub_entity_types(cell: str, dim: int) -> list[str]:
    return [_entity_type(cell, e, dim) for e in sub_entities(cell, dim)]


def num_lagrange_nodes(cell: str, p: int) -> int:
    """tetraloma-refcell/src/lagrange.rs:59-78."""
    a, b = p + 1, p + 2
    return {
        "Point": 1,
        "Interval": a,
        "Triangle": a * b // 2,
        "Quadrilateral": a * a,
        "Tetrahedron": a * b * (p + 3) // 6,
        "Hexahedron": a * a * a,
        "Prism": a * a * b // 2,
        "Pyramid": a * b * (2 * p + 3) // 6,
    }[cell]


# ------------------------------------------------------------------------------------------
# Jacobi polynomials and Gauss rules (Golub-Welsch).

def _golub_welsch(m: int, a: float, b: float) -> tuple[np.ndarray, np.ndarray]:
    """Nodes on [-1, 1] and weights for the weight (1 - t)^a (1 + t)^b, m points."""
    n = np.arange(m, dtype=np.float64)
    s = 2.0 * n + a + b
    with np.errstate(divide="ignore", invalid="ignore"):
        diag = np.where(s == 0.0, 0.0, (b * b - a * a) / (s * (s + 2.0)))
    if m > 0 and a + b == 0.0:
        diag[0] = (b - a) / (a + b + 2.0)
    k = np.arange(1, m, dtype=np.float64)
    s1 = 2.0 * k + a + b
    off = np.sqrt(4.0 * k * (k + a) * (k + b) * (k + a + b) / (s1 * s1 * (s1 + 1.0) * (s1 - 1.0)))
    jac = np.diag(diag) + np.diag(off, 1) + np.diag(off, -1)
    t, vecs = np.linalg.eigh(jac)
    mu0 = 2.0 ** (a + b + 1.0) * math.gamma(a + 1.0) * math.gamma(b + 1.0) / math.gamma(a + b + 2.0)
    w = mu0 * vecs[0, :] ** 2
    return t, w


def gauss_jacobi(m: int, alpha: float) -> tuple[np.ndarray, np.ndarray]:
    """m-point Gauss rule on [0, 1] for the weight (1 - x)^alpha, ascending nodes, weights
    summing to 1 / (alpha + 1) (tetraloma-refcell/src/jacobi.rs, `gauss_jacobi`)."""
    t, w = _golub_welsch(m, alpha, 0.0)
    x = 0.5 * (1.0 + t)
    w = w / w.sum() / (alpha + 1.0)
    return x, w


def gll_points(m: int) -> np.ndarray:
    """Gauss-Lobatto-Legendre points on [0, 1]: the ends and the zeros of P'_{m-1}, which are
    the Gauss-Jacobi(1, 1) nodes (tetraloma-refcell/src/jacobi.rs, `gll_points`)."""
    pts = np.zeros(m)
    pts[-1] = 1.0
    if m > 2:
        t, _ = _golub_welsch(m - 2, 1.0, 1.0)
        inner = 0.5 * (1.0 + t)
        # Symmetric by construction, as in the reference.
        inner = 0.5 * (inner + (1.0 - inner[::-1]))
        pts[1:-1] = inner
    if m % 2 == 1:
        pts[m // 2] = 0.5
    return pts


def _tensor(rules, mapping):
    """Collapsed tensor rule, first direction fastest (tetraloma-refcell/src/quadrature.rs:130-159)."""
    grids = np.meshgrid(*[r[0] for r in rules], indexing="ij")
    wgrids = np.meshgrid(*[r[1] for r in rules], indexing="ij")
    # Fortran order: the first index runs fastest.
    coords = np.stack([g.ravel(order="F") for g in grids], axis=1)
    w = np.prod(np.stack([g.ravel(order="F") for g in wgrids], axis=1), axis=1)
    return mapping(coords), w


def gauss_rule(cell: str, degree: int) -> tuple[np.ndarray, np.ndarray]:
    """Gauss rule with m = degree // 2 + 1 points per collapsed direction
    (tetraloma-refcell/src/quadrature.rs:77-128). Points `[q][tdim]`, weights `[q]`."""
    m = degree // 2 + 1
    return collapsed_rule(cell, [m] * max(tdim(cell), 1))


def collapsed_rule(cell: str, counts) -> tuple[np.ndarray, np.ndarray]:
    """The collapsed Gauss-Jacobi product rule of `cell` with `counts[d]` points in direction d
    (the maps of tetraloma-refcell/src/quadrature.rs:83-126; equal counts give `gauss_rule`)."""
    if cell == "Point":
        return np.zeros((1, 0)), np.ones(1)
    g = [gauss_jacobi(m, 0.0) for m in counts]
    j1 = [gauss_jacobi(m, 1.0) for m in counts]
    j2 = [gauss_jacobi(m, 2.0) for m in counts]
    if cell == "Interval":
        return _tensor([g[0]], lambda p: p)
    if cell == "Quadrilateral":
        return _tensor([g[0], g[1]], lambda p: p)
    if cell == "Hexahedron":
        return _tensor([g[0], g[1], g[2]], lambda p: p)
    if cell == "Triangle":
        return _tensor([g[0], j1[1]], lambda p: np.stack([p[:, 0] * (1.0 - p[:, 1]), p[:, 1]], 1))
    if cell == "Tetrahedron":
        def tet(p):
            s = 1.0 - p[:, 2]
            return np.stack([p[:, 0] * (1.0 - p[:, 1]) * s, p[:, 1] * s, p[:, 2]], 1)
        return _tensor([g[0], j1[1], j2[2]], tet)
    if cell == "Prism":
        return _tensor([g[0], j1[1], g[2]],
                       lambda p: np.stack([p[:, 0] * (1.0 - p[:, 1]), p[:, 1], p[:, 2]], 1))
    if cell == "Pyramid":
        def pyr(p):
            s = 1.0 - p[:, 2]
            return np.stack([p[:, 0] * s, p[:, 1] * s, p[:, 2]], 1)
        return _tensor([g[0], g[1], j2[2]], pyr)
    raise ValueError(cell)


# ------------------------------------------------------------------------------------------
# Lagrange nodes.

def _interior_line(p: int, family: str, cell: str) -> np.ndarray:
    if family == "Equispaced":
        return np.arange(1, p) / p
    if family == "Gll":
        if cell not in ("Interval", "Quadrilateral", "Hexahedron"):
            raise ValueError(f"GLL nodes are not defined on {cell}")
        return gll_points(p + 1)[1:p]
    raise ValueError(family)


def lagrange_points(cell: str, p: int, family: str = "Equispaced") -> np.ndarray:
    """Nodes `[k][tdim]` in the reference order: vertices, edges, faces, interior; inside each
    entity along that entity's vertex list (tetraloma-refcell/src/lagrange.rs:163-266)."""
    if p < 1:
        raise ValueError("degree 0 has no Lagrange layout")
    line = _interior_line(p, family, cell)
    td = tdim(cell)
    verts = vertices(cell)
    out: list[np.ndarray] = []

    def push(v, t, axes):
        x = v[0].copy()
        for tk, a in zip(t, axes):
            x = x + tk * (v[a] - v[0])
        out.append(x)

    for dim in range(td + 1):
        for ent, etype in zip(sub_entities(cell, dim), sub_entity_types(cell, dim)):
            v = verts[ent]
            if etype == "Point":
                push(v, [], [])
            elif etype == "Interval":
                for t in line:
                    push(v, [t], [1])
            elif etype == "Triangle":
                for i1 in range(1, p):
                    for i0 in range(1, p - i1):
                        push(v, [i0 / p, i1 / p], [1, 2])
            elif etype == "Quadrilateral":
                for t1 in line:
                    for t0 in line:
                        push(v, [t0, t1], [1, 2])
            elif etype == "Tetrahedron":
                for i2 in range(1, p):
                    for i1 in range(1, p - i2):
                        for i0 in range(1, p - i2 - i1):
                            push(v, [i0 / p, i1 / p, i2 / p], [1, 2, 3])
            elif etype == "Hexahedron":
                for t2 in line:
                    for t1 in line:
                        for t0 in line:
                            push(v, [t0, t1, t2], [1, 2, 4])
            elif etype == "Prism":
                for i2 in range(1, p):
                    for i1 in range(1, p):
                        for i0 in range(1, p - i1):
                            push(v, [i0 / p, i1 / p, i2 / p], [1, 2, 3])
            elif etype == "Pyramid":
                for i2 in range(1, max(p - 1, 0)):
                    for i1 in range(1, p - i2):
                        for i0 in range(1, p - i2):
                            out.append(np.array([i0 / p, i1 / p, i2 / p]))
    pts = np.array(out, dtype=np.float64).reshape(len(out), td)
    assert pts.shape[0] == num_lagrange_nodes(cell, p)
    return pts


# ------------------------------------------------------------------------------------------
# Tabulation by explicit Lagrange products (no Vandermonde inversion).

def _line_nodes(p: int, family: str, cell: str) -> np.ndarray:
    return np.concatenate([[0.0], _interior_line(p, family, cell), [1.0]])


def _lagrange_1d(t: np.ndarray, i: int, x: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """The 1D Lagrange polynomial of node t[i] over the nodes t, and its derivative, at x."""
    val = np.ones_like(x)
    der = np.zeros_like(x)
    for j in range(t.size):
        if j == i:
            continue
        f = (x - t[j]) / (t[i] - t[j])
        der = der * f + val / (t[i] - t[j])
        val = val * f
    return val, der


def _simplex_factor(a: int, z: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """s_a(z) = prod_{j<a} (z - j) / (j + 1) and ds/dz: the equispaced simplex factors."""
    val = np.ones_like(z)
    der = np.zeros_like(z)
    for j in range(a):
        f = (z - j) / (j + 1.0)
        der = der * f + val / (j + 1.0)
        val = val * f
    return val, der


def _simplex(td: int, p: int, nodes: np.ndarray, pts: np.ndarray):
    """Equispaced simplex Lagrange functions: psi_alpha = prod_i s_{alpha_i}(p lambda_i), with
    lambda the barycentric coordinates and alpha = p lambda(node)."""
    lam_nodes = np.concatenate([1.0 - nodes.sum(1, keepdims=True), nodes], axis=1)
    alpha = np.rint(p * lam_nodes).astype(int)
    assert np.allclose(alpha, p * lam_nodes, atol=1e-9)
    lam = np.concatenate([1.0 - pts.sum(1, keepdims=True), pts], axis=1)  # [q][td + 1]
    # dlambda_i / dx_d: -1 for i = 0, 1 for i = d + 1.
    dl = np.zeros((td + 1, td))
    dl[0, :] = -1.0
    dl[1:, :] = np.eye(td)
    out = np.zeros((1 + td, pts.shape[0], nodes.shape[0]))
    for k in range(nodes.shape[0]):
        fac = [_simplex_factor(alpha[k, i], p * lam[:, i]) for i in range(td + 1)]
        out[0, :, k] = np.prod([f[0] for f in fac], axis=0)
        for d in range(td):
            acc = np.zeros(pts.shape[0])
            for i in range(td + 1):
                if dl[i, d] == 0.0:
                    continue
                prod = p * dl[i, d] * fac[i][1]
                for m in range(td + 1):
                    if m != i:
                        prod = prod * fac[m][0]
                acc += prod
            out[1 + d, :, k] = acc
    return out


def pyramid_exponents(p: int) -> list[tuple[int, int, int]]:
    """(a, b, c) with a + c <= p and b + c <= p: the exponents of the rationomials
    x^a y^b z^c / (1 - z)^min(a,b) spanning the pyramid's Lagrange space (tabulation.rs:446-460),
    and of the centred ones this module expands in."""
    return [(a, b, c) for c in range(p + 1) for b in range(p + 1 - c) for a in range(p + 1 - c)]


def _centred_exact(e, x) -> fractions.Fraction:
    """u^a v^b w^c / s^r (r = min(a, b)) at a point of exact fractions; 0 at s = 0 when r >= 1
    (there u = v = 0 inside the cell: the limit along the axis)."""
    a, b, c = e
    r = min(a, b)
    s = 1 - x[2]
    if s == 0 and r > 0:
        return fractions.Fraction(0)
    return (2 * x[0] - s) ** a * (2 * x[1] - s) ** b * (2 * x[2] - 1) ** c / s ** r


@functools.lru_cache(maxsize=None)
def pyramid_coefficients(p: int) -> np.ndarray:
    """C [m][k]: the pyramid's Lagrange function k is sum_m C[m][k] f_m, f_m the centred
    rationomials of `pyramid_exponents(p)`; the Vandermonde matrix V[i][m] = f_m(node_i) at the
    equispaced nodes (i0/p, i1/p, i2/p) is inverted exactly (Gauss-Jordan over fractions), then
    rounded."""
    exps = pyramid_exponents(p)
    nodes = [[fractions.Fraction(int(round(v * p)), p) for v in row] for row in lagrange_points("Pyramid", p)]
    n = len(nodes)
    assert len(exps) == n
    a = [[_centred_exact(e, x) for e in exps] + [fractions.Fraction(int(i == j)) for j in range(n)]
         for i, x in enumerate(nodes)]
    for col in range(n):
        piv = next(r for r in range(col, n) if a[r][col] != 0)
        a[col], a[piv] = a[piv], a[col]
        inv = 1 / a[col][col]
        a[col] = [v * inv for v in a[col]]
        for r in range(n):
            if r != col and a[r][col] != 0:
                f = a[r][col]
                a[r] = [v - f * w for v, w in zip(a[r], a[col])]
    return np.array([[float(v) for v in row[n:]] for row in a])


def _centred_terms(e):
    """The value and the three first derivatives of u^a v^b w^c s^-r as lists of terms
    (coefficient, (eu, ev, ew, es)); du = (2, 0, 1), dv = (0, 2, 1), dw = (0, 0, 2), ds = (0, 0, -1)."""
    a, b, c = e
    r = min(a, b)
    out = [[(1.0, (a, b, c, -r))], [], [], []]
    if a:
        out[1].append((2.0 * a, (a - 1, b, c, -r)))
        out[3].append((float(a), (a - 1, b, c, -r)))
    if b:
        out[2].append((2.0 * b, (a, b - 1, c, -r)))
        out[3].append((float(b), (a, b - 1, c, -r)))
    if c:
        out[3].append((2.0 * c, (a, b, c - 1, -r)))
    if r:
        out[3].append((float(r), (a, b, c, -r - 1)))
    return out


def _pyramid(p: int, pts: np.ndarray) -> np.ndarray:
    exps = pyramid_exponents(p)
    coef = pyramid_coefficients(p)
    s = 1.0 - pts[:, 2]
    u, v, w = 2.0 * pts[:, 0] - s, 2.0 * pts[:, 1] - s, 2.0 * pts[:, 2] - 1.0
    apex = s == 0.0
    safe = np.where(apex, 1.0, s)
    f = np.zeros((4, pts.shape[0], len(exps)))
    for m, e in enumerate(exps):
        for d, terms in enumerate(_centred_terms(e)):
            for c, (eu, ev, ew, es) in terms:
                val = c * u ** eu * v ** ev * w ** ew * safe ** es
                # On the axis (u = v = 0) a term with eu = ev = 0 has es = 0: its limit is c w^ew.
                lim = c * w ** ew if eu == 0 and ev == 0 and es == 0 else 0.0
                f[d, :, m] += np.where(apex, lim, val)
    return f @ coef


def tabulate(cell: str, degree: int, points, nderivs: int = 1, family: str = "Equispaced") -> np.ndarray:
    """``[deriv][q][k]``: values (deriv 0) and d/dxi_d (deriv 1 + d) of the Lagrange functions of
    (cell, degree, family) at `points`, like ``Tabulation::get`` (tabulation.rs:266). The
    functions come from explicit Lagrange products: 1D Lagrange polynomials over the node
    coordinates on tensor cells, equispaced barycentric products on simplices, and their
    product on prisms."""
    td = tdim(cell)
    p = degree
    pts = np.asarray(points, dtype=np.float64).reshape(-1, td)
    nodes = lagrange_points(cell, p, family)
    nq, nk = pts.shape[0], nodes.shape[0]
    if cell in ("Triangle", "Tetrahedron"):
        out = _simplex(td, p, nodes, pts)
    elif cell in ("Interval", "Quadrilateral", "Hexahedron"):
        t = _line_nodes(p, family, cell)
        out = np.zeros((1 + td, nq, nk))
        for k in range(nk):
            idx = [int(np.argmin(np.abs(t - nodes[k, d]))) for d in range(td)]
            f = [_lagrange_1d(t, idx[d], pts[:, d]) for d in range(td)]
            out[0, :, k] = np.prod([x[0] for x in f], axis=0)
            for dd in range(td):
                out[1 + dd, :, k] = np.prod([f[d][1] if d == dd else f[d][0] for d in range(td)], axis=0)
    elif cell == "Prism":
        t = _line_nodes(p, family, "Interval")
        tri_nodes = lagrange_points("Triangle", p)
        tri = _simplex(2, p, tri_nodes, pts[:, :2])
        out = np.zeros((4, nq, nk))
        for k in range(nk):
            it = int(np.argmin(np.abs(tri_nodes - nodes[k, :2]).sum(1)))
            iz = int(np.argmin(np.abs(t - nodes[k, 2])))
            fz = _lagrange_1d(t, iz, pts[:, 2])
            out[0, :, k] = tri[0, :, it] * fz[0]
            out[1, :, k] = tri[1, :, it] * fz[0]
            out[2, :, k] = tri[2, :, it] * fz[0]
            out[3, :, k] = tri[0, :, it] * fz[1]
    elif cell == "Pyramid":
        if family != "Equispaced":
            raise ValueError("pyramids have equispaced nodes only")
        out = _pyramid(p, pts)
    else:
        raise NotImplementedError(f"{cell} is not restated by the oracle")
    return out if nderivs else out[:1]


class LagrangeElement:
    """The Lagrange element (cell, degree, family) (tetraloma-refcell/src/tabulation.rs)."""

    def __init__(self, cell: str, degree: int, family: str = "Equispaced"):
        self.cell, self.degree, self.family = cell, degree, family
        self.points = lagrange_points(cell, degree, family)
        self.dim = self.points.shape[0]

    def tabulate(self, points, nderivs: int) -> np.ndarray:
        return tabulate(self.cell, self.degree, points, nderivs, self.family)


def reference_facet_normals(cell: str) -> np.ndarray:
    """Outward unit normals of the reference cell's facets, `[facet][tdim]`
    (tetraloma-refcell/src/facet.rs): for a facet with vertices v0.. the normal of the facet's
    plane, oriented away from the cell centroid."""
    td = tdim(cell)
    verts = vertices(cell)
    centroid = verts.mean(axis=0)
    out = []
    for ent in sub_entities(cell, td - 1):
        v = verts[ent]
        if td == 1:
            n = np.array([1.0])
        elif td == 2:
            e = v[1] - v[0]
            n = np.array([e[1], -e[0]])
        else:
            n = np.cross(v[1] - v[0], v[2] - v[0])
        n = n / np.linalg.norm(n)
        if np.dot(n, v[0] - centroid) < 0:
            n = -n
        out.append(n)
    return np.array(out)
