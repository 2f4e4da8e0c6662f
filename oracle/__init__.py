"""Oracle: test infrastructure only.

A CPU restatement of the reference's host f64 evaluation of the geometry path (C, with
OpenMP) and of its reference-cell tables (numpy). It is the checker of the CUDA path and the
timed CPU baseline. Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import it; the product (``gridcl_gb300``) never does.

Parity is pinned: the reference-cell tables and Lagrange node layouts are checked against the
reference's own golden fixtures (``tests/golden/``), and the factor math against the
reference's known-answer tests (unit volume, J = I/2, K = 2I, K J = I, constant det J on affine
cells, quadrature weights summing to the cell volume).
"""
