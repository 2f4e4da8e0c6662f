"""Copies the reference's own refcell golden fixtures into this directory.

The reference (tetraloma, https://github.com/tbetcke/gridcl) checks its reference cells and
Lagrange node layouts against tables exported from ndelement (commit recorded in the source
file ``tetraloma-refcell/tests/fixtures/sources.json``). Those JSON files are data, not code;
this script copies the two that pin the geometry path, unchanged, so that the tests here can
run without the reference checkout:

- ``tetraloma-refcell/tests/fixtures/tables.json`` -> ``refcell_tables.json``
  (vertices, sub-entities and sub-entity types of the eight reference cells);
- ``tetraloma-refcell/tests/fixtures/lagrange_points.json`` -> ``lagrange_points.json``
  (Lagrange nodes, p = 1..4, equispaced and GLL).

Run from the repository root: ``python tests/golden/extract_refcell_fixtures.py [REFERENCE]``.
"""

import json
import pathlib
import sys

REFERENCE = pathlib.Path(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
HERE = pathlib.Path(__file__).resolve().parent
FIXTURES = REFERENCE / "tetraloma-refcell" / "tests" / "fixtures"

for src, dst in (("tables.json", "refcell_tables.json"), ("lagrange_points.json", "lagrange_points.json")):
    data = json.loads((FIXTURES / src).read_text())
    (HERE / dst).write_text(json.dumps(data, sort_keys=True) + "\n")
    print(f"{FIXTURES / src} -> {HERE / dst}")
sources = json.loads((FIXTURES / "sources.json").read_text())
(HERE / "refcell_sources.json").write_text(json.dumps(sources, indent=1, sort_keys=True) + "\n")
