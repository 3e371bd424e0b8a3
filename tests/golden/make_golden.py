"""Regenerate ``embedded_tetra.json`` from the reference's own end-to-end test.

The reference (liblaf/apple) cannot be imported here (Warp and JAX are not
installed), so this script reads its test file as text and extracts the
geometry, boundary conditions and expected answer of
``tests/forward/test_static_simulation.py`` (mesh 16-55, boundary values
69-76, assertions 85-93).  Run it only where the reference tree is present:

    python tests/golden/make_golden.py <path-to-liblaf-apple>

or with ``APPLE_REFERENCE_ROOT`` set.

Nothing at test time reads the reference tree; tests read the JSON.
"""

from __future__ import annotations

import ast
import json
import os
import pathlib
import re
import sys

HERE = pathlib.Path(__file__).resolve().parent


def _array_literal(src: str, name: str) -> list:
    """First ``name = np.array(<literal>, ...)`` in ``src``."""
    m = re.search(rf"{name}\s*=\s*np\.array\(\s*(\[.*?\])\s*,\s*dtype", src, re.S)
    if m is None:
        raise ValueError(f"no literal array {name!r}")
    return ast.literal_eval(m.group(1))


def main(ref_root: str) -> None:
    path = pathlib.Path(ref_root) / "tests/forward/test_static_simulation.py"
    src = path.read_text()
    points = _array_literal(src, "points")
    flat = _array_literal(src, "cells")
    cells = [flat[i + 1 : i + 1 + flat[i]] for i in range(0, len(flat), flat[0] + 1)]
    fixed_rows = int(re.search(r"fixed_mask\[:(\d+), :\] = True", src).group(1))
    m = re.search(r"fixed_value\[(\d+)\] = np\.array\((\[.*?\])\)", src)
    fixed_vertex, fixed_disp = int(m.group(1)), ast.literal_eval(m.group(2))
    m = re.search(r"assert_allclose\(u_full\[(\d+)\], (\[.*?\]), atol=([0-9.e-]+)\)", src)
    expect_vertex, expect_u, atol = int(m.group(1)), ast.literal_eval(m.group(2)), float(m.group(3))
    n_free = int(re.search(r"model\.n_free == (\d+)", src).group(1))
    out = {
        "source": "tests/forward/test_static_simulation.py:16-93 (liblaf/apple)",
        "material": "Arap",
        "mu": 1.0,
        "points": points,
        "cells": cells,
        "fixed_vertices": list(range(fixed_rows)),
        "fixed_value_vertex": fixed_vertex,
        "fixed_value": fixed_disp,
        "expect_vertex": expect_vertex,
        "expect_u": expect_u,
        "atol": atol,
        "n_free": n_free,
        "result": "PRIMARY_SUCCESS",
    }
    (HERE / "embedded_tetra.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("APPLE_REFERENCE_ROOT")
    if not root:
        raise SystemExit("usage: make_golden.py <path-to-liblaf-apple> (or set APPLE_REFERENCE_ROOT)")
    main(root)
