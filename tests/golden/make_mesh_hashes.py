"""Generates tests/golden/mesh_hashes.json: the SHA-256 of every array of the
grids the host builder makes at icos levels 0-6 ("eqs" and "pol").

The fixture pins the builder's numbering and geometry bit for bit, so that a
rewrite of its loops (parallel topology, the GPU geometry) can be checked
against the builder as it stood when the fixture was made.  It is a
regression guard, not a reference result: the reference numbers nodes in
STRIPACK's order (see include/imodel_mesh.h).

Run from the repository root:  python tests/golden/make_mesh_hashes.py
"""
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from imodel_gb300 import _build, mesh  # noqa: E402
from imodel_gb300.mesh import meshbuild  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
LEVELS = range(0, 7)


def array_names():
    """Every array a Grid carries (the step's fields and the extras)."""
    return list(mesh._I32) + list(mesh._F64) + list(mesh._EXTRA_F64) + list(mesh._EXTRA_I32)


def grid_hashes(g) -> dict:
    """SHA-256 of each array of a Grid, in its native dtype and layout."""
    out = {}
    for name in sorted(array_names()):
        a = np.ascontiguousarray(getattr(g, name))
        out[name] = hashlib.sha256(a.tobytes()).hexdigest()
    out["delaunay_count"] = int(g.delaunay_violations)
    return out


def main():
    _build.build_mesh_lib()
    table = {}
    for pos in ("eqs", "pol"):
        for level in LEVELS:
            table[f"{pos}{level}"] = grid_hashes(meshbuild(level, pos, nthreads=1))
    with open(os.path.join(HERE, "mesh_hashes.json"), "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    print("wrote", len(table), "grids")


if __name__ == "__main__":
    main()
