"""The ctypes mirrors of the C ABI's structs (imodel_gb300/_capi.py) have the
C compiler's layout: every field at the offset the headers in include/ give
it, and the same total size.  A field added to a header without its mirror
(or in another place) shows up here, on the CPU."""
import ctypes
import os
import shutil
import subprocess

import pytest

from imodel_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")

# C struct name -> ctypes mirror
STRUCTS = {
    "imodel_swm_mesh": _capi.Mesh,
    "imodel_mesh_extra": _capi.MeshExtra,
    "imodel_swm_opts": _capi.Opts,
    "imodel_swm_diag": _capi.Diag,
    "imodel_moist_opts": _capi.MoistOpts,
}


def _c_layout(tmp_path):
    """{struct: (sizeof, {field: offsetof})} from the C compiler."""
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "imodel_swm.h"',
             '#include "imodel_mesh.h"', '#include "imodel_moist.h"', "int main(void) {"]
    for cname, mirror in STRUCTS.items():
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for fname, _ in mirror._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", INCLUDE, str(src), "-o", str(exe)], check=True,
                   capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    layout = {}
    for ln in out.splitlines():
        cname, key, val = ln.split()
        size, fields = layout.setdefault(cname, [0, {}])
        if key == "sizeof":
            layout[cname][0] = int(val)
        else:
            fields[key] = int(val)
    return layout


@pytest.mark.skipif(shutil.which("gcc") is None, reason="needs a C compiler")
def test_ctypes_mirrors_match_the_headers(tmp_path):
    layout = _c_layout(tmp_path)
    for cname, mirror in STRUCTS.items():
        size, offsets = layout[cname]
        assert ctypes.sizeof(mirror) == size, (cname, ctypes.sizeof(mirror), size)
        for fname, _ in mirror._fields_:
            assert getattr(mirror, fname).offset == offsets[fname], (cname, fname)
