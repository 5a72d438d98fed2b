"""The ctypes mirrors in rusterize_gb300/_lib.py have the layout of the C
structs in include/rusterize_gb300.h: a small C program compiled from the
header prints every size and field offset, and they must equal ctypes'.
CPU only."""

import ctypes
import shutil
import subprocess
from pathlib import Path

import pytest

from rusterize_gb300 import _lib

ROOT = Path(__file__).resolve().parents[1]

STRUCTS = {
    "rz_geoms": _lib.RzGeoms,
    "rz_raster_info": _lib.RzRasterInfo,
    "rz_stats": _lib.RzStats,
    "rz_sparse_view": _lib.RzSparseView,
    "rz_job": _lib.RzJob,
    "rz_batch_stats": _lib.RzBatchStats,
    "rz_tuning": _lib.RzTuning,
}


def test_struct_layouts_match_the_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "rusterize_gb300.h"', "int main(void) {"]
    for cname, cls in STRUCTS.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    exe = tmp_path / "layout"
    src.write_text("\n".join(lines))
    subprocess.run([cc, "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    c = {}
    for line in out:
        if line:
            a, b, v = line.split()
            c[(a, b)] = int(v)
    for cname, cls in STRUCTS.items():
        assert c[(cname, "size")] == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert c[(cname, fname)] == getattr(cls, fname).offset, f"{cname}.{fname}"
