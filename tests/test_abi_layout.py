"""The ctypes structures of the Python view have the C header's layout:
every field's offset and every structure's size, from a small C program
compiled against include/vertexsurge_gb300.h (CPU only)."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import pytest

from vertexsurge_gb300 import _abi

ROOT = Path(__file__).resolve().parent.parent
PAIRS = [("vs_expand_params", _abi.ExpandParams), ("vs_expand_stats", _abi.ExpandStats),
         ("vs_bitmat_info", _abi.BitmatInfo), ("vs_table_ref", _abi.TableRef),
         ("vs_isect_dep", _abi.IsectDep), ("vs_row_block", _abi.RowBlock)]


def test_struct_layouts_match_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "vertexsurge_gb300.h"', "int main(void) {"]
    for cname, py in PAIRS:
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for f in py._fields_:
            lines.append(f'  printf("{cname} {f[0]} %zu\\n", offsetof({cname}, {f[0]}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        name, field, val = line.split()
        got[(name, field)] = int(val)
    for cname, py in PAIRS:
        assert got[(cname, "size")] == C.sizeof(py), cname
        for f in py._fields_:
            assert got[(cname, f[0])] == getattr(py, f[0]).offset, (cname, f[0])
