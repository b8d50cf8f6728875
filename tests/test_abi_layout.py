"""The header's structs as a C compiler lays them out, against the ctypes
mirror in fargocpt_gb300/abi.py (no GPU): a C program built with gcc against
include/fargocpt_gb300.h prints sizeof and offsetof of every field of
fgpu_params, fgpu_body, fgpu_accretor, fgpu_frame_center, fgpu_cfl_cell,
fgpu_tiles and fgpu_clock; each must equal the mirror's.  A field added to
one side and not the other, or a changed type, fails here."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

from fargocpt_gb300 import abi

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = {
    "fgpu_params": abi.FgpuParams,
    "fgpu_body": abi.FgpuBody,
    "fgpu_accretor": abi.FgpuAccretor,
    "fgpu_frame_center": abi.FgpuFrameCenter,
    "fgpu_cfl_cell": abi.FgpuCflCell,
    "fgpu_tiles": abi.FgpuTiles,
    "fgpu_clock": abi.FgpuClock,
}


def test_struct_layouts_match_the_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include "fargocpt_gb300.h"', "#include <stddef.h>", "#include <stdio.h>",
             "int main(void) {"]
    for cname, cls in STRUCTS.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in cls._fields_:
            lines.append(f'  printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", "-Wall", "-I", os.path.join(REPO, "include"), str(src),
                    "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = {}
    for line in out.splitlines():
        cname, field, value = line.split()
        got[(cname, field)] = int(value)
    for cname, cls in STRUCTS.items():
        assert got[(cname, "size")] == C.sizeof(cls), cname
        for field, _ in cls._fields_:
            assert got[(cname, field)] == getattr(cls, field).offset, (cname, field)
