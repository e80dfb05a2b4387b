"""The ctypes mirrors of the C-ABI structs (convector_gb300/__init__.py) have
the sizes and field offsets of the C header: a C program compiled against
include/convector_gpu.h prints them, so a field added on one side only fails
here instead of corrupting calls."""

import ctypes
import os
import shutil
import subprocess

import pytest

import convector_gb300 as cg

INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")

PAIRS = [
    ("cvx_camera", cg._Camera),
    ("cvx_view", cg._View),
    ("cvx_server_config", cg._ServerConfig),
    ("cvx_request", cg._Request),
    ("cvx_request_result", cg._Result),
    ("cvx_render_config", cg.RenderConfig),
]


def test_struct_layouts_match_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "convector_gpu.h"', "int main(void) {"]
    for cname, py in PAIRS:
        lines.append('printf("%s sizeof %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in py._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", INCLUDE, str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = {}
    for line in out.splitlines():
        name, field, value = line.split()
        got[(name, field)] = int(value)
    for cname, py in PAIRS:
        assert got[(cname, "sizeof")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
