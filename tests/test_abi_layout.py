"""The ctypes mirrors of the C-ABI structs (convector_gb300/__init__.py) have
the sizes and field offsets of the C header: a C program compiled against
include/convector_gpu.h prints them, so a field added on one side only fails
here instead of corrupting calls. The Rust FFI stub of INTEGRATION.md binds
every function of the header, and its structs have the header's fields."""

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


def _header_text():
    import re
    with open(os.path.join(INCLUDE, "convector_gpu.h")) as f:
        return re.sub(r"/\*.*?\*/", "", f.read(), flags=re.S)


def _integration_text():
    with open(os.path.join(os.path.dirname(INCLUDE), "INTEGRATION.md")) as f:
        return f.read()


def test_rust_stub_binds_every_entry_point():
    """The Rust FFI stub in INTEGRATION.md declares each function of the
    header, and nothing else."""
    import re
    hdr = set(re.findall(r"\b(cvx_\w+)\s*\(", _header_text()))
    stub = set(re.findall(r"\bfn (cvx_\w+)\s*\(", _integration_text()))
    assert hdr - stub == set(), sorted(hdr - stub)
    assert stub - hdr == set(), sorted(stub - hdr)


def test_rust_stub_structs_follow_the_header():
    """Each #[repr(C)] struct of the stub has the C struct's fields, by name
    and in order."""
    import re
    c_structs = {}
    for m in re.finditer(r"typedef struct (\w+) \{(.*?)\} \1;", _header_text(), flags=re.S):
        names = []
        for decl in m.group(2).split(";"):
            decl = decl.strip()
            if decl:
                names += [re.sub(r"\[.*?\]", "", n).strip().lstrip("*") for n in decl.split(None, 1)[1].split(",")]
        c_structs[m.group(1)] = names
    rust = {}
    for m in re.finditer(r"#\[repr\(C\)\] pub struct (\w+) \{(.*?)\}", _integration_text(), flags=re.S):
        rust[m.group(1)] = re.findall(r"pub (\w+):", m.group(2))
    pairs = {"CvxTriangle": "cvx_triangle", "CvxBvhNode": "cvx_bvh_node", "CvxCamera": "cvx_camera",
             "CvxRenderConfig": "cvx_render_config", "CvxView": "cvx_view", "CvxServerConfig": "cvx_server_config",
             "CvxRequest": "cvx_request", "CvxRequestResult": "cvx_request_result"}
    assert set(rust) == set(pairs), sorted(rust)
    for r_name, c_name in pairs.items():
        assert rust[r_name] == c_structs[c_name], (r_name, rust[r_name], c_structs[c_name])
