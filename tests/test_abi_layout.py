"""The ctypes mirrors of the C ABI structs (bachelorarbeit-mlem_gb300/__init__.py)
have the size and the field offsets of the structs declared in include/mlem.h:
a probe compiled with gcc against the header prints them."""
from __future__ import annotations

import ctypes as C
import shutil
import subprocess

import pytest

from conftest import ROOT, load_pkg

# ctypes class -> C typedef
PAIRS = {
    "CsrHost": "mlem_csr_host",
    "MatrixOpts": "mlem_matrix_opts",
    "MatrixInfo": "mlem_matrix_info",
    "RunOpts": "mlem_run_opts",
    "Stats": "mlem_stats",
    "Csr4Header": "mlem_csr4_header",
    "Csr4Scanner": "mlem_csr4_scanner",
    "Geometry": "mlem_geometry",
    "BatchOpts": "mlem_batch_opts",
    "ServerOpts": "mlem_server_opts",
    "ServerStats": "mlem_server_stats",
}


def test_struct_layouts_match_the_header(tmp_path):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    pkg = load_pkg()
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "mlem.h"', "int main(void) {"]
    for py, cname in PAIRS.items():
        cls = getattr(pkg, py)
        lines.append(f'printf("{py} %zu\\n", sizeof({cname}));')
        for field, _ in cls._fields_:
            lines.append(f'printf("{py}.{field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "abi.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "abi"
    subprocess.run([gcc, "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True,
                   capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = dict(line.split() for line in out.splitlines())
    for py in PAIRS:
        cls = getattr(pkg, py)
        assert int(got[py]) == C.sizeof(cls), py
        for field, _ in cls._fields_:
            assert int(got[f"{py}.{field}"]) == getattr(cls, field).offset, f"{py}.{field}"
