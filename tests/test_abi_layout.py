"""The ctypes structures of the Python binding have the memory layout of the
C structures in include/cm_fe.h (sizes and field offsets, as the C compiler
lays them out).  CPU only: compiles a small C program with the host compiler."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

from cm_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = {
    "fe_mesh_desc": _lib.FEMeshDesc,
    "fe_newton_options": _lib.FENewtonOptions,
    "fe_newton_report": _lib.FENewtonReport,
}


def _c_layout(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "cm_fe.h"', "int main(void) {"]
    for name, cls in STRUCTS.items():
        lines.append('  printf("%s sizeof %%zu\\n", sizeof(%s));' % (name, name))
        for field, _ in cls._fields_:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (name, field, name, field))
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {tuple(l.split()[:2]): int(l.split()[2]) for l in out.splitlines()}


def test_ctypes_structures_match_the_c_header(tmp_path):
    layout = _c_layout(tmp_path)
    for name, cls in STRUCTS.items():
        assert layout[(name, "sizeof")] == C.sizeof(cls), name
        for field, _ in cls._fields_:
            assert layout[(name, field)] == getattr(cls, field).offset, (name, field)
