"""Build recipes for the CPU oracle and the reference's own C writer (test
infrastructure only).

``build()`` compiles ``oracle/fe_oracle.cpp`` into
``oracle/_build/libfe_oracle.so`` with plain ``g++``.  FP contraction is
switched off so the oracle gives the same bits on x86-64 and aarch64 hosts.
The reference's assembly path (Fortran 2003 + MPI + PETSc) cannot be compiled
on these machines.

``build_ref()`` compiles the one part of the reference that is plain C -- its
exnode/exelem writer ``src/FieldExport.c`` (stdio only) -- from the reference
tree, unchanged, into ``oracle/_ref/libfieldexport.so``, when the reference
tree is present (it is not on machines that only run the library); the field
export tests compare the library's writer with it.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "fe_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libfe_oracle.so")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
           SRC, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


REF_SRC = "/root/reference/src"
REF_DIR = os.path.join(HERE, "_ref")
REF_LIB = os.path.join(REF_DIR, "libfieldexport.so")


def build_ref(force: bool = False):
    """The reference's FieldExport.c as a shared library; None when the
    reference tree is absent."""
    src = os.path.join(REF_SRC, "FieldExport.c")
    if not os.path.exists(src):
        return None
    os.makedirs(REF_DIR, exist_ok=True)
    if not force and os.path.exists(REF_LIB) and os.path.getmtime(REF_LIB) >= os.path.getmtime(src):
        return REF_LIB
    tmp = REF_LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-w", "-I", REF_SRC, src, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, REF_LIB)
    return REF_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
