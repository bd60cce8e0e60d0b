"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``oracle/fe_oracle.cpp`` into ``oracle/_build/libfe_oracle.so`` with
plain ``g++``.  FP contraction is switched off so the oracle gives the same
bits on x86-64 and aarch64 hosts.  The reference itself (Fortran 2003 + MPI +
PETSc) cannot be compiled on these machines, so there is no ``oracle/_ref``.
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


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
