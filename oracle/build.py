"""Build recipe for the parity oracle (test infrastructure only).

Compiles gdc_oracle.c with gcc into oracle/_build/libgdc_oracle.so at -O2
with FMA contraction and fast-math disabled, so that the C evaluation order
is the order written in the source (which follows the reference's).  The
reference (Fortran 2003) itself cannot be compiled here: no Fortran compiler
exists on either machine, and its datetime/container submodules and NetCDF
are absent.
"""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
SRC = HERE / "gdc_oracle.c"
LIB = OUT / "libgdc_oracle.so"


def build(force: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    if force or not LIB.exists() or LIB.stat().st_mtime < max(SRC.stat().st_mtime,
                                                               (HERE / "gdc_oracle.h").stat().st_mtime):
        cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-std=c99", "-fPIC", "-shared",
               "-o", str(LIB), str(SRC), "-lm"]
        subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
