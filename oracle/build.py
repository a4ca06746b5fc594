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
# Timing variant for the CPU baseline: plain running sums, compiled with the
# reference's own optimisation flags (-Ofast, CMakeLists.txt:13).  Never
# used as a checker.
LIB_FAST = OUT / "libgdc_oracle_fast.so"


def _compile(out: Path, flags: list[str], force: bool) -> None:
    newest = max(SRC.stat().st_mtime, (HERE / "gdc_oracle.h").stat().st_mtime)
    if force or not out.exists() or out.stat().st_mtime < newest:
        cmd = ["gcc", *flags, "-std=c99", "-fPIC", "-shared", "-o", str(out), str(SRC), "-lm"]
        subprocess.run(cmd, check=True)


def build(force: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    _compile(LIB, ["-O2", "-ffp-contract=off", "-fno-fast-math"], force)
    _compile(LIB_FAST, ["-Ofast", "-DGDO_PLAIN_SUMS"], force)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
