"""Build recipe for the parity oracle (test infrastructure only).

Compiles gdc_oracle.c and gdc_fftpack.c with gcc into oracle/_build/ at -O2
with FMA contraction and fast-math disabled, so that the C evaluation order
is the order written in the source (which follows the reference's):

* libgdc_oracle.so -- the exact build: correctly rounded sums, the filter as a
  projection onto the kept modes (the CUDA path's arithmetic);
* libgdc_oracle_ref.so -- the reference's order: plain running sums in the
  reference's loop order (-DGDO_PLAIN_SUMS); with gdo_set_fft the filter
  runs FFTPACK's transforms as the reference does;
* libgdc_oracle_fast.so -- the same reference-order arithmetic compiled
  with the reference's own flags (-Ofast, CMakeLists.txt:13): the timed CPU
  baseline, never used to check.

The reference (Fortran 2003) itself cannot be compiled here: no Fortran
compiler exists on either machine, and its datetime/container submodules
and NetCDF are absent.
"""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
SRCS = [HERE / "gdc_oracle.c", HERE / "gdc_fftpack.c", HERE / "gdc_oracle_ic.c"]
HDRS = [HERE / "gdc_oracle.h", HERE / "gdc_fftpack.h"]
LIB = OUT / "libgdc_oracle.so"
LIB_REF = OUT / "libgdc_oracle_ref.so"
LIB_FAST = OUT / "libgdc_oracle_fast.so"
EXACT = ["-O2", "-ffp-contract=off", "-fno-fast-math"]
LIBS = {"exact": (LIB, EXACT),
        "ref": (LIB_REF, EXACT + ["-DGDO_PLAIN_SUMS"]),
        "fast": (LIB_FAST, ["-Ofast", "-DGDO_PLAIN_SUMS"])}


def _compile(out: Path, flags: list[str], force: bool) -> None:
    newest = max(p.stat().st_mtime for p in SRCS + HDRS)
    if force or not out.exists() or out.stat().st_mtime < newest:
        cmd = ["gcc", *flags, "-std=c99", "-fPIC", "-shared", "-o", str(out), *map(str, SRCS), "-lm"]
        subprocess.run(cmd, check=True)


def build(force: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    for out, flags in LIBS.values():
        _compile(out, flags, force)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
