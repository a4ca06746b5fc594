"""Build the native library (libgdc.so) and the dycore_test driver in-tree.

The CUDA translation unit is compiled for sm_103a only; host C++ units are
compiled with the system g++; everything links with nvcc into
``_build/libgdc.so`` next to this file.  Translation units compile in
parallel.  No cmake, no network.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
ROOT = PKG.parent
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Tile shapes of the stage kernel (rows x columns) per real type; the
# engine's tile_shape_supported accepts exactly these.
STAGE_SHAPES = {"f64": [(16, 64), (8, 64), (8, 32), (4, 128), (4, 32)],
                "f32": [(16, 64), (8, 64), (8, 32), (4, 128)]}


def _cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _run_all(cmds: list[list[str]]) -> None:
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for c in cmds]
    failed = []
    for c, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((c, out.decode(errors="replace")))
    if failed:
        msg = "\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("native build failed:\n" + msg)


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile libgdc.so (and the dycore_test executable); return the .so path."""
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    OUT.mkdir(exist_ok=True)
    lib = OUT / "libgdc.so"
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [INCLUDE / "gdc.h"]
    cu = [CSRC / "gdc_kernels_f64.cu", CSRC / "gdc_kernels_f32.cu", CSRC / "gdc_noalloc.cu", CSRC / "gdc_ic.cu"]
    shape_src = CSRC / "gdc_stage_shape.cu"
    cpp = [CSRC / "gdc_engine.cpp", CSRC / "gdc_host.cpp"]
    # (stem, source, defines): the stage kernels compile once per real type
    # and tile shape, in parallel with the other units.
    units = [(src.stem, src, []) for src in cu]
    for real, tag in (("double", "f64"), ("float", "f32")):
        for r, w in STAGE_SHAPES[tag]:
            units.append((f"gdc_stage_{r}x{w}_{tag}", shape_src,
                          [f"-DGDC_REAL={real}", f"-DGDC_TILE_R={r}", f"-DGDC_TILE_W={w}"]))
    if force or _stale(lib, cu + [shape_src] + cpp + headers):
        cmds, objs = [], []
        for stem, src, defs in units:
            obj = OUT / (stem + ".o")
            objs.append(obj)
            # The FP64 units keep the reference's rounding: no FMA contraction.
            # The FP32 units use fast single-precision division and square
            # root (fast math affects single precision only).
            fmad = ["--fmad=false"] if stem.endswith(("_f64", "_noalloc", "_ic")) else ["--use_fast_math"]
            cmds.append([nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", *fmad, *defs, "-Xcompiler",
                         "-fPIC,-ffp-contract=off", f"-I{INCLUDE}", "-c", str(src), "-o", str(obj)])
        for src in cpp:
            obj = OUT / (src.stem + ".o")
            objs.append(obj)
            # No FMA contraction in host code: the mesh and coefficient tables
            # round exactly as the reference's (and the same on x86 and Arm,
            # where g++ contracts by default).
            cmds.append(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-Wall", "-pthread",
                         f"-I{cuda / 'include'}", f"-I{INCLUDE}", "-c", str(src), "-o", str(obj)])
        if verbose:
            for c in cmds:
                print(" ".join(c))
        _run_all(cmds)
        link = [nvcc, *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-lcudart", "-lpthread"]
        _run_all([link])
    drv_src = CSRC / "dycore_test.cpp"
    drv = OUT / "dycore_test"
    if drv_src.exists() and (force or _stale(drv, [drv_src, lib])):
        _run_all([["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-Wall", f"-I{INCLUDE}", str(drv_src), "-o", str(drv),
                   f"-L{OUT}", "-lgdc", f"-Wl,-rpath,{OUT}"]])
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
