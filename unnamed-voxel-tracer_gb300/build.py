"""Builds libvt.so (the CUDA library behind include/vt.h) in-tree.

CUDA sources are compiled for sm_103a only, host C++ with g++; every unit is
compiled in parallel and the shared object is linked with nvcc (static CUDA
runtime).  Parity-critical float code depends on --fmad=false (device) and
-ffp-contract=off (host): no multiply-add is fused unless the source says so.

Usage: python build.py [--force]
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
CSRC = HERE / "csrc"
OUT_DIR = HERE / "lib"
OBJ_DIR = HERE / "_build"
LIB = OUT_DIR / "libvt.so"

CUDA_SOURCES = ["api.cu", "world.cu", "render.cu", "tune.cu", "render_static.cu", "adjoint.cu", "batch.cu", "refmode.cu", "world_gen.cu", "edit.cu", "bounce.cu"]
CXX_SOURCES = ["gen.cpp", "vox.cpp", "procgen_ref.cpp"]

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libvt")


def _deps() -> list[Path]:
    return sorted(CSRC.glob("*")) + [ROOT / "include" / "vt.h", Path(__file__)]


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build step failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def build(force: bool = False, verbose: bool = False) -> Path:
    deps = _deps()
    if not force and not _stale(LIB, deps):
        return LIB
    OUT_DIR.mkdir(exist_ok=True)
    OBJ_DIR.mkdir(exist_ok=True)
    nv = nvcc()
    cmds = []
    objs = []
    for src in CUDA_SOURCES:
        obj = OBJ_DIR / (src + ".o")
        objs.append(obj)
        cmds.append([nv, GENCODE, "-lineinfo", "-O3", "-std=c++17", "--fmad=false", "-prec-div=true",
                     "-prec-sqrt=true", "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
                     "-Xptxas", "-warn-spills", "-c", str(CSRC / src), "-o", str(obj)])
    for src in CXX_SOURCES:
        obj = OBJ_DIR / (src + ".o")
        objs.append(obj)
        cmds.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-pthread",
                     "-Wall", "-c", str(CSRC / src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        for fut in [ex.submit(_run, c) for c in cmds]:
            fut.result()
    tmp = LIB.with_suffix(".so.tmp")
    _run([nv, GENCODE, "-shared", "-o", str(tmp)] + [str(o) for o in objs] + ["-lpthread"])
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
