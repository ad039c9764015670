"""Builds the CPU oracle (test infrastructure only) into oracle/_build/.

    liboracle.so   vt_oracle.c (traversal, shading, gradient) and
                   vt_oracle_gen.c (the seeded scenes): gcc -O2
                   -ffp-contract=off (no fused multiply-add unless fmaf() is
                   written), POSIX threads.

The reference's own shader code compiled as C++ lives in oracle/_ref and is
built by oracle/build_ref.py when the reference sources are present.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "liboracle.so"
SOURCES = [HERE / "vt_oracle.c", HERE / "vt_oracle_gen.c", HERE / "vt_oracle.h", HERE.parent / "include" / "vt.h", Path(__file__)]


def build(force: bool = False) -> Path:
    if not force and LIB.exists() and all(s.stat().st_mtime <= LIB.stat().st_mtime for s in SOURCES):
        return LIB
    OUT.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread",
           "-Wall", "-o", str(tmp), str(HERE / "vt_oracle.c"), str(HERE / "vt_oracle_gen.c"), "-lm"]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
