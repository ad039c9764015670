"""Builds oracle/_ref/libref.so: the reference's own shader functions compiled
as C++ (TEST INFRASTRUCTURE).

Reads the reference's GLSL where it lies (REFERENCE_ROOT, default
/root/reference) and writes only into oracle/_ref/ (git-ignored):

  ref_map.inc      map.glsl: its #defines and every function from
                   intersectAABB to the end (traceMap, traceEntities, ...);
                   the SSBO/image declarations are replaced by ref_shim.cpp
  ref_camera.inc   camera.glsl after the uniform block (SUN_DIR, SkyDome2)
  ref_primary.inc  primary.comp.glsl from `vec2 rayUV` to the traceMap call
  ref_edit.inc     terrain_edit.comp.glsl, the same span (the pick ray)

Two mechanical rewrites make GLSL parse as C++ with GLSL's float semantics:
float literals get an `f` suffix (GLSL literals are single precision) and the
`.xyz` swizzle becomes a call.  `in` parameter qualifiers are dropped.  The
rest is glsl_compat.hpp.  When the reference is not present nothing is built.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
LIB = OUT / "libref.so"
REF = Path(os.environ.get("REFERENCE_ROOT", "/root/reference"))
SHADERS = REF / "assets" / "shaders"

_FLOAT = re.compile(r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][-+]?\d+)?)(?![\w.])")
_IN = re.compile(r"\bin\s+(?=(?:vec[234]|ivec[234]|uvec[234]|float|int|uint|bool)\b)")


def to_cpp(src: str) -> str:
    src = _FLOAT.sub(r"\1f", src)
    src = re.sub(r"\.xyz\b", ".xyz()", src)
    return _IN.sub("", src)


def extract_map(text: str) -> str:
    lines = text.splitlines()
    defines = [ln for ln in lines if ln.startswith("#define")]
    start = next(i for i, ln in enumerate(lines) if ln.startswith("vec2 intersectAABB"))
    return "\n".join(defines + lines[start:]) + "\n"


def extract_camera(text: str) -> str:
    lines = text.splitlines()
    start = next(i for i, ln in enumerate(lines) if ln.startswith("const vec3 SUN_DIR"))
    return "\n".join(lines[start:]) + "\n"


def extract_primary(text: str) -> str:
    lines = text.splitlines()
    start = next(i for i, ln in enumerate(lines) if ln.strip().startswith("vec2 rayUV"))
    end = next(i for i, ln in enumerate(lines) if "HitInfo inter = traceMap(" in ln)
    return "\n".join(lines[start:end + 1]) + "\n"


SOURCES = ("map.glsl", "camera.glsl", "primary.comp.glsl", "terrain_edit.comp.glsl")


def available() -> bool:
    return all((SHADERS / f).exists() for f in SOURCES)


def build(force: bool = False) -> Path:
    if not available():
        raise FileNotFoundError(f"reference shaders not found under {SHADERS}")
    deps = [SHADERS / f for f in SOURCES] + [HERE / "ref_shim.cpp", HERE / "glsl_compat.hpp", Path(__file__)]
    if not force and LIB.exists() and all(d.stat().st_mtime <= LIB.stat().st_mtime for d in deps):
        return LIB
    OUT.mkdir(exist_ok=True)
    (OUT / "ref_map.inc").write_text(to_cpp(extract_map((SHADERS / "map.glsl").read_text())))
    (OUT / "ref_camera.inc").write_text(to_cpp(extract_camera((SHADERS / "camera.glsl").read_text())))
    (OUT / "ref_primary.inc").write_text(to_cpp(extract_primary((SHADERS / "primary.comp.glsl").read_text())))
    (OUT / "ref_edit.inc").write_text(to_cpp(extract_primary((SHADERS / "terrain_edit.comp.glsl").read_text())))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = ["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-w",
           "-I", str(HERE), "-I", str(OUT), str(HERE / "ref_shim.cpp"), "-o", str(tmp)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"reference shader build failed: {' '.join(cmd)}\n{proc.stderr[-4000:]}")
    os.replace(tmp, LIB)
    return LIB


def build_if_available() -> Path | None:
    return build() if available() else None


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
