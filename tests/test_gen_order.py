"""The device generator plants all leaves, then all trunks, in parallel; the
host generator plants tree by tree in seed order.  This checks on the CPU,
with the shared generator code (gen_noise.cuh) compiled as host C++, that the
parallel order gives the sequential bytes on scenes where trees overlap."""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
SRC = HERE / "host" / "gen_host.cpp"
OUT = HERE / "host" / "_build" / "libgen_host.so"
DEPS = [SRC, HERE.parent / "unnamed-voxel-tracer_gb300" / "csrc" / "gen_noise.cuh"]


@pytest.fixture(scope="module")
def gh(vtlib):
    if not OUT.exists() or any(d.stat().st_mtime > OUT.stat().st_mtime for d in DEPS):
        OUT.parent.mkdir(exist_ok=True)
        subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", str(SRC), "-o", str(OUT)],
                       check=True)
    lib = C.CDLL(str(OUT))
    lib.gh_compare.restype = C.c_int
    lib.gh_compare.argtypes = [C.POINTER(vtlib.GenDesc_t), C.c_void_p, C.c_void_p]
    return lib


@pytest.mark.parametrize("dims,scale,seed,trees,caves", [
    ((96, 64, 80), 0.5, 7, 400, False),      # dense forest: many overlapping crowns and trunks
    ((48, 48, 48), 0.4, 3, 300, True),
    ((7, 40, 9), 0.3, 5, 50, False),         # barely wide enough for trees
    ((128, 96, 128), 0.6, 11, 1500, True),
])
def test_parallel_tree_order_equals_sequential(vtlib, gh, dims, scale, seed, trees, caves):
    d = vtlib.gen_desc(dims, scale=scale, seed=seed, trees=trees, caves=caves)
    n = dims[0] * dims[1] * dims[2]
    seq, par = np.zeros(n, np.uint8), np.zeros(n, np.uint8)
    assert gh.gh_compare(C.byref(d), seq.ctypes.data, par.ctypes.data) == 0
    assert np.array_equal(seq.reshape(dims[::-1]), vtlib.gen_world(d))
    assert (seq == 5).sum() > 0 and (seq == 6).sum() > 0
