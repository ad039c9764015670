"""The device traversal (trace_p.cuh, with its chunk and brick jumps) compiled
as host C++ and compared with the unit-step oracle, bit for bit, on the CPU.

This checks the skip logic and the index arithmetic of the kernel's traversal
without a GPU; the GPU tests then check the same code as compiled by nvcc.
"""
import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
SRC = HERE / "host" / "trace_host.cpp"
OUT = HERE / "host" / "_build" / "libtrace_host.so"
DEPS = [SRC, HERE.parent / "unnamed-voxel-tracer_gb300" / "csrc" / "trace_p.cuh",
        HERE.parent / "unnamed-voxel-tracer_gb300" / "csrc" / "vt_internal.h"]


def cuda_include():
    for p in ("/usr/local/cuda/include", "/usr/local/cuda/targets/x86_64-linux/include",
              "/usr/local/cuda/targets/sbsa-linux/include"):
        if (Path(p) / "cuda_runtime.h").exists():
            return p
    pytest.skip("CUDA headers not found")


@pytest.fixture(scope="module")
def ht():
    if not OUT.exists() or any(d.stat().st_mtime > OUT.stat().st_mtime for d in DEPS):
        OUT.parent.mkdir(exist_ok=True)
        subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", "-I", cuda_include(),
                        str(SRC), "-o", str(OUT)], check=True)
    lib = C.CDLL(str(OUT))
    lib.ht_trace_rays.restype = C.c_int
    P = C.c_void_p
    lib.ht_trace_rays.argtypes = [C.POINTER(C.c_int32), P, P, P, C.c_int32, C.c_int32, P, P, C.c_int32]
    return lib


def run_host(ht, mats, o, d, steps, fast=0):
    Z, Y, X = mats.shape
    n = o.shape[0]
    out = np.zeros(n * 4, dtype=np.uint32)
    cnt = np.zeros(2, dtype=np.uint64)
    st = ht.ht_trace_rays((C.c_int32 * 3)(X, Y, Z), mats.ctypes.data, o.ctypes.data, d.ctypes.data, n, steps,
                          out.ctypes.data, cnt.ctypes.data, fast)
    assert st == 0, "bounds check fired"
    return out.view(np.dtype([("voxel", "<u4"), ("t", "<f4"), ("rgba", "<u4"), ("face", "u1"),
                              ("material", "u1"), ("flags", "u1"), ("pad", "u1")])), cnt


def random_rays(rng, dims, n):
    X, Y, Z = dims
    o = np.stack([rng.uniform(-8, X + 8, n), rng.uniform(-8, Y + 8, n), rng.uniform(-8, Z + 8, n)], 1)
    d = rng.normal(size=(n, 3))
    d[rng.random(n) < 0.1, 0] = 0.0
    d[rng.random(n) < 0.1, 2] = 0.0
    k = rng.random(n) < 0.1
    d[k] = np.sign(d[k]) + (d[k] == 0)
    k = rng.random(n) < 0.1                      # origins on integer planes
    o[k] = np.round(o[k])
    return np.ascontiguousarray(o, np.float32), np.ascontiguousarray(d, np.float32)


def check(ht, oracle, mats, o, d, steps):
    ref = oracle.trace_rays(oracle.OracleWorld(mats), o, d, steps)
    for fast in (0, 1, 2):   # model walk, production walk, its one-path variant (bounce pass)
        got, _ = run_host(ht, mats, o, d, steps, fast)
        compare_exact(got, ref, o, d, fields=("voxel", "face", "material", "flags"))


def compare_exact(got, ref, o, d, fields):
    for f in fields:
        bad = np.flatnonzero(got[f] != ref[f])
        assert bad.size == 0, (f, bad[:5], o[bad[:3]], d[bad[:3]], got[bad[:3]], ref[bad[:3]])
    assert np.array_equal(got["t"].view(np.uint32), ref["t"].view(np.uint32))


@pytest.mark.parametrize("dims,seed", [((64, 64, 64), 1), ((90, 70, 100), 2), ((33, 97, 65), 3)])
def test_jumps_match_unit_steps(ht, oracle, vtlib, dims, seed):
    d = vtlib.gen_desc(dims, scale=0.5, seed=seed, trees=10, caves=True)
    mats = vtlib.gen_world(d)
    rng = np.random.default_rng(seed)
    o, dirs = random_rays(rng, dims, 6000)
    for steps in (1, 5, 40, 100000):
        check(ht, oracle, mats, o, dirs, steps)


def test_sparse_world_long_rays(ht, oracle):
    rng = np.random.default_rng(7)
    mats = np.zeros((128, 96, 160), np.uint8)
    idx = rng.integers(0, mats.size, 300)
    mats.reshape(-1)[idx] = rng.integers(1, 255, 300)
    o, d = random_rays(rng, (160, 96, 128), 20000)
    check(ht, oracle, mats, o, d, 1 << 20)


def test_far_origins_and_unnormalised_directions(ht, oracle, vtlib):
    """Origins up to ~4e6 away (both sides of the 2^20 bound below which the
    jump's plane search takes a single correction) aimed at the world, with
    direction lengths from 1e-3 to 1e3."""
    dims = (96, 64, 80)
    d = vtlib.gen_desc(dims, scale=0.5, seed=9, trees=15, caves=True)
    mats = vtlib.gen_world(d)
    rng = np.random.default_rng(9)
    n = 6000
    target = rng.uniform([0, 0, 0], dims, (n, 3))
    away = rng.normal(size=(n, 3))
    away /= np.linalg.norm(away, axis=1, keepdims=True)
    dist = 10.0 ** rng.uniform(1, 6.6, n)
    o = target + away * dist[:, None]
    dirs = (target - o) / dist[:, None] * (10.0 ** rng.uniform(-3, 3, n))[:, None]
    o, dirs = np.ascontiguousarray(o, np.float32), np.ascontiguousarray(dirs, np.float32)
    assert (np.abs(o).max(axis=1) >= 2 ** 20).sum() > 300 and (np.abs(o).max(axis=1) < 2 ** 20).sum() > 3000
    check(ht, oracle, mats, o, dirs, 1 << 24)
    got, _ = run_host(ht, mats, o, dirs, 1 << 24, 1)
    assert (got["face"] != 0xFF).sum() > 1500


def test_inside_origins_extreme_directions(ht, oracle, vtlib):
    """Origins inside the grid, on and near the one-cell margin of the walk's
    inside-start shortcut, with direction components from 1e-38 to 1e38
    (their reciprocals overflow, underflow or stay ordinary) and zero."""
    dims = (64, 48, 72)
    d = vtlib.gen_desc(dims, scale=0.5, seed=11, trees=8, caves=True)
    mats = vtlib.gen_world(d)
    rng = np.random.default_rng(11)
    n = 8000
    o = rng.uniform([0.0, 0.0, 0.0], dims, (n, 3))
    k = rng.random((n, 3))
    edge = np.array(dims, np.float64)
    o = np.where(k < 0.15, rng.choice([0.0, 0.5, 1.0, 1.0001, 0.9999], (n, 3)), o)
    o = np.where(k > 0.85, edge - rng.choice([0.0, 0.5, 1.0, 1.0001, 0.9999], (n, 3)), o)
    mags = np.array([0.0, 1e-38, 1e-30, 1e-8, 1.0, 1e8, 1e30, 1e38])
    dirs = rng.normal(size=(n, 3))
    pick = rng.random((n, 3)) < 0.3
    dirs = np.where(pick, np.sign(dirs) * rng.choice(mags, (n, 3)), dirs)
    o, dirs = np.ascontiguousarray(o, np.float32), np.ascontiguousarray(dirs, np.float32)
    check(ht, oracle, mats, o, dirs, 5000)
    got, _ = run_host(ht, mats, o, dirs, 5000, 1)
    assert (got["face"] != 0xFF).sum() > 1000


def test_counters_match_oracle(ht, oracle, vtlib):
    d = vtlib.gen_desc((128, 64, 96), scale=0.5, seed=4, trees=5)
    mats = vtlib.gen_world(d)
    rng = np.random.default_rng(4)
    o, dirs = random_rays(rng, (128, 64, 96), 3000)
    _, cnt = run_host(ht, mats, o, dirs, 4096)
    w = oracle.OracleWorld(mats)
    mw = cw = 0
    for i in range(o.shape[0]):
        tr = oracle.trace_one(w, o[i], dirs[i], 4096)
        mw += tr.mask_words
        cw += tr.coarse_words
    assert (int(cnt[0]), int(cnt[1])) == (mw, cw)


def test_threaded_frame_tracer_matches_oracle(ht, oracle, vtlib):
    """The benchmark's CPU leg for the skipping walk (ht_world_new, ht_trace_mt,
    ht_frame_mt on several threads) against the unit-step oracle: the same
    primary records, and the same primary + shadow ray and blocked counts."""
    ht.ht_world_new.restype = C.c_void_p
    ht.ht_world_new.argtypes = [C.POINTER(C.c_int32), C.c_void_p]
    ht.ht_world_free.argtypes = [C.c_void_p]
    ht.ht_trace_mt.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_int32]
    ht.ht_frame_mt.restype = C.c_int64
    ht.ht_frame_mt.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.POINTER(C.c_float),
                               C.c_int32, C.c_int32, C.POINTER(C.c_int64)]
    d = oracle.gen_desc((160, 96, 128), seed=4, trees=20)
    mats = oracle.gen_world(d)
    cam = oracle.gen_camera(d, 2, 120, 80)
    sun = oracle.gen_sun(4)
    p = oracle.default_params(rays=vtlib.RAYS_PRIMARY | vtlib.RAYS_SHADOW, sun_dir=sun)
    Z, Y, X = mats.shape
    hw = ht.ht_world_new((C.c_int32 * 3)(X, Y, Z), mats.ctypes.data)
    try:
        o, dd = oracle.primary_rays(cam)
        n = o.shape[0]
        out = np.zeros(n * 4, np.uint32)
        ht.ht_trace_mt(hw, o.ctypes.data, dd.ctypes.data, n, 512, out.ctypes.data, 3)
        recs, st = oracle.render(oracle.OracleWorld(mats), oracle.default_palette(), cam, p, threads=2)
        out = out.reshape(n, 4)
        assert np.array_equal(out[:, 0], recs["voxel"])
        assert np.array_equal(out[:, 1], recs["t"].view(np.uint32))
        hitm = out[:, 0] != 0xFFFFFFFF
        assert np.array_equal(out[hitm, 2], recs["material"][hitm])
        assert np.array_equal(out[hitm, 3] & 0xFF, recs["face"][hitm])
        dark = C.c_int64()
        rays = ht.ht_frame_mt(hw, o.ctypes.data, dd.ctypes.data, n, 512, (C.c_float * 3)(*sun), 512, 4,
                              C.byref(dark))
        assert rays == st["primary_rays"] + st["shadow_rays"]
        assert dark.value == st["shadow_hits"] and st["shadow_hits"] > 100
    finally:
        ht.ht_world_free(hw)
