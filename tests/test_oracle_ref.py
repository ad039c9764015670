"""Pins the CPU oracle to the reference's own code (CPU only).

The reference has no tests for its render path, so its shader functions are
compiled as C++ (oracle/build_ref.py -> oracle/_ref/libref.so) where the
reference sources are present, and their outputs are committed as fixtures
(tests/golden/make_golden.py) for everywhere else.

  - mode R: vto_tracemap / vto_primary_r restate traceMap and the primary ray
    (map.glsl:83-168, primary.comp.glsl:31-43) and must match bit for bit;
  - mode P: on worlds of full 8^3 models the reference's traceMap is a voxel
    DDA too; on the same rays the mode-P traversal finds the same voxel and
    face except on a pinned number of pixels, each of them a case of the
    reference's 0.999 snap (map.glsl:162) or its iteration cap;
  - the sky: SkyDome2 with pow() vs the products used here.
"""
import ctypes as C
import json
import sys
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))
import make_golden as G  # noqa: E402
import refworld  # noqa: E402


@pytest.fixture(scope="module")
def world(oracle):
    _, mats, chunks, data, atlas = G.golden_world()
    return mats, oracle.OracleRefWorld(chunks, data, atlas)


@pytest.fixture(scope="module")
def ref(oracle):
    lib = oracle.load_ref()
    if lib is None:
        pytest.skip("reference sources not present; the golden fixtures cover mode R")
    return lib


def test_tracemap_matches_reference_fixture(oracle, world):
    """vto_tracemap vs the reference's traceMap outputs committed from a run of
    the compiled reference (2000 rays x 3 step limits)."""
    _, rw = world
    g = np.load(HERE / "golden" / "ref_tracemap.npz")
    o, d = g["o"], g["d"]
    hits = 0
    for steps in G.STEPS:
        for i in range(o.shape[0]):
            h = oracle.tracemap(rw, o[i], d[i], steps)
            assert h.data == g[f"data_{steps}"][i], (steps, i)
            assert np.array_equal(np.array(h.hit_pos, np.float32).view(np.uint32),
                                  g[f"hit_pos_{steps}"][i].view(np.uint32)), (steps, i)
            assert np.array_equal(np.array(h.normal, np.float32), g[f"normal_{steps}"][i]), (steps, i)
            hits += h.data != 0
    assert hits > 1000


def test_primary_matches_reference_fixture(oracle, world):
    _, rw = world
    g = np.load(HERE / "golden" / "ref_primary.npz")
    cam = G.golden_camera()
    for py in range(cam.height):
        for px in range(cam.width):
            dvec, h = oracle.primary_r(rw, list(cam.pos), list(cam.view), cam.fov, px, py, cam.width, cam.height)
            assert np.array_equal(np.array(dvec, np.float32).view(np.uint32), g["dir"][py, px].view(np.uint32))
            assert h.data == g["data"][py, px]
            assert np.array_equal(np.array(h.hit_pos, np.float32).view(np.uint32),
                                  g["hit_pos"][py, px].view(np.uint32))


def test_tracemap_matches_compiled_reference_live(oracle, ref):
    """Fresh random worlds and rays against the compiled reference itself."""
    rng = np.random.default_rng(99)
    for trial in range(3):
        mats = (rng.random((40, 48, 56)) < 0.08).astype(np.uint8) * rng.integers(1, 9, (40, 48, 56)).astype(np.uint8)
        models = refworld.random_models(rng, 9, full=(trial == 2))
        chunks, data = refworld.build_map(mats, np.arange(256, dtype=np.uint32) % 9)
        atlas = refworld.build_atlas(models)
        rw = oracle.OracleRefWorld(chunks, data, atlas)
        ref.ref_set_world(rw.chunks.ctypes.data, rw.data.ctypes.data, rw.atlas.ctypes.data)
        o, d = refworld.random_rays(rng, -3.0, 60.0, 1500)
        for i in range(o.shape[0]):
            h = oracle.tracemap(rw, o[i], d[i], 300)
            v, hp, nm = C.c_uint32(), (C.c_float * 3)(), (C.c_float * 3)()
            ref.ref_trace_map((C.c_float * 3)(*o[i]), (C.c_float * 3)(*d[i]), 300, C.byref(v), hp, nm)
            assert h.data == v.value
            assert list(h.hit_pos) == list(hp) and list(h.normal) == list(nm)


# (camera seed, width, height) -> disagreeing pixels, measured; every one is a snap case
AGREEMENT_PINS = {(1, 96, 64): 6, (2, 160, 100): 119}


@pytest.mark.parametrize("cam_seed,width,height", sorted(AGREEMENT_PINS))
def test_mode_p_agrees_with_reference_on_full_models(oracle, ref, vtlib, cam_seed, width, height):
    """With every model a full 8^3 block, both traversals are voxel DDAs.  The
    same ray (the reference's: origin o + d max(tNear, 0) - 0.001,
    primary.comp.glsl:41-43) goes through the reference's traceMap (compiled)
    and the mode-P walk.  They disagree on the pinned number of pixels, and
    each disagreement is the reference's 0.999 snap (map.glsl:162), shown by
    the reference's stepping restated in float64 (refworld.tracemap_f64): with
    the snap it reproduces the compiled reference's voxel and face, with a
    vanishing snap it reproduces mode P's.  A miss of the reference that mode P
    hits is its 192-iteration cap (primary.comp.glsl:43) when the float64
    restatement also misses under the cap and finds mode P's hit without it."""
    desc = vtlib.gen_desc((128, 96, 128), seed=8, trees=25)
    mats = vtlib.gen_world(desc)
    rng = np.random.default_rng(8)
    models = refworld.random_models(rng, 7, full=True)
    chunks, data = refworld.build_map(mats, np.arange(256, dtype=np.uint32) % 7)
    rw = oracle.OracleRefWorld(chunks, data, refworld.build_atlas(models))
    ref.ref_set_world(rw.chunks.ctypes.data, rw.data.ctypes.data, rw.atlas.ctypes.data)
    ow = oracle.OracleWorld(mats)
    Z, Y, X = mats.shape

    def occupied(x, y, z):
        return 0 <= x < X and 0 <= y < Y and 0 <= z < Z and mats[z, y, x] != 0

    cam = vtlib.gen_camera(desc, cam_seed, width, height)
    assert all(0 < cam.pos[k] < mats.shape[2 - k] for k in range(3))   # inside the grid: tNear < 0
    o = [float(np.float32(cam.pos[k]) - np.float32(0.001)) for k in range(3)]
    face_of = {(-1, 0, 0): 0, (1, 0, 0): 1, (0, -1, 0): 2, (0, 1, 0): 3, (0, 0, -1): 4, (0, 0, 1): 5}
    snapped = capped = checked = 0
    disagree = []
    for py in range(cam.height):
        for px in range(cam.width):
            d3, v, hp, nm = (C.c_float * 3)(), C.c_uint32(), (C.c_float * 3)(), (C.c_float * 3)()
            ref.ref_primary((C.c_float * 4)(*cam.pos), (C.c_float * 16)(*cam.view), cam.fov, px, py, cam.width,
                            cam.height, d3, C.byref(v), hp, nm)
            d = list(d3)
            tr = oracle.trace_one(ow, o, d, 4096)
            want = None if v.value == 0 else (tuple(int(np.floor(hp[k] / 8.0)) for k in range(3)),
                                               face_of[tuple(int(nm[k]) for k in range(3))])
            got = (tuple(tr.cell), tr.face) if tr.hit else None
            if (px * 7 + py * 13) % 97 == 0:   # the float64 restatement against the compiled reference
                assert refworld.tracemap_f64(occupied, o, d, 192, 0.999) == want, (px, py)
                checked += 1
            if got == want:
                continue
            disagree.append((px, py))
            assert refworld.tracemap_f64(occupied, o, d, 192, 0.999) == want, (px, py)
            if want is None and refworld.tracemap_f64(occupied, o, d, 4096, 0.999) == got:
                capped += 1
                continue
            assert refworld.tracemap_f64(occupied, o, d, 4096, 1.0 - 1e-9) == got, (px, py, got, want)
            snapped += 1
    assert len(disagree) == AGREEMENT_PINS[(cam_seed, width, height)], len(disagree)
    assert snapped + capped == len(disagree) and checked > 50
    assert 1.0 - len(disagree) / (cam.width * cam.height) >= 0.99


def test_sky_products_match_reference_pow(oracle, ref):
    rng = np.random.default_rng(5)
    sun = np.array([7.52185881e-01, 6.58950984e-01, 7.52185881e-01], np.float32)
    for _ in range(500):
        rd = rng.normal(size=3).astype(np.float32)
        out = (C.c_float * 4)()
        ref.ref_sky((C.c_float * 3)(0, 0, 0), (C.c_float * 3)(*rd), out)
        sn = sun / np.sqrt(np.float32(sun @ sun))
        rn = rd / np.sqrt(np.float32(rd @ rd))
        s = np.float32(min(max(np.float32(sn @ rn), 0.0), 1.2))
        col = np.array([0.6, 0.71, 0.75], np.float32) - rd[1] * np.float32(0.2) * np.array([1, .5, 1], np.float32) \
            + np.float32(0.075) + np.float32(0.4) * np.array([1, .6, .1], np.float32) * s ** 8 \
            + np.array([0.2, 0.08, 0.04], np.float32) * s ** 3
        assert np.max(np.abs(col - np.array(out[:3]))) < 2e-6


def test_oracle_frames_match_fixture(oracle, vtlib):
    """The oracle's mode-P records for fixed seeds (hash-pinned)."""
    want = json.loads((HERE / "golden" / "oracle_frames.json").read_text())
    got = G.oracle_frames()
    for k in want:
        assert got[k]["world_sha256"] == want[k]["world_sha256"], k
        assert got[k]["stats"] == want[k]["stats"], k
        assert got[k]["records_sha256"] == want[k]["records_sha256"], k
