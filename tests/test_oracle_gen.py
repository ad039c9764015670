"""The oracle's restatement of the seeded scenes (oracle/vt_oracle_gen.c)
against the library's host generator (vt_gen_*), byte for byte, on the CPU.
The benchmark's CPU legs build their inputs from the oracle's copy so that
they never load the GPU library."""
import ctypes as C

import numpy as np
import pytest

CASES = [
    ((128, 128, 128), 1.0, 0, 0, False),     # the small plain scene
    ((96, 64, 80), 1.0, 5, 12, False),       # trees
    ((64, 96, 72), 0.75, 9, 6, True),        # caves, scaled terrain
    ((33, 41, 7), 0.3, 123, 3, True),        # ragged sizes, trees near the edges
    ((5, 9, 5), 1.0, 2, 4, False),           # too narrow for trees
]


@pytest.mark.parametrize("dims,scale,seed,trees,caves", CASES)
def test_scene_bytes_equal_library(oracle, vtlib, dims, scale, seed, trees, caves):
    a = vtlib.gen_desc(dims, scale=scale, seed=seed, trees=trees, caves=caves)
    b = oracle.gen_desc(dims, scale=scale, seed=seed, trees=trees, caves=caves)
    assert bytes(a) == bytes(b)
    wa, wb = vtlib.gen_world(a, threads=3), oracle.gen_world(b, threads=5)
    assert np.array_equal(wa, wb)
    assert (wa > 0).any()
    for x, z in ((0, 0), (dims[0] - 1, dims[2] - 1), (dims[0] // 2, dims[2] // 3)):
        assert vtlib.load().vt_gen_height(C.byref(a), x, z) == oracle.load().vto_gen_height(C.byref(b), x, z)


def test_cameras_sun_palette_params_equal_library(oracle, vtlib):
    for dims, scale, seed, trees, caves in CASES[:4]:
        a = vtlib.gen_desc(dims, scale=scale, seed=seed, trees=trees, caves=caves)
        b = oracle.gen_desc(dims, scale=scale, seed=seed, trees=trees, caves=caves)
        for cs in range(6):
            for w, h in ((640, 360), (17, 3)):
                assert bytes(vtlib.gen_camera(a, cs, w, h)) == bytes(oracle.gen_camera(b, cs, w, h))
    for s in range(20):
        assert np.array_equal(np.array(vtlib.gen_sun(s), np.float32), np.array(oracle.gen_sun(s), np.float32))
    assert np.array_equal(vtlib.default_palette(), oracle.default_palette())
    kw = dict(rays=7, max_steps=300, sun_dir=(0.1, 0.9, -0.2))
    assert bytes(vtlib.default_params()) == bytes(oracle.default_params())
    assert bytes(vtlib.default_params(**kw)) == bytes(oracle.default_params(**kw))


def test_benchmark_world_equals_library(oracle, vtlib):
    """The 512 x 256 x 512 world with 200 trees the benchmark renders."""
    a = vtlib.gen_desc((512, 256, 512), seed=1, trees=200)
    b = oracle.gen_desc((512, 256, 512), seed=1, trees=200)
    assert np.array_equal(vtlib.gen_world(a), oracle.gen_world(b))
