"""Mode R pieces on the CPU: traceEntities and SkyDome2 against the
reference's own code compiled as C++, and the .vox reader against the
reference's asset files (where present) and a written-out synthetic file."""
import ctypes as C
import os
from pathlib import Path

import numpy as np
import pytest

import refworld

# the reference checkout, where oracle/build_ref.py reads it too
ASSETS = Path(os.environ.get("REFERENCE_ROOT", "/root/reference")) / "assets"
# VoxelModelAtlas load order of the reference (game.zig:101-113)
LOAD_ORDER = ["models", "grass", "grass2", "grass3", "grass4", "grass5", "rock", "flower", "water", "tree",
              "leaves", "dirt", "sand"]


@pytest.fixture(scope="module")
def ref(oracle):
    lib = oracle.load_ref()
    if lib is None:
        pytest.skip("reference sources not present")
    return lib


def test_trace_entities_matches_reference(oracle, ref):
    rng = np.random.default_rng(17)
    hits = 0
    for _ in range(4000):
        o = rng.uniform([245, 15, 250], [263, 28, 266]).astype(np.float32)
        d = rng.normal(size=3).astype(np.float32)
        maxd = np.float32(rng.uniform(0.5, 20.0))
        h = oracle.trace_entities(o, d, float(maxd))
        v, hp, nm = C.c_uint32(), (C.c_float * 3)(), (C.c_float * 3)()
        ref.ref_trace_entities((C.c_float * 3)(*o), (C.c_float * 3)(*d), float(maxd), C.byref(v), hp, nm)
        assert h.data == v.value and list(h.hit_pos) == list(hp)
        hits += v.value != 0
    assert hits > 50


def test_sky_matches_reference(oracle, ref):
    rng = np.random.default_rng(18)
    for _ in range(2000):
        rd = rng.normal(size=3).astype(np.float32)
        out = (C.c_float * 4)()
        ref.ref_sky((C.c_float * 3)(0, 0, 0), (C.c_float * 3)(*rd), out)
        assert oracle.sky_ref(rd) == list(out)


def test_vox_reader_on_synthetic_file(vtlib):
    rng = np.random.default_rng(19)
    pal = rng.integers(1, 2 ** 32, 256, dtype=np.uint64).astype(np.uint32)
    models = []
    for _ in range(3):
        vox = {(int(x), int(y), int(z)): int(c) for x, y, z, c in
               zip(*(rng.integers(0, 8, 60) for _ in range(3)), rng.integers(1, 256, 60))}
        models.append([(x, y, z, c) for (x, y, z), c in vox.items()])
    data = refworld.write_vox(models, pal)
    got = vtlib.vox_decode(data)
    assert got.shape == (3, 8, 8, 8)
    assert np.array_equal(got, refworld.read_vox(data))
    x, y, z, c = models[0][0]
    assert got[0, y, z, x] == pal[c - 1]


def test_vox_reader_rejects_garbage(vtlib):
    with pytest.raises(vtlib.VTError):
        vtlib.vox_decode(b"not a vox file at all")


def test_vox_reader_on_reference_assets(vtlib):
    if not ASSETS.exists():
        pytest.skip("reference assets not present")
    total = 0
    for name in LOAD_ORDER:
        data = (ASSETS / f"{name}.vox").read_bytes()
        got = vtlib.vox_decode(data)
        assert np.array_equal(got, refworld.read_vox(data)), name
        assert (got != 0).any()
        total += got.shape[0]
    assert total == 29   # atlas slots 0..28 in the reference's load order
