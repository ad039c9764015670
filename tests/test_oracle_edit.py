"""The editing pass on the CPU: the oracle's restatement of the pick ray and
map_setVoxel (terrain_edit.comp.glsl:11-24, map.glsl:49-55) against the
reference's own code (a committed fixture from the compiled reference, and
live where the reference sources are present); the mode-P pick against the
mode-P primary ray of the centre pixel."""
import ctypes as C
import hashlib
import sys
from pathlib import Path

import numpy as np
import pytest

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))
import make_golden as G  # noqa: E402
import refworld  # noqa: E402


def run_oracle_edits(oracle, chunks, data, atlas, seq):
    rw = oracle.OracleRefWorld(chunks, data.copy(), atlas)
    out = []
    for cam, mode in seq:
        h = oracle.edit_r(rw, cam, mode)
        out.append((h.data, np.array(h.hit_pos, np.float32), np.array(h.normal, np.float32),
                    hashlib.sha256(rw.data.tobytes()).hexdigest()))
    return out


def test_edit_r_matches_reference_fixture(oracle):
    _, _, chunks, data, atlas = G.golden_world()
    g = np.load(HERE / "golden" / "ref_edit.npz")
    got = run_oracle_edits(oracle, chunks, data, atlas, G.edit_sequence())
    for i, (d, hp, nm, sha) in enumerate(got):
        assert d == g["data"][i], i
        assert np.array_equal(hp.view(np.uint32), g["hit_pos"][i].view(np.uint32)), i
        assert np.array_equal(nm, g["normal"][i]), i
        assert sha == g["pool_sha256"][i], i
    assert len(set(g["pool_sha256"])) > 20     # most passes changed the world


def test_edit_r_matches_compiled_reference_live(oracle):
    ref = oracle.load_ref()
    if ref is None:
        pytest.skip("reference sources not present; the fixture covers the editing pass")
    rng = np.random.default_rng(5)
    desc = oracle.vt.gen_desc((120, 72, 88), scale=0.5, seed=77, trees=10)
    mats = oracle.vt.gen_world(desc)
    chunks, data = refworld.build_map(mats, np.arange(256, dtype=np.uint32) % 6)
    atlas = refworld.build_atlas(refworld.random_models(rng, 6))
    seq = [(oracle.vt.gen_camera(desc, s, 2, 2), int(rng.choice([-1, 0, 2, 7]))) for s in range(40)]
    got = run_oracle_edits(oracle, chunks, data, atlas, seq)
    ref_data = data.copy()
    ref.ref_set_world(chunks.ctypes.data, ref_data.ctypes.data, atlas.ctypes.data)
    for i, (cam, mode) in enumerate(seq):
        v, hp, nm = C.c_uint32(), (C.c_float * 3)(), (C.c_float * 3)()
        ref.ref_pick((C.c_float * 4)(*cam.pos), (C.c_float * 16)(*cam.view), C.byref(v), hp, nm)
        if v.value != 0 and mode >= 0:
            h = np.array(list(hp), np.float32)
            src = h + np.array(list(nm), np.float32) if mode > 0 else h
            p = [int(x) >> 3 for x in src]
            ref.ref_set_voxel(p[0], p[1], p[2], (1 << 28) + mode - 1 if mode > 0 else 0)
        assert got[i][0] == v.value and list(got[i][1]) == list(hp), i
        assert got[i][3] == hashlib.sha256(ref_data.tobytes()).hexdigest(), i
    assert len({g[3] for g in got}) > 10


def test_pick_p_is_the_centre_pixel_ray(oracle, vtlib):
    desc = vtlib.gen_desc((96, 64, 96), scale=0.5, seed=3, trees=15)
    mats = vtlib.gen_world(desc)
    ow = oracle.OracleWorld(mats)
    p = vtlib.default_params(rays=vtlib.RAYS_PRIMARY, shade=vtlib.SHADE_NONE, max_steps=300)
    hits = 0
    for s in range(12):
        cam = vtlib.gen_camera(desc, s, 8, 6)
        rec, _ = oracle.render(ow, vtlib.default_palette(), cam, p)
        c = rec[3 * 8 + 4]
        tr, tgt = oracle.pick_p(ow, cam, 300, edit_mode=3)
        assert bool(tr.hit) == (c["face"] != 0xFF)
        if tr.hit:
            hits += 1
            assert tr.voxel == c["voxel"] and tr.face == c["face"]
            assert np.float32(tr.t).view(np.uint32) == c["t"].view(np.uint32)
            # the placed voxel is the hit voxel's neighbour across the hit face
            step = np.zeros(3, int)
            step[tr.face >> 1] = 1 if tr.face & 1 else -1
            want = np.array(tr.cell) + step
            inside = all(0 <= want[i] < ow.dims[i] for i in range(3))
            assert tgt[3] == int(inside) and (not inside or list(want) == tgt[:3])
            tr0, tgt0 = oracle.pick_p(ow, cam, 300, edit_mode=0)
            assert tgt0 == list(tr.cell) + [1]
    assert hits >= 6
