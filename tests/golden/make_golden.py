"""Generates the golden fixtures of tests/golden/ (run where the reference
sources are present; the output is committed so the checks also run where
they are not).

  ref_tracemap.npz   rays and the reference's own traceMap results for them
                     (map.glsl:83-168 compiled as C++ by oracle/build_ref.py),
                     on a seeded world in the reference's format
  ref_primary.npz    the reference's primary rays and hits (primary.comp.glsl:31-43)
  ref_edit.npz       a sequence of editing passes (terrain_edit.comp.glsl's pick
                     ray, then map_setVoxel) and the brick pool after each
  oracle_frames.json hashes of the mode-P oracle's records for fixed seeds

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "unnamed-voxel-tracer_gb300"))
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(HERE.parent))

import oracle_py  # noqa: E402
import refworld  # noqa: E402
import vt  # noqa: E402

WORLD_SEED = 1234
N_RAYS = 2000
STEPS = (16, 192, 1024)


def golden_world():
    """The seeded reference-format world every fixture uses."""
    desc = vt.gen_desc((96, 80, 112), scale=0.5, seed=WORLD_SEED, trees=12, caves=True)
    mats = vt.gen_world(desc)
    rng = np.random.default_rng(WORLD_SEED)
    models = refworld.random_models(rng, 8)
    model_of = np.arange(256, dtype=np.uint32) % 8
    chunks, data = refworld.build_map(mats, model_of)
    return desc, mats, chunks, data, refworld.build_atlas(models)


def golden_rays():
    rng = np.random.default_rng(WORLD_SEED + 1)
    return refworld.random_rays(rng, -4.0, 120.0, N_RAYS)


def golden_camera():
    desc = vt.gen_desc((96, 80, 112), scale=0.5, seed=WORLD_SEED)
    return vt.gen_camera(desc, 3, 64, 48)


N_EDITS = 48


def edit_sequence():
    """(camera, edit_mode) pairs of the editing fixture: cameras over the golden
    world, edit_mode -1 (pick only), 0 (clear) or 1..29 (place model)."""
    desc = vt.gen_desc((96, 80, 112), scale=0.5, seed=WORLD_SEED)
    rng = np.random.default_rng(WORLD_SEED + 2)
    seq = []
    for i in range(N_EDITS):
        cam = vt.gen_camera(desc, 100 + i, 2, 2)
        seq.append((cam, int(rng.choice([-1, 0, 0, 1, 5, 13, 29]))))
    return seq


def ref_edit_run(ref, chunks, data, atlas):
    """Runs edit_sequence on the compiled reference: its pick (terrain_edit.comp
    .glsl:11-17) and its map_setVoxel (map.glsl:49-55), with the placement of
    the commented-out tail (:19-24).  Writes into `data`."""
    ref.ref_set_world(chunks.ctypes.data, data.ctypes.data, atlas.ctypes.data)
    out = {"data": [], "hit_pos": [], "normal": [], "pool_sha256": []}
    for cam, mode in edit_sequence():
        v, hp, nm = C.c_uint32(), (C.c_float * 3)(), (C.c_float * 3)()
        ref.ref_pick((C.c_float * 4)(*cam.pos), (C.c_float * 16)(*cam.view), C.byref(v), hp, nm)
        if v.value != 0 and mode >= 0:
            h = np.array(list(hp), np.float32)
            if mode > 0:
                p = [int(x) >> 3 for x in (h + np.array(list(nm), np.float32))]
                ref.ref_set_voxel(p[0], p[1], p[2], (1 << 28) + mode - 1)
            else:
                p = [int(x) >> 3 for x in h]
                ref.ref_set_voxel(p[0], p[1], p[2], 0)
        out["data"].append(v.value)
        out["hit_pos"].append(list(hp))
        out["normal"].append(list(nm))
        out["pool_sha256"].append(hashlib.sha256(data.tobytes()).hexdigest())
    return out


def frame_hash(records: np.ndarray) -> str:
    r = records.copy()
    return hashlib.sha256(r.tobytes()).hexdigest()


def oracle_frames() -> dict:
    out = {}
    cases = {
        "cfg0_primary_none": (vt.gen_desc((128, 128, 128), seed=0), 0, (160, 90),
                              dict(rays=vt.RAYS_PRIMARY, shade=vt.SHADE_NONE)),
        "cfg0_primary_shadow_ref": (vt.gen_desc((128, 128, 128), seed=0), 0, (160, 90),
                                    dict(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW, flags=0)),
        "trees_bounce": (vt.gen_desc((128, 96, 128), seed=5, trees=20, caves=True), 2, (96, 64),
                         dict(rays=7, seed=77, flags=0)),
    }
    for name, (desc, cam_seed, (W, H), kw) in cases.items():
        mats = vt.gen_world(desc)
        cam = vt.gen_camera(desc, cam_seed, W, H)
        p = vt.default_params(sun_dir=vt.gen_sun(desc.seed), **kw)
        rec, st = oracle_py.render(oracle_py.OracleWorld(mats), vt.default_palette(), cam, p, threads=4)
        out[name] = {"records_sha256": frame_hash(rec), "stats": st,
                     "world_sha256": hashlib.sha256(mats.tobytes()).hexdigest()}
    return out


def main() -> None:
    ref = oracle_py.load_ref()
    if ref is None:
        raise SystemExit("the reference sources are needed to make the fixtures")
    _, _, chunks, data, atlas = golden_world()
    ref.ref_set_world(chunks.ctypes.data, data.ctypes.data, atlas.ctypes.data)
    o, d = golden_rays()
    res = {"o": o, "d": d}
    for steps in STEPS:
        rd = np.zeros(N_RAYS, np.uint32)
        hp = np.zeros((N_RAYS, 3), np.float32)
        nm = np.zeros((N_RAYS, 3), np.float32)
        for i in range(N_RAYS):
            v = C.c_uint32()
            h3 = (C.c_float * 3)()
            n3 = (C.c_float * 3)()
            ref.ref_trace_map((C.c_float * 3)(*o[i]), (C.c_float * 3)(*d[i]), steps, C.byref(v), h3, n3)
            rd[i], hp[i], nm[i] = v.value, list(h3), list(n3)
        res[f"data_{steps}"], res[f"hit_pos_{steps}"], res[f"normal_{steps}"] = rd, hp, nm
    np.savez_compressed(HERE / "ref_tracemap.npz", **res)

    cam = golden_camera()
    W, H = cam.width, cam.height
    dirs = np.zeros((H, W, 3), np.float32)
    data_p = np.zeros((H, W), np.uint32)
    hp = np.zeros((H, W, 3), np.float32)
    nm = np.zeros((H, W, 3), np.float32)
    for py in range(H):
        for px in range(W):
            d3, v, h3, n3 = (C.c_float * 3)(), C.c_uint32(), (C.c_float * 3)(), (C.c_float * 3)()
            ref.ref_primary((C.c_float * 4)(*cam.pos), (C.c_float * 16)(*cam.view), cam.fov, px, py, W, H, d3,
                            C.byref(v), h3, n3)
            dirs[py, px], data_p[py, px], hp[py, px], nm[py, px] = list(d3), v.value, list(h3), list(n3)
    np.savez_compressed(HERE / "ref_primary.npz", dir=dirs, data=data_p, hit_pos=hp, normal=nm)

    _, _, chunks, data, atlas = golden_world()
    ed = ref_edit_run(ref, chunks, data.copy(), atlas)
    np.savez_compressed(HERE / "ref_edit.npz", data=np.array(ed["data"], np.uint32),
                        hit_pos=np.array(ed["hit_pos"], np.float32), normal=np.array(ed["normal"], np.float32),
                        pool_sha256=np.array(ed["pool_sha256"]))

    (HERE / "oracle_frames.json").write_text(json.dumps(oracle_frames(), indent=1, sort_keys=True) + "\n")
    print("fixtures written")


if __name__ == "__main__":
    main()
