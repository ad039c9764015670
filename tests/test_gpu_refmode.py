"""Mode R on the GPU (the reference's world format and frame) against the CPU
restatement, which test_oracle_ref pins to the reference's compiled code.

Bar: traceMap results (data, hit position, normal) bit-exact; G-buffer
normal, position and illumination bit-exact; albedo and final colour within
1/255 (SkyDome2 and the vignette call powf, whose last bit may differ)."""
import numpy as np
import pytest

import refworld

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def refscene(vt, ctx, oracle):
    desc = vt.gen_desc((160, 96, 192), scale=0.6, seed=61, trees=20, caves=True)
    mats = vt.gen_world(desc)
    rng = np.random.default_rng(61)
    models = refworld.random_models(rng, 12)
    models[3] = refworld.random_models(rng, 1, full=True)[0]
    chunks, data = refworld.build_map(mats, np.arange(256, dtype=np.uint32) % 12)
    atlas = refworld.build_atlas(models)
    bm = vt.Brickmap(ctx)
    bm.upload(chunks, data)
    bm.set_atlas(atlas, 12)
    yield dict(desc=desc, bm=bm, ow=oracle.OracleRefWorld(chunks, data, atlas))
    bm.close()


def test_trace_map_bit_exact(vt, oracle, refscene):
    rng = np.random.default_rng(62)
    o, d = refworld.random_rays(rng, -4.0, 200.0, 6000)
    for steps in (5, 48, 192, 2000):
        got = refscene["bm"].trace_map(o, d, steps)
        for i in range(o.shape[0]):
            h = oracle.tracemap(refscene["ow"], o[i], d[i], steps)
            assert got["data"][i] == h.data, (steps, i)
            assert np.array_equal(got["hit_pos"][i].view(np.uint32), np.array(h.hit_pos, np.float32).view(np.uint32))
            assert np.array_equal(got["normal"][i], np.array(h.normal, np.float32))
        assert (got["data"] != 0).sum() > 500


def test_reference_frame(vt, oracle, refscene):
    for cs in range(2):
        cam = vt.gen_camera(refscene["desc"], cs, 96, 72)
        got = refscene["bm"].render(cam)
        want = oracle.render_reference(refscene["ow"], cam)
        for f in ("normal", "illumination"):
            assert np.array_equal(got[f], want[f]), f
        assert np.array_equal(got["position"].view(np.uint32), want["position"].view(np.uint32))
        for f in ("albedo", "color"):
            g = np.ascontiguousarray(got[f]).view(np.uint8).astype(int)
            w = np.ascontiguousarray(want[f]).view(np.uint8).astype(int)
            assert np.abs(g - w).max() <= 1, f
        hit = got["position"][:, 0] >= 0
        assert hit.sum() > 100 and (~hit).sum() > 0
        # lit: 0.3 stored in RGBA8 (0.3f * 255 rounds to 76.5, ties to even: 76); shadowed: -0.3 -> 0
        assert (got["illumination"] >> 24 == 0).sum() > 0 and (got["illumination"] >> 24 == 76).sum() > 0


def test_load_vox_equals_decoded_models(vt, ctx, refscene):
    rng = np.random.default_rng(63)
    pal = rng.integers(1, 2 ** 32, 256, dtype=np.uint64).astype(np.uint32)
    models = [[(int(x), int(y), int(z), int(c)) for x, y, z, c in
               zip(*(rng.integers(0, 8, 200) for _ in range(3)), rng.integers(1, 256, 200))] for _ in range(4)]
    data = refworld.write_vox(models, pal)
    desc = vt.gen_desc((64, 64, 64), scale=0.5, seed=64)
    mats = vt.gen_world(desc)
    chunks, bricks = refworld.build_map(mats, np.arange(256, dtype=np.uint32) % 4)
    a, b = vt.Brickmap(ctx), vt.Brickmap(ctx)
    try:
        a.upload(chunks, bricks)
        b.upload(chunks, bricks)
        assert a.load_vox(data) == 4
        for s, m in enumerate(vt.vox_decode(data)):
            b.set_model(s, m)
        o, d = refworld.random_rays(rng, -2.0, 70.0, 3000)
        ga, gb = a.trace_map(o, d, 500), b.trace_map(o, d, 500)
        assert np.array_equal(ga, gb) and (ga["data"] != 0).sum() > 100
    finally:
        a.close()
        b.close()


def test_reference_procgen_world_frame(vt, ctx, oracle):
    """The reference's own generator (vt_procgen_reference, 512^3, seeded
    noise) uploaded as a brickmap and rendered: the GPU frame equals the
    oracle's."""
    chunks, bricks = vt.procgen_reference(512, None, seed=11)
    rng = np.random.default_rng(11)
    atlas = refworld.build_atlas(refworld.random_models(rng, 29))
    bm = vt.Brickmap(ctx)
    try:
        bm.upload(chunks, bricks)
        bm.set_atlas(atlas, 29)
        ow = oracle.OracleRefWorld(chunks, bricks, atlas)
        for yaw in (0.7, 2.5):
            cam = vt.Camera(pos=(200.0, 70.0, 180.0), yaw=yaw, pitch=-0.45, fov=1.2, width=96, height=72)
            c = cam.as_uniform_data()
            got, want = bm.render(c), oracle.render_reference(ow, c)
            for f in ("normal", "illumination"):
                assert np.array_equal(got[f], want[f]), f
            assert np.array_equal(got["position"].view(np.uint32), want["position"].view(np.uint32))
            assert (got["position"][:, 0] >= 0).sum() > 1000
    finally:
        bm.close()
