"""Scene generation on the device (vt_world_generate) against the host
generator (vt_gen_world), byte for byte through vt_world_download_dense, and
frames rendered from a generated world against frames from an uploaded one."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims,scale,seed,trees,caves", [
    ((90, 70, 100), 0.6, 5, 20, True),        # dims not multiples of the chunk
    ((96, 64, 80), 0.5, 7, 400, False),       # overlapping trees
    ((256, 128, 192), 0.8, 9, 800, True),
    ((7, 40, 9), 0.3, 5, 50, False),
    ((5, 33, 5), 0.3, 2, 10, True),           # too narrow for trees
])
def test_generate_equals_host_generator(vt, ctx, dims, scale, seed, trees, caves):
    d = vt.gen_desc(dims, scale=scale, seed=seed, trees=trees, caves=caves)
    want = vt.gen_world(d)
    w = vt.World(ctx, dims)
    try:
        w.upload_dense(np.full(want.shape, 9, np.uint8))     # stale content must be overwritten
        w.generate(d)
        got = w.download_dense()
        assert np.array_equal(got, want), np.argwhere(got != want)[:5]
        for (z, y, x) in [(0, 0, 0), (dims[2] - 1, dims[1] - 1, dims[0] - 1), (dims[2] // 2, 1, dims[0] // 3)]:
            assert w.get(x, y, z) == want[z, y, x]
    finally:
        w.close()


def test_download_round_trips_upload(vt, ctx):
    rng = np.random.default_rng(3)
    mats = (rng.random((45, 37, 70)) < 0.2).astype(np.uint8) * rng.integers(1, 256, (45, 37, 70), dtype=np.uint8)
    w = vt.World(ctx, (70, 37, 45))
    try:
        w.upload_dense(mats)
        assert np.array_equal(w.download_dense(), mats)
    finally:
        w.close()


def test_generated_world_renders_like_uploaded(vt, ctx):
    d = vt.gen_desc((192, 128, 160), scale=0.7, seed=21, trees=120, caves=True)
    cam = vt.gen_camera(d, 1, 160, 96)
    p = vt.default_params()
    a, b = vt.World(ctx, (192, 128, 160)), vt.World(ctx, (192, 128, 160))
    try:
        a.upload_dense(vt.gen_world(d))
        b.generate(d)
        ra, rb = vt.render_host(ctx, a, cam, p), vt.render_host(ctx, b, cam, p)
        assert np.array_equal(ra, rb) and (ra["material"] != 0).sum() > 1000
    finally:
        a.close()
        b.close()


def test_generate_rejects_mismatched_dims(vt, ctx):
    d = vt.gen_desc((64, 64, 64), scale=0.5, seed=1)
    w = vt.World(ctx, (64, 64, 32))
    try:
        with pytest.raises(vt.VTError):
            w.generate(d)
    finally:
        w.close()
