"""vt_render_host_static: rendering to host memory without any device
allocation, for hosts that own all device memory or must not call cudaMalloc
inside their frame loop.  It must return exactly what vt_render_host returns.

Named to be collected last, so that a run stopping at the first failure has
already run every other test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _world(vt, ctx, seed):
    d = vt.gen_desc((256, 128, 256), seed=seed, trees=30)
    w = vt.World(ctx, (256, 128, 256))
    w.upload_dense(vt.gen_world(d))
    return d, w


def test_static_staging_matches_render_host(vt, ctx):
    d, w = _world(vt, ctx, 21)
    p = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW, sun_dir=vt.gen_sun(21))
    try:
        # two calls in a row: the second reuses the shared array the first filled
        for cam_seed, (W, H) in ((0, (512, 288)), (1, (480, 270))):
            cam = vt.gen_camera(d, cam_seed, W, H)
            want = vt.render_host(ctx, w, cam, p)
            got = vt.render_host_static(ctx, w, cam, p)
            assert np.array_equal(got, want)
            assert (got["flags"] & vt.HIT_PRIMARY).any()
    finally:
        w.close()


def test_static_staging_rejects_large_frames(vt, ctx):
    d, w = _world(vt, ctx, 22)
    try:
        cam = vt.gen_camera(d, 0, 640, 480)   # 307200 > 262144 pixels
        with pytest.raises(vt.VTError) as err:
            vt.render_host_static(ctx, w, cam, vt.default_params())
        assert err.value.status == 1 and "262144" in str(err.value)
        cam = vt.gen_camera(d, 0, 512, 512)   # exactly the limit
        out = vt.render_host_static(ctx, w, cam, vt.default_params())
        assert np.array_equal(out, vt.render_host(ctx, w, cam, vt.default_params()))
    finally:
        w.close()
