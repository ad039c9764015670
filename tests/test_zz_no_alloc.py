"""vt_render_host_static: rendering to host memory without any device
allocation, for hosts that own all device memory or must not call cudaMalloc
inside their frame loop.  It must return exactly what vt_render_host returns,
on every branch of the render path it runs (bounce rays traced inline, a
world edited since the last frame so its distances are updated first, the
persistent queue kernel), and it must allocate nothing: with the library's
allocation hook armed to fail the next allocation, it still succeeds, and
the library's allocation count does not move.

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


def _no_alloc_static(vt, ctx, w, cam, p):
    """render_host_static with the next library allocation armed to fail:
    the call must succeed without allocating."""
    made0, live0 = vt.alloc_counts()
    vt.fail_alloc(1)
    try:
        out = vt.render_host_static(ctx, w, cam, p)
    finally:
        vt.fail_alloc(0)
    assert vt.alloc_counts() == (made0, live0)
    return out


def test_static_staging_allocates_nothing(vt, ctx):
    d, w = _world(vt, ctx, 23)
    try:
        p = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW, sun_dir=vt.gen_sun(23))
        # an image size no other call of this context has rendered: no screen table exists for it
        cam = vt.gen_camera(d, 3, 333, 211)
        got = _no_alloc_static(vt, ctx, w, cam, p)
        assert np.array_equal(got, vt.render_host(ctx, w, cam, p))
    finally:
        w.close()


def test_static_staging_bounce_rays(vt, ctx):
    d, w = _world(vt, ctx, 24)
    try:
        p = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW | vt.RAYS_BOUNCE, seed=5,
                              sun_dir=vt.gen_sun(24))
        for cam_seed in (0, 1):   # two calls in a row
            cam = vt.gen_camera(d, cam_seed, 400, 300)
            want = vt.render_host(ctx, w, cam, p)   # deferred bounce pass
            got = _no_alloc_static(vt, ctx, w, cam, p)
            assert np.array_equal(got, want)
            assert (got["flags"] & vt.HIT_BOUNCE).any()
    finally:
        w.close()


def test_static_staging_after_edits(vt, ctx):
    """A voxel set on the host leaves the world's distances stale; the static
    call brings them up to date itself (update_distances) before tracing."""
    d, w = _world(vt, ctx, 25)
    try:
        p = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW, sun_dir=vt.gen_sun(25))
        cam = vt.gen_camera(d, 2, 480, 270)
        before = vt.render_host_static(ctx, w, cam, p)
        hit = before[(before["flags"] & vt.HIT_PRIMARY) != 0]
        X, Y = w.dims[0], w.dims[1]
        rng = np.random.default_rng(25)
        for v in rng.choice(hit["voxel"], 40, replace=False):
            w.set(int(v % X), int(v // X % Y), int(v // (X * Y)), 0)      # dig holes where rays hit
        for x, y, z in rng.integers(0, [256, 128, 256], (40, 3)):
            w.set(int(x), int(y), int(z), 7)                              # new voxels anywhere
        got = _no_alloc_static(vt, ctx, w, cam, p)
        assert not np.array_equal(got, before)
        assert np.array_equal(got, vt.render_host(ctx, w, cam, p))
    finally:
        w.close()


def test_static_staging_queue_kernel(vt, ctx):
    d, w = _world(vt, ctx, 26)
    p = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW, sun_dir=vt.gen_sun(26))
    try:
        cam = vt.gen_camera(d, 4, 512, 384)
        want = vt.render_host(ctx, w, cam, p)
        ctx.set_tuning(kernel=vt.KERNEL_QUEUE, batch=16)
        vt.render_host_static(ctx, w, cam, p)       # first queue launch: occupancy query
        for _ in range(2):
            got = _no_alloc_static(vt, ctx, w, cam, p)
            assert np.array_equal(got, want)
    finally:
        ctx.set_tuning()
        w.close()
