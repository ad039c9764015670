"""The batched launch (vt_batch_*): many worlds of different sizes, several
cameras each at different resolutions, one CUDA-graph launch, in both shapes
(per-job launches on concurrent graph chains; one persistent unit-queue
kernel).  Every job's records must equal what vt_render writes for that job
alone (and hence the oracle's, which test_gpu_render checks for vt_render)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kernel", [0, 1], ids=["tile-graph", "queue"])
def test_batch_matches_per_job_renders(vt, ctx, oracle, kernel):
    rng = np.random.default_rng(31)
    worlds, jobs, outs = [], [], []
    params = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW, sun_dir=vt.gen_sun(31))
    for s in range(6):
        edge = int(rng.integers(32, 200))
        d = vt.gen_desc((edge, edge, edge), scale=edge / 128.0, seed=500 + s)
        w = vt.World(ctx, (edge, edge, edge))
        w.upload_dense(vt.gen_world(d))
        worlds.append(w)
        for c in range(int(rng.integers(1, 4))):
            W, H = [(96, 64), (160, 120), (200, 75), (33, 17)][int(rng.integers(0, 4))]
            cam = vt.gen_camera(d, c, W, H)
            buf = ctx.alloc(W * H * 16)
            jobs.append((w, cam, buf))
    batch = vt.Batch(ctx, jobs, params)
    info = batch.info()
    assert info["jobs"] == len(jobs)
    try:
        ctx.set_tuning(kernel=kernel)        # the graph is captured at the first launch
        for rep in range(3):   # graph replays reuse the queue counter
            for _, cam, buf in jobs:
                buf.zero()
            batch.launch()
            ctx.sync()
            ctx.set_tuning()
            for w, cam, buf in jobs:
                got = buf.download(np.zeros(cam.width * cam.height, vt.HIT_DTYPE))
                want = vt.render_host(ctx, w, cam, params)
                assert np.array_equal(got, want)
    finally:
        ctx.set_tuning()
    batch.close()
    for _, _, buf in jobs:
        buf.free()
    for w in worlds:
        w.close()


def test_batch_captured_in_a_fresh_context(vt):
    """A context that has rendered nothing yet holds no screen tables: the
    batch graph is captured without making any (no allocation or
    synchronisation inside a capture) and still equals the per-job renders,
    which then make the tables."""
    ctx = vt.Context(0)
    try:
        d = vt.gen_desc((96, 64, 80), scale=0.5, seed=77)
        w = vt.World(ctx, (96, 64, 80))
        w.upload_dense(vt.gen_world(d))
        params = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW, sun_dir=vt.gen_sun(77))
        jobs = []
        for c, (W, H) in enumerate([(70, 41), (128, 72), (70, 41)]):
            cam = vt.gen_camera(d, c, W, H)
            jobs.append((w, cam, ctx.alloc(W * H * 16)))
        batch = vt.Batch(ctx, jobs, params)
        batch.launch()
        ctx.sync()
        for i, (_, cam, buf) in enumerate(jobs):
            got = buf.download(np.zeros(cam.width * cam.height, vt.HIT_DTYPE))
            if i == 0:  # the allocation-free entry point before any table of this size exists
                assert np.array_equal(got, vt.render_host_static(ctx, w, cam, params))
            assert np.array_equal(got, vt.render_host(ctx, w, cam, params))
            assert np.array_equal(got, vt.render_host_static(ctx, w, cam, params))
        batch.close()
        for _, _, buf in jobs:
            buf.free()
        w.close()
    finally:
        ctx.close()
