"""The batched launch (vt_batch_*): many worlds of different sizes, several
cameras each at different resolutions, one CUDA-graph launch, in all three
shapes (one launch per chunk of jobs with the job table as the launch's
parameters; per-job launches on concurrent graph chains; one persistent
unit-queue kernel).  Every job's records must equal what vt_render writes for
that job alone (and hence the oracle's, which test_gpu_render checks for
vt_render)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kernel", [0, 1, 2], ids=["chunks", "queue", "per-job"])
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
    batch makes those it needs before its capture (no allocation or
    synchronisation inside a capture) and equals the per-job renders and the
    allocation-free entry point."""
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
            if i == 0:
                assert np.array_equal(got, vt.render_host_static(ctx, w, cam, params))
            assert np.array_equal(got, vt.render_host(ctx, w, cam, params))
            assert np.array_equal(got, vt.render_host_static(ctx, w, cam, params))
        batch.close()
        for _, _, buf in jobs:
            buf.free()
        w.close()
    finally:
        ctx.close()


@pytest.mark.parametrize("checked", [False, True], ids=["plain", "checked"])
def test_batch_many_chunks(vt, ctx, checked):
    """126 jobs over 42 worlds (one launch per world in the default shape),
    small and ragged frames, the bounds-checked variant too, and one world
    with more jobs (300 one-pixel cameras) than one launch holds (256).  Every
    job equals its own vt_render."""
    rng = np.random.default_rng(41)
    flags = vt.FLAG_CROSSHAIR | vt.FLAG_VIGNETTE | (vt.FLAG_CHECKED if checked else 0)
    params = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW, sun_dir=vt.gen_sun(41), flags=flags)
    worlds, jobs = [], []
    try:
        for s in range(42):
            edge = int(rng.integers(24, 72))
            d = vt.gen_desc((edge, edge, edge), scale=edge / 128.0, seed=900 + s)
            w = vt.World(ctx, (edge, edge, edge))
            w.upload_dense(vt.gen_world(d))
            worlds.append(w)
            for c in range(3):
                W, H = [(24, 16), (17, 33), (40, 24), (1, 1)][int(rng.integers(0, 4))]
                cam = vt.gen_camera(d, c, W, H)
                jobs.append((w, cam, ctx.alloc(W * H * 16)))
        for c in range(300):
            cam = vt.gen_camera(d, 1000 + c, 1 + c % 3, 1 + c % 2)
            jobs.append((w, cam, ctx.alloc(cam.width * cam.height * 16)))
        batch = vt.Batch(ctx, jobs, params)
        for _ in range(2):
            for _, _, buf in jobs:
                buf.zero()
            batch.launch()
            ctx.sync()
            for w, cam, buf in jobs:
                got = buf.download(np.zeros(cam.width * cam.height, vt.HIT_DTYPE))
                assert np.array_equal(got, vt.render_host(ctx, w, cam, params))
        batch.close()
    finally:
        for _, _, buf in jobs:
            buf.free()
        for w in worlds:
            w.close()


def test_batch_autotune_keeps_identical_records(vt, ctx):
    """vt_batch_autotune times the three launch shapes, keeps the fastest,
    and the batch launched afterwards still equals the per-job renders."""
    params = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW, sun_dir=vt.gen_sun(51))
    worlds, jobs = [], []
    try:
        for s, edge in enumerate((48, 96, 130)):
            d = vt.gen_desc((edge, edge, edge), scale=edge / 128.0, seed=950 + s)
            w = vt.World(ctx, (edge, edge, edge))
            w.upload_dense(vt.gen_world(d))
            worlds.append(w)
            for c, (W, H) in enumerate([(120, 90), (64, 33)]):
                cam = vt.gen_camera(d, c, W, H)
                jobs.append((w, cam, ctx.alloc(W * H * 16)))
        batch = vt.Batch(ctx, jobs, params)
        shape, ms = batch.autotune(reps=2)
        assert shape in (vt.KERNEL_TILE, vt.KERNEL_QUEUE, vt.KERNEL_PER_JOB) and ms > 0
        for _, _, buf in jobs:
            buf.zero()
        batch.launch()
        ctx.sync()
        for w, cam, buf in jobs:
            got = buf.download(np.zeros(cam.width * cam.height, vt.HIT_DTYPE))
            assert np.array_equal(got, vt.render_host(ctx, w, cam, params))
        batch.close()
    finally:
        for _, _, buf in jobs:
            buf.free()
        for w in worlds:
            w.close()
