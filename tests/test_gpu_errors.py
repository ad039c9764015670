"""Error paths on the GPU, made on the host (nothing faults the device):

  - allocation failures injected by the library's own allocation hook
    (vt_debug_fail_alloc) in context, world, batch, staging, screen-table and
    bounce-queue allocations: each call returns VT_ERR_OOM, the object stays
    usable or is not created, and once everything is destroyed no allocation
    of the library is left live (vt_debug_alloc_counts);
  - vt_wait's deadline: VT_ERR_TIMEOUT while a stream is still busy, the work
    untouched, then success once it is done;
  - the device status word's event covers every pending checked launch, also
    across streams: a vt_sync on one stream is not satisfied before a checked
    launch still running on another stream is done.

The reference has no error returns on this path: its block allocator panics
when it cannot grow (src/engine/graphics/gpu_block_allocator.zig:22)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OOM = 2


@pytest.fixture
def hook(vt):
    vt.fail_alloc(0)
    yield vt
    vt.fail_alloc(0)


def _oom(fn):
    try:
        fn()
    except Exception as e:  # noqa: BLE001
        assert getattr(e, "status", None) == OOM, e
        return True
    return False


def test_context_create_fails_cleanly(hook):
    vt = hook
    _, live0 = vt.alloc_counts()
    failures = 0
    for k in range(1, 12):
        vt.fail_alloc(k)
        try:
            c = vt.Context(0)
        except vt.VTError as e:
            assert e.status == OOM
            failures += 1
            assert vt.alloc_counts()[1] == live0, k
            continue
        vt.fail_alloc(0)
        c.close()
        break
    assert failures >= 4          # status word, counters, queue counters, pinned status
    assert vt.alloc_counts()[1] == live0


def test_world_create_and_upload_fail_cleanly(hook):
    vt = hook
    _, live0 = vt.alloc_counts()
    d = vt.gen_desc((96, 64, 80), seed=5, trees=4)
    mats = vt.gen_world(d)
    with vt.Context(0) as ctx:
        live_ctx = vt.alloc_counts()[1]
        failures = 0
        for k in range(1, 20):
            vt.fail_alloc(k)
            try:
                w = vt.World(ctx, (96, 64, 80))
            except vt.VTError as e:
                assert e.status == OOM
                failures += 1
                assert vt.alloc_counts()[1] == live_ctx, k
                continue
            vt.fail_alloc(0)
            break
        assert failures >= 10         # every array of the world
        # the staging buffer of the first upload fails; the world stays usable
        vt.fail_alloc(1)
        assert _oom(lambda: w.upload_dense(mats))
        vt.fail_alloc(0)
        w.upload_dense(mats)
        cam = vt.gen_camera(d, 0, 64, 48)
        p = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW)
        ok = vt.render_host(ctx, w, cam, p)
        assert (ok["flags"] & vt.HIT_PRIMARY).any()
        w.close()
    assert vt.alloc_counts()[1] == live0


def test_frame_buffers_and_batch_fail_cleanly(hook, oracle):
    """A fresh context's first bounce frame allocates its screen table and
    the deferred bounce queue; a batch allocates its job table and counter.
    Each injected failure returns VT_ERR_OOM and the next call succeeds with
    the oracle's records."""
    vt = hook
    _, live0 = vt.alloc_counts()
    d = vt.gen_desc((128, 96, 128), seed=6, trees=10)
    mats = vt.gen_world(d)
    cam = vt.gen_camera(d, 1, 96, 64)
    p = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW | vt.RAYS_BOUNCE, seed=3)
    ref, _ = oracle.render(oracle.OracleWorld(mats), vt.default_palette(), cam, p, threads=4)
    with vt.Context(0) as ctx:
        w = vt.World(ctx, (128, 96, 128))
        w.upload_dense(mats)
        buf = ctx.alloc(cam.width * cam.height * 16)
        ctx.sync()
        failures = 0
        for k in range(1, 8):
            vt.fail_alloc(k)
            if _oom(lambda: (vt.render(ctx, w, cam, p, buf), ctx.sync())):
                failures += 1
                continue
            vt.fail_alloc(0)
            break
        assert failures >= 3          # screen table, bounce rays, bounce results
        got = buf.download(np.zeros(cam.width * cam.height, vt.HIT_DTYPE))
        for f in ("voxel", "face", "material", "flags"):
            assert np.array_equal(got[f], ref[f]), f
        for k in (1, 2):
            vt.fail_alloc(k)
            assert _oom(lambda: vt.Batch(ctx, [(w, cam, buf)], p))
        vt.fail_alloc(0)
        b = vt.Batch(ctx, [(w, cam, buf)], p)
        b.launch()
        ctx.sync()
        b.close()
        buf.free()
        w.close()
    assert vt.alloc_counts()[1] == live0


def test_wait_deadline(vt, ctx):
    d = vt.gen_desc((256, 128, 256), seed=7, trees=20)
    w = vt.World(ctx, (256, 128, 256))
    w.upload_dense(vt.gen_world(d))
    cam = vt.gen_camera(d, 0, 1920, 1080)
    p = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW)
    buf = ctx.alloc(1920 * 1080 * 16)
    st = ctx.stream()
    try:
        vt.render(ctx, w, cam, p, buf, st)
        ctx.sync(st)
        for _ in range(40):            # several ms of queued frames
            vt.render(ctx, w, cam, p, buf, st)
        assert ctx.wait(0, st) is False
        assert "still busy" in ctx.lib.vt_last_error_string(ctx.handle).decode()
        assert ctx.wait(20_000_000, st) is True
        assert ctx.wait(0, st) is True
    finally:
        ctx.sync(st)
        ctx.lib.vt_stream_destroy(ctx.handle, st)
        buf.free()
        w.close()


def test_status_event_covers_writers_on_other_streams(vt, ctx):
    """Checked 4K frames on stream A, then one checked ray on stream B:
    vt_sync(B) returns only once A's checked launches are done too (the status
    word is then read after every launch that may set it)."""
    d = vt.gen_desc((256, 128, 256), seed=8, trees=20)
    w = vt.World(ctx, (256, 128, 256))
    w.upload_dense(vt.gen_world(d))
    cam = vt.gen_camera(d, 1, 3840, 2160)
    p = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW, flags=vt.FLAG_CHECKED)
    buf = ctx.alloc(3840 * 2160 * 16)
    a, b = ctx.stream(), ctx.stream()
    # buffers first: allocation and upload may synchronise the device
    dev_o, dev_d, out = ctx.alloc(12), ctx.alloc(12), ctx.alloc(16)
    dev_o.upload(np.array([[128.5, 120.0, 128.5]], np.float32))
    dev_d.upload(np.array([[0.1, -1.0, 0.2]], np.float32))
    try:
        vt.render(ctx, w, cam, p, buf, a)
        ctx.sync(a)
        for _ in range(6):
            vt.render(ctx, w, cam, p, buf, a)
        ctx.check(ctx.lib.vt_trace_rays(ctx.handle, w.handle, dev_o.ptr, dev_d.ptr, 1, 512, out.ptr, b))
        ctx.sync(b)
        assert ctx.wait(0, a) is True   # A's checked frames finished before B's sync returned
        for x in (dev_o, dev_d, out):
            x.free()
    finally:
        ctx.sync(a)
        ctx.sync(b)
        ctx.lib.vt_stream_destroy(ctx.handle, a)
        ctx.lib.vt_stream_destroy(ctx.handle, b)
        buf.free()
        w.close()
