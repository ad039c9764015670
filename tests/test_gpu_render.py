"""CUDA path vs the CPU oracle, through the C ABI (needs a GPU).

Bar: hit voxel, entry face, material, flags and t bit-exact; shaded RGBA8
within 1/255 per channel (the only float code outside the traversal whose
rounding may differ is the vignette: the device multiplies a column and a row
power, the oracle takes one powf of the product, as the reference does).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RGB_TOL = 1  # units of 1/255


def compare(gpu, ref, rgb_tol=RGB_TOL):
    assert gpu.shape == ref.shape
    for f in ("voxel", "face", "material", "flags"):
        bad = np.flatnonzero(gpu[f] != ref[f])
        assert bad.size == 0, f"{f}: {bad.size} mismatches, first at {bad[:5]}: gpu {gpu[bad[:5]]} ref {ref[bad[:5]]}"
    bad = np.flatnonzero(gpu["t"].view(np.uint32) != ref["t"].view(np.uint32))
    assert bad.size == 0, f"t: {bad.size} mismatches, first {gpu['t'][bad[:5]]} vs {ref['t'][bad[:5]]}"
    g = np.ascontiguousarray(gpu["rgba"]).view(np.uint8).reshape(-1, 4).astype(np.int16)
    r = np.ascontiguousarray(ref["rgba"]).view(np.uint8).reshape(-1, 4).astype(np.int16)
    assert np.abs(g - r).max(initial=0) <= rgb_tol


def make_world(vt, ctx, mats):
    Z, Y, X = mats.shape
    w = vt.World(ctx, (X, Y, Z))
    w.upload_dense(mats)
    return w


def render_both(vt, oracle, ctx, mats, cam, params, threads=8):
    w = make_world(vt, ctx, mats)
    try:
        gpu = vt.render_host(ctx, w, cam, params)
    finally:
        w.close()
    ref, stats = oracle.render(oracle.OracleWorld(mats), vt.default_palette(), cam, params, threads=threads)
    return gpu, ref, stats


def random_rays(rng, dims, n):
    X, Y, Z = dims
    o = np.stack([rng.uniform(-8, X + 8, n), rng.uniform(-8, Y + 8, n), rng.uniform(-8, Z + 8, n)], 1)
    d = rng.normal(size=(n, 3))
    d[rng.random(n) < 0.1, 0] = 0.0          # zero components
    d[rng.random(n) < 0.1, 1] = 0.0
    k = rng.random(n) < 0.05                 # axis-aligned diagonals (exact ties)
    d[k] = np.sign(d[k]) + (d[k] == 0)
    return o.astype(np.float32), d.astype(np.float32)


def test_trace_rays_random_padded_world(vt, oracle, ctx):
    """Ray list on a world whose dims are not multiples of the 32-voxel chunk."""
    d = vt.gen_desc((90, 70, 100), scale=0.6, seed=5, trees=20, caves=True)
    mats = vt.gen_world(d)
    w = make_world(vt, ctx, mats)
    rng = np.random.default_rng(1)
    o, dirs = random_rays(rng, (90, 70, 100), 20000)
    for steps in (1, 7, 64, 4096):
        gpu = vt.trace_rays(ctx, w, o, dirs, steps)
        ref = oracle.trace_rays(oracle.OracleWorld(mats), o, dirs, steps)
        compare(gpu, ref, rgb_tol=0)  # rgba carries the crossing count here
    w.close()


def test_trace_rays_kat(vt, oracle, ctx):
    mats = np.zeros((32, 32, 32), dtype=np.uint8)
    for (x, y, z) in ((10, 5, 7), (0, 1, 0), (0, 1, 1), (1, 1, 1), (0, 5, 7), (4, 0, 4)):
        mats[z, y, x] = 3
    o = np.array([(0.5, 5.5, 7.5), (20.5, 5.5, 7.5), (0.5, 0.5, 0.5), (0.5, 0.5, 0.5), (0.5, 0.5, 0.5),
                  (10.25, 5.5, 7.5), (-3.5, 5.5, 7.5), (4.5, -2.0, 4.5), (-5, 50, 5)], np.float32)
    d = np.array([(1, 0, 0), (-1, 0, 0), (1, 1, 0), (1, 1, 1), (0, 0, 0), (-1, .2, .3), (1, 0, 0), (0, 1, 0),
                  (0, 1, 0)], np.float32)
    w = make_world(vt, ctx, mats)
    for steps in (2, 10, 11, 512):
        compare(vt.trace_rays(ctx, w, o, d, steps), oracle.trace_rays(oracle.OracleWorld(mats), o, d, steps),
                rgb_tol=0)
    w.close()


def test_trace_rays_inside_origins_extreme_directions(vt, oracle, ctx):
    """Origins inside the grid, on and near the one-cell margin below which a
    walk starts in its own cell without the entry-box test, with direction
    components from 1e-38 to 1e38 (reciprocals that overflow, underflow or
    stay ordinary) and zero."""
    dims = (64, 48, 72)
    d = vt.gen_desc(dims, scale=0.5, seed=11, trees=8, caves=True)
    mats = vt.gen_world(d)
    w = make_world(vt, ctx, mats)
    rng = np.random.default_rng(12)
    n = 20000
    o = rng.uniform([0.0, 0.0, 0.0], dims, (n, 3))
    k = rng.random((n, 3))
    edge = np.array(dims, np.float64)
    o = np.where(k < 0.15, rng.choice([0.0, 0.5, 1.0, 1.0001, 0.9999], (n, 3)), o)
    o = np.where(k > 0.85, edge - rng.choice([0.0, 0.5, 1.0, 1.0001, 0.9999], (n, 3)), o)
    mags = np.array([0.0, 1e-38, 1e-30, 1e-8, 1.0, 1e8, 1e30, 1e38])
    dirs = rng.normal(size=(n, 3))
    dirs = np.where(rng.random((n, 3)) < 0.3, np.sign(dirs) * rng.choice(mags, (n, 3)), dirs)
    o, dirs = np.ascontiguousarray(o, np.float32), np.ascontiguousarray(dirs, np.float32)
    for steps in (1, 5000):
        gpu = vt.trace_rays(ctx, w, o, dirs, steps)
        compare(gpu, oracle.trace_rays(oracle.OracleWorld(mats), o, dirs, steps), rgb_tol=0)
    assert (gpu["face"] != 0xFF).sum() > 3000
    w.close()


def test_far_origins_both_walker_variants(vt, oracle, ctx):
    """Origins on both sides of |o| = 2^20 (the walker's one-correction plane
    search below it, the correction loop above), aimed at the world, with
    direction lengths from 1e-3 to 1e3; then a frame from a camera 3e6 voxels
    away, whose primary rays take the far variant."""
    dims = (96, 64, 80)
    d = vt.gen_desc(dims, scale=0.5, seed=9, trees=15, caves=True)
    mats = vt.gen_world(d)
    w = make_world(vt, ctx, mats)
    rng = np.random.default_rng(9)
    n = 20000
    target = rng.uniform([0, 0, 0], dims, (n, 3))
    away = rng.normal(size=(n, 3))
    away /= np.linalg.norm(away, axis=1, keepdims=True)
    dist = 10.0 ** rng.uniform(1, 6.6, n)
    o = (target + away * dist[:, None]).astype(np.float32)
    dirs = ((target - o) / dist[:, None] * (10.0 ** rng.uniform(-3, 3, n))[:, None]).astype(np.float32)
    far = np.abs(o).max(axis=1) >= 2 ** 20
    assert far.sum() > 1000 and (~far).sum() > 10000
    gpu = vt.trace_rays(ctx, w, o, dirs, 1 << 24)
    compare(gpu, oracle.trace_rays(oracle.OracleWorld(mats), o, dirs, 1 << 24), rgb_tol=0)
    assert (gpu["face"][far] != 0xFF).sum() > 300
    pos = np.array([3.0e6, 3.0e4, 2.5e6])
    to = np.array(dims, float) / 2 - pos
    cam = vt.Camera(pos=tuple(pos), yaw=float(np.arctan2(to[0], to[2])),
                    pitch=float(np.arcsin(to[1] / np.linalg.norm(to))), fov=4e-5, width=96, height=64)
    p = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW, max_steps=1 << 26, sun_dir=vt.gen_sun(9))
    c = cam.as_uniform_data()
    gpu = vt.render_host(ctx, w, c, p)
    ref, _ = oracle.render(oracle.OracleWorld(mats), vt.default_palette(), c, p, threads=8)
    compare(gpu, ref)
    assert (gpu["face"] != 0xFF).sum() > 500
    w.close()


@pytest.mark.parametrize("shade", ["none", "reference"])
def test_config0_frame(vt, oracle, ctx, shade):
    """128^3 terrain, 640x360, primary rays, max 512 steps."""
    d = vt.gen_desc((128, 128, 128), seed=0)
    mats = vt.gen_world(d)
    cam = vt.gen_camera(d, 0, 640, 360)
    p = vt.default_params(rays=vt.RAYS_PRIMARY, max_steps=512,
                          shade=vt.SHADE_NONE if shade == "none" else vt.SHADE_REFERENCE)
    gpu, ref, _ = render_both(vt, oracle, ctx, mats, cam, p)
    compare(gpu, ref)
    assert (gpu["flags"] & vt.HIT_PRIMARY).mean() > 0.3


TUNINGS = [dict(kernel=0, warp_tile_w=tw, occupancy=o) for tw in (4, 8, 16, 32) for o in (0, 1)] + \
          [dict(kernel=0, warp_tile_w=8, occupancy=1, share_bricks=1), dict(kernel=0, l2_persist=1),
           dict(kernel=2, warp_tile_w=16, occupancy=1)] + \
          [dict(kernel=1, batch=b) for b in (1, 16, 32)] + [dict(kernel=1, batch=16, l2_persist=1)]


@pytest.fixture
def tuned(ctx):
    yield ctx
    ctx.set_tuning()  # back to the default configuration


@pytest.mark.parametrize("tuning", TUNINGS, ids=lambda t: "-".join(f"{k}{v}" for k, v in t.items()))
def test_config1_world_primary_shadow(vt, oracle, tuned, tuning):
    """512x256x512 with 200 trees; primary + shadow, reference shading
    (reduced image so the oracle finishes in seconds), under every launch
    configuration the autotuner may pick."""
    d = vt.gen_desc((512, 256, 512), seed=1, trees=200)
    mats = vt.gen_world(d)
    sun = vt.gen_sun(1)
    tuned.set_tuning(**tuning)
    for cs in range(2):
        cam = vt.gen_camera(d, cs, 333, 187)   # partial tiles at the edges
        p = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW, sun_dir=sun)
        gpu, ref, _ = render_both(vt, oracle, tuned, mats, cam, p)
        compare(gpu, ref)


def test_repeated_frames_are_identical(vt, tuned):
    """The pixel queue hands pixels out in a different order every launch;
    the records must not depend on it, nor on the configuration."""
    d = vt.gen_desc((256, 128, 256), seed=3, trees=40)
    w = make_world(vt, tuned, vt.gen_world(d))
    cam = vt.gen_camera(d, 1, 640, 360)
    p = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW | vt.RAYS_BOUNCE, sun_dir=vt.gen_sun(3))
    first = vt.render_host(tuned, w, cam, p)
    tuned.set_tuning(kernel=vt.KERNEL_QUEUE, batch=16)
    for _ in range(4):
        assert np.array_equal(vt.render_host(tuned, w, cam, p), first)
    w.close()


@pytest.mark.parametrize("tw", [8, 16, 32])
def test_render_host_pipeline_equals_device_render(vt, tuned, tw):
    """Frames of >= 2^18 pixels go through vt_render_host's row-band pipeline
    (bands on several streams, each copied out when done) into pageable
    memory, and are written by the kernel itself into pinned memory; both
    equal one device-side vt_render of the frame."""
    d = vt.gen_desc((256, 128, 256), seed=6, trees=40)
    w = make_world(vt, tuned, vt.gen_world(d))
    tuned.set_tuning(kernel=0, warp_tile_w=tw, occupancy=1)
    p = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW, sun_dir=vt.gen_sun(6))
    try:
        for cs, (W, H) in enumerate([(1280, 720), (701, 397), (512, 1031)]):
            cam = vt.gen_camera(d, cs, W, H)
            buf = tuned.alloc(W * H * 16)
            vt.render(tuned, w, cam, p, buf)
            tuned.sync()
            want = buf.download(np.zeros(W * H, vt.HIT_DTYPE))
            buf.free()
            got = vt.render_host(tuned, w, cam, p)
            assert np.array_equal(got, want), (W, H)
            assert (got["face"] != 0xFF).sum() > 1000
            # pinned memory: the kernel writes the records straight into it
            pb = vt.PinnedBuffer(tuned, W * H, vt.HIT_DTYPE)
            try:
                pb.array[:] = np.zeros(1, vt.HIT_DTYPE)
                vt.render_host(tuned, w, cam, p, pb.array)
                assert np.array_equal(pb.array, want), (W, H)
            finally:
                pb.free()
    finally:
        w.close()


def test_autotune_picks_a_candidate_and_caches_it(vt, tuned, tmp_path):
    d = vt.gen_desc((256, 128, 256), seed=5, trees=20)
    w = make_world(vt, tuned, vt.gen_world(d))
    cam = vt.gen_camera(d, 0, 480, 270)
    p = vt.default_params()
    cache = str(tmp_path / "tune.txt")
    best, ms = tuned.autotune(w, cam, p, reps=2, cache_path=cache)
    assert ms > 0 and tuned.get_tuning() == best
    tuned.set_tuning()
    again, ms2 = tuned.autotune(w, cam, p, reps=2, cache_path=cache)   # served from the cache
    assert again == best and ms2 == pytest.approx(ms)
    assert len(open(cache).read().splitlines()) == 1
    ref = vt.render_host(tuned, w, cam, p)
    tuned.set_tuning()
    assert np.array_equal(vt.render_host(tuned, w, cam, p), ref)
    w.close()


def test_bounce_rays(vt, oracle, ctx):
    d = vt.gen_desc((256, 128, 256), seed=2, trees=60, caves=True)
    mats = vt.gen_world(d)
    cam = vt.gen_camera(d, 4, 256, 144)
    p = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW | vt.RAYS_BOUNCE, seed=1234, sun_dir=vt.gen_sun(2))
    gpu, ref, _ = render_both(vt, oracle, ctx, mats, cam, p)
    compare(gpu, ref)
    assert (gpu["flags"] & vt.HIT_BOUNCE).any()


BOUNCE_TUNINGS = [dict(bounce_walk=wk, bounce_refill=r) for wk in (0, 1) for r in (0, 1, 4, 16, 32)] + \
                 [dict(bounce_walk=1, l2_persist=1), dict(warp_tile_w=4, bounce_walk=1, bounce_refill=8)] + \
                 [dict(bounce_sort=1, warp_tile_w=tw, bounce_walk=wk) for tw in (4, 8, 16, 32) for wk in (0, 1)]


@pytest.mark.parametrize("tuning", BOUNCE_TUNINGS, ids=lambda t: "-".join(f"{k}{v}" for k, v in t.items()))
def test_bounce_pass_variants(vt, oracle, tuned, tuning):
    """The deferred bounce pass under every walk and refill setting the
    autotuner may pick (and with the L2 window): the records equal the
    oracle's."""
    d = vt.gen_desc((256, 128, 256), seed=12, trees=60, caves=True)
    mats = vt.gen_world(d)
    cam = vt.gen_camera(d, 2, 300, 170)
    p = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW | vt.RAYS_BOUNCE, seed=77, sun_dir=vt.gen_sun(12))
    tuned.set_tuning(**tuning)
    gpu, ref, _ = render_both(vt, oracle, tuned, mats, cam, p)
    compare(gpu, ref)
    assert (gpu["flags"] & vt.HIT_BOUNCE).any() and ((gpu["flags"] & 5) == 1).any()


def test_binned_bounce_pass_across_frame_sizes(vt, tuned):
    """The direction-sorted bounce append (each frame-kernel block sorts its
    rays in shared memory and appends them with one atomic): frames of
    different sizes, ragged edge blocks included, equal the default pass."""
    d = vt.gen_desc((256, 128, 256), seed=13, trees=40, caves=True)
    w = make_world(vt, tuned, vt.gen_world(d))
    p = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW | vt.RAYS_BOUNCE, seed=9, sun_dir=vt.gen_sun(13))
    try:
        cams = [vt.gen_camera(d, c, W, H) for c, (W, H) in enumerate([(640, 360), (97, 61), (640, 360), (333, 500)])]
        want = [vt.render_host(tuned, w, cam, p) for cam in cams]
        tuned.set_tuning(bounce_sort=1)
        for _ in range(2):
            for cam, ref in zip(cams, want):
                assert np.array_equal(vt.render_host(tuned, w, cam, p), ref)
    finally:
        w.close()


def test_lambert_and_checked_variant(vt, oracle, ctx):
    d = vt.gen_desc((128, 96, 160), seed=9, trees=15)
    mats = vt.gen_world(d)
    cam = vt.gen_camera(d, 1, 200, 120)
    p = vt.default_params(shade=vt.SHADE_LAMBERT, flags=vt.FLAG_CHECKED, sun_dir=vt.gen_sun(9))
    gpu, ref, _ = render_both(vt, oracle, ctx, mats, cam, p)
    compare(gpu, ref)


def test_stats_match_oracle_counters(vt, oracle, ctx):
    """Algorithmic byte counters of the instrumented kernel equal the oracle's."""
    d = vt.gen_desc((256, 128, 256), seed=4, trees=50)
    mats = vt.gen_world(d)
    cam = vt.gen_camera(d, 2, 240, 135)
    p = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW | vt.RAYS_BOUNCE, sun_dir=vt.gen_sun(4))
    w = make_world(vt, ctx, mats)
    st = vt.render_stats(ctx, w, cam, p)
    w.close()
    _, ref = oracle.render(oracle.OracleWorld(mats), vt.default_palette(), cam, p, threads=8)
    for k in ("primary_rays", "primary_hits", "shadow_rays", "shadow_hits", "bounce_rays", "bounce_hits",
              "mask_words", "coarse_words", "material_bytes", "record_bytes", "steps"):
        assert st[k] == ref[k], (k, st[k], ref[k])


def test_world_edits_match_oracle(vt, oracle, ctx):
    """set / get / upload_chunk (VoxelBrickmap.set/get, voxel.zig:58-70)."""
    d = vt.gen_desc((96, 64, 96), scale=0.5, seed=6, trees=10)
    mats = vt.gen_world(d)
    w = make_world(vt, ctx, mats)
    rng = np.random.default_rng(3)
    for _ in range(200):
        x, y, z = rng.integers(0, 96), rng.integers(0, 64), rng.integers(0, 96)
        m = int(rng.integers(0, 7)) if rng.random() < 0.5 else 0
        w.set(int(x), int(y), int(z), m)
        mats[z, y, x] = m
    chunk = rng.integers(0, 3, size=(32, 32, 32)).astype(np.uint8) * (rng.random((32, 32, 32)) < 0.1)
    w.upload_chunk(1, 0, 2, chunk)
    mats[64:96, 0:32, 32:64] = chunk
    empty = np.zeros((32, 32, 32), np.uint8)
    w.upload_chunk(0, 1, 0, empty)
    mats[0:32, 32:64, 0:32] = 0
    for (x, y, z) in ((5, 5, 5), (40, 10, 70), (95, 63, 95)):
        assert w.get(x, y, z) == mats[z, y, x]
    cam = vt.gen_camera(d, 3, 160, 90)
    p = vt.default_params()
    gpu = vt.render_host(ctx, w, cam, p)
    ref, _ = oracle.render(oracle.OracleWorld(mats), vt.default_palette(), cam, p, threads=8)
    compare(gpu, ref)
    w.clear()
    ctx.sync()
    gpu = vt.render_host(ctx, w, cam, p)
    assert not (gpu["flags"] & vt.HIT_PRIMARY).any()
    w.close()


def test_deferred_bounce_pass_equals_inline(vt, ctx):
    """Bounce rays of vt_render / vt_render_host go through the deferred pass
    (queue, persistent refill kernel, shading kernel); a batch job traces them
    inline.  Records must be identical, also for two deferred frames queued
    back to back on different streams (they share the context's queue)."""
    d = vt.gen_desc((256, 160, 256), seed=12, trees=80, caves=True)
    w = make_world(vt, ctx, vt.gen_world(d))
    p = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW | vt.RAYS_BOUNCE, seed=5, sun_dir=vt.gen_sun(12))
    cams = [vt.gen_camera(d, cs, 640, 400) for cs in range(2)]
    inline = []
    for cam in cams:
        buf = ctx.alloc(cam.width * cam.height * 16)
        b = vt.Batch(ctx, [(w, cam, buf)], p)
        b.launch()
        ctx.sync()
        inline.append(buf.download(np.zeros(cam.width * cam.height, vt.HIT_DTYPE)))
        b.close()
        buf.free()
    s1, s2 = ctx.stream(), ctx.stream()
    bufs = [ctx.alloc(c.width * c.height * 16) for c in cams]
    try:
        vt.render(ctx, w, cams[0], p, bufs[0], s1)
        vt.render(ctx, w, cams[1], p, bufs[1], s2)
        ctx.sync(s1)
        ctx.sync(s2)
        for c, buf, want in zip(cams, bufs, inline):
            got = buf.download(np.zeros(c.width * c.height, vt.HIT_DTYPE))
            assert np.array_equal(got, want)
            assert ((got["flags"] & vt.HIT_BOUNCE) != 0).sum() > 1000
            assert np.array_equal(vt.render_host(ctx, w, c, p), want)
            pb = vt.PinnedBuffer(ctx, c.width * c.height, vt.HIT_DTYPE)   # kernels write host memory directly
            try:
                vt.render_host(ctx, w, c, p, pb.array)
                assert np.array_equal(pb.array, want)
            finally:
                pb.free()
    finally:
        for b in bufs:
            b.free()
        for s in (s1, s2):
            ctx.lib.vt_stream_destroy(ctx.handle, s)
        w.close()
