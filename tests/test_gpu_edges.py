"""Edge cases of the frame and ray-list paths against the oracle (needs a GPU).

Empty, solid and sub-brick worlds; image shapes of one row, one column and
one pixel; cameras outside the grid looking in and looking away; step limits
of 0 and 1.  Same bar as test_gpu_render.py: records bit-exact, RGBA8 within
1/255 (the vignette).
"""
import math

import numpy as np
import pytest

from test_gpu_render import compare, make_world, random_rays

pytestmark = pytest.mark.gpu


def frame_both(vt, oracle, ctx, mats, cam, params):
    w = make_world(vt, ctx, mats)
    try:
        gpu = vt.render_host(ctx, w, cam, params)
        dev = ctx.alloc(cam.width * cam.height * 16)
        try:
            vt.render(ctx, w, cam, params, dev)
            ctx.sync()
            dv = dev.download(np.zeros(cam.width * cam.height, dtype=vt.HIT_DTYPE))
        finally:
            dev.free()
    finally:
        w.close()
    ref, _ = oracle.render(oracle.OracleWorld(mats), vt.default_palette(), cam, params, threads=8)
    assert np.array_equal(gpu.view(np.uint8), dv.view(np.uint8)), "device and host-output frames differ"
    return gpu, ref


def look_at(vt, pos, target, w, h, fov=math.radians(70)):
    to = np.asarray(target, float) - np.asarray(pos, float)
    yaw = float(np.arctan2(to[0], to[2]))
    pitch = float(np.arcsin(to[1] / np.linalg.norm(to)))
    return vt.Camera(pos=tuple(float(x) for x in pos), yaw=yaw, pitch=pitch, fov=fov, width=w, height=h).as_uniform_data()


PARAMS = dict(rays=3, sun_dir=(0.3, 0.8, 0.5))


def terrain(vt, dims, seed=3):
    return vt.gen_world(vt.gen_desc(dims, scale=0.5, seed=seed, trees=5))


def test_empty_world_is_all_sky(vt, oracle, ctx):
    mats = np.zeros((40, 24, 56), np.uint8)
    cam = look_at(vt, (20, 12, -30), (20, 12, 28), 97, 61)
    gpu, ref = frame_both(vt, oracle, ctx, mats, cam, vt.default_params(**PARAMS))
    compare(gpu, ref)
    assert (gpu["face"] == 0xFF).all()


def test_solid_world_hits_the_first_cell(vt, oracle, ctx):
    """Every voxel set: a camera inside hits its own cell at t = 0; a camera
    outside hits the face it enters through; shadow rays start inside solid."""
    mats = np.full((33, 20, 35), 3, np.uint8)
    for pos, inside in (((16.5, 10.25, 17.75), True), ((16.5, 40.0, -12.0), False)):
        cam = look_at(vt, pos, (16, 5, 17), 64, 48)
        gpu, ref = frame_both(vt, oracle, ctx, mats, cam, vt.default_params(**PARAMS))
        compare(gpu, ref)
        hit = (gpu["flags"] & vt.HIT_PRIMARY) != 0
        if inside:
            assert hit.all() and (gpu["t"] == 0.0).all()
        else:
            assert 0.3 < hit.mean() < 1.0  # the box fills part of the view


@pytest.mark.parametrize("dims", [(1, 1, 1), (3, 2, 5), (4, 4, 4), (7, 33, 2)])
def test_sub_brick_and_ragged_worlds(vt, oracle, ctx, dims):
    rng = np.random.default_rng(sum(dims))
    X, Y, Z = dims
    mats = (rng.random((Z, Y, X)) < 0.3).astype(np.uint8) * rng.integers(1, 7, (Z, Y, X), dtype=np.uint8)
    w = make_world(vt, ctx, mats)
    try:
        o, d = random_rays(rng, dims, 4000)
        for steps in (0, 1, 3, 64):
            compare(vt.trace_rays(ctx, w, o, d, steps), oracle.trace_rays(oracle.OracleWorld(mats), o, d, steps),
                    rgb_tol=0)
    finally:
        w.close()
    cam = look_at(vt, (X + 6.5, Y + 5.0, -4.25), (X / 2, Y / 2, Z / 2), 40, 30)
    gpu, ref = frame_both(vt, oracle, ctx, mats, cam, vt.default_params(**PARAMS))
    compare(gpu, ref)


@pytest.mark.parametrize("size", [(1, 1), (1, 517), (611, 1), (17, 13), (255, 3)])
def test_degenerate_image_shapes(vt, oracle, ctx, size):
    mats = terrain(vt, (96, 64, 96))
    cam = look_at(vt, (48, 55, 5), (48, 20, 70), *size)
    gpu, ref = frame_both(vt, oracle, ctx, mats, cam, vt.default_params(**PARAMS))
    compare(gpu, ref)


def test_cameras_outside_the_grid(vt, oracle, ctx):
    """Primary rays entering the grid from each side, and a camera looking away
    from it (every ray misses the box or has it behind its origin)."""
    dims = (80, 48, 72)
    mats = terrain(vt, dims, seed=4)
    centre = np.array(dims, float) / 2
    for off in ((-60, 5, 0), (70, 10, 3), (0, 90, 1), (2, -40, 0), (0, 4, -50), (3, 6, 65)):
        pos = centre + np.array(off, float)
        cam = look_at(vt, pos, centre, 72, 40)
        gpu, ref = frame_both(vt, oracle, ctx, mats, cam, vt.default_params(**PARAMS))
        compare(gpu, ref)
    away = look_at(vt, centre + np.array((-60.0, 5.0, 0.0)), centre + np.array((-200.0, 5.0, 0.0)), 72, 40)
    gpu, ref = frame_both(vt, oracle, ctx, mats, away, vt.default_params(**PARAMS))
    compare(gpu, ref)
    assert (gpu["face"] == 0xFF).all()


@pytest.mark.parametrize("steps", [0, 1, 2])
def test_tiny_step_limits_in_a_frame(vt, oracle, ctx, steps):
    mats = terrain(vt, (64, 48, 64), seed=5)
    cam = look_at(vt, (32, 30, 31), (40, 10, 60), 64, 40)
    p = vt.default_params(rays=3, sun_dir=(0.3, 0.8, 0.5), max_steps=steps, shadow_max_steps=steps)
    gpu, ref = frame_both(vt, oracle, ctx, mats, cam, p)
    compare(gpu, ref)


@pytest.mark.parametrize("size", [(32768, 2), (3, 32768)])
def test_largest_image_sides(vt, oracle, ctx, size):
    """Frames at the largest accepted width and height (32768)."""
    mats = terrain(vt, (64, 48, 64), seed=6)
    cam = look_at(vt, (32, 40, 30), (32, 10, 60), *size, fov=math.radians(20))
    gpu, ref = frame_both(vt, oracle, ctx, mats, cam, vt.default_params(**PARAMS))
    compare(gpu, ref)
    assert (gpu["flags"] & vt.HIT_PRIMARY).mean() > 0.2


@pytest.mark.parametrize("dims", [(8192, 8, 4), (4, 8192, 8), (8, 4, 8192)])
def test_longest_world_axes(vt, oracle, ctx, dims):
    """Worlds at the largest accepted extent (8192) along one axis: rays along
    and across the long axis."""
    rng = np.random.default_rng(dims.index(8192))
    X, Y, Z = dims
    mats = (rng.random((Z, Y, X)) < 0.02).astype(np.uint8) * 5
    w = make_world(vt, ctx, mats)
    try:
        o, d = random_rays(rng, dims, 6000)
        long_axis = dims.index(8192)
        d[:2000, long_axis] = np.where(d[:2000, long_axis] >= 0, 50.0, -50.0)  # mostly along the long axis
        d = d.astype(np.float32)
        for steps in (64, 20000):
            compare(vt.trace_rays(ctx, w, o, d, steps), oracle.trace_rays(oracle.OracleWorld(mats), o, d, steps),
                    rgb_tol=0)
    finally:
        w.close()


def test_sizes_beyond_the_limits_are_rejected(vt, ctx):
    for dims in ((8193, 4, 4), (0, 4, 4), (4, 4, -1)):
        with pytest.raises(vt.VTError):
            vt.World(ctx, dims)
    mats = np.zeros((8, 8, 8), np.uint8)
    w = make_world(vt, ctx, mats)
    try:
        for size in ((32769, 2), (2, 32769), (0, 5)):
            cam = look_at(vt, (4, 4, -4), (4, 4, 4), 1, 1)
            cam.width, cam.height = size
            with pytest.raises(vt.VTError):
                vt.render_host(ctx, w, cam, vt.default_params(**PARAMS), np.zeros(max(1, size[0] * size[1]), vt.HIT_DTYPE))
    finally:
        w.close()
