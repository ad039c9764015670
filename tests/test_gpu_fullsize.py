"""Parity at the benchmark's full sizes.

  - the 512x256x512 world (200 trees) at 1920x1080, primary + shadow rays,
    all 8 benchmark cameras, every pixel against the oracle;
  - the 2048x256x2048 world with caves (1 GiB of materials) at 3840x2160,
    primary + shadow + bounce rays, both cameras, every 16th row against the
    oracle;
  - size-independent properties of the full frames: the records of the
    batched graph and of the pinned-memory path equal vt_render's, and the
    instrumented kernel's counters equal the oracle's on sampled rows;
  - the batch workload's scenes up to 300 voxels on a side, as one batch
    graph, every 4th row of every job against the oracle (about 11 M rays),
    and all its scenes above 300 voxels on a side, every 8th row;
  - the shading benchmark at full size (16 views of 512x512): one fused
    forward + backward over all views against the FP64 gradient.

The oracle runs multithreaded on the host (about a second per 1080p frame on
16 cores)."""
import os

import numpy as np
import pytest

from test_gpu_adjoint import grad_close
from test_gpu_render import compare

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 4


@pytest.fixture(scope="module")
def world1(vt, ctx, oracle):
    d = vt.gen_desc((512, 256, 512), seed=1, trees=200)
    mats = vt.gen_world(d)
    w = vt.World(ctx, (512, 256, 512))
    w.upload_dense(mats)
    yield d, mats, w, oracle.OracleWorld(mats)
    w.close()


def test_benchmark_frames_match_oracle(vt, ctx, oracle, world1):
    d, mats, w, ow = world1
    p = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW, max_steps=512, shadow_max_steps=512,
                          sun_dir=vt.gen_sun(1))
    hits = 0
    for cs in range(8):
        cam = vt.gen_camera(d, cs, 1920, 1080)
        gpu = vt.render_host(ctx, w, cam, p)
        ref, _ = oracle.render(ow, vt.default_palette(), cam, p, threads=THREADS)
        compare(gpu, ref)
        hits += int((gpu["flags"] & vt.HIT_PRIMARY).sum())
    assert hits > 8 * 1920 * 1080 // 3


def test_benchmark_frame_paths_agree(vt, ctx, world1):
    """vt_render (device), vt_render_host into pinned memory and a batch of
    the 8 cameras give the same records."""
    d, mats, w, _ = world1
    p = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW, sun_dir=vt.gen_sun(1))
    cams = [vt.gen_camera(d, cs, 1920, 1080) for cs in range(8)]
    bufs = [ctx.alloc(1920 * 1080 * 16) for _ in cams]
    pb = vt.PinnedBuffer(ctx, 1920 * 1080, vt.HIT_DTYPE)
    try:
        batch = vt.Batch(ctx, [(w, c, b) for c, b in zip(cams, bufs)], p)
        batch.launch()
        ctx.sync()
        for c, b in zip(cams, bufs):
            want = b.download(np.zeros(1920 * 1080, vt.HIT_DTYPE))
            vt.render_host(ctx, w, c, p, pb.array)
            assert np.array_equal(pb.array, want)
        batch.close()
    finally:
        pb.free()
        for b in bufs:
            b.free()


def test_counters_match_oracle_full_frame(vt, ctx, oracle, world1):
    d, mats, w, ow = world1
    p = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW, sun_dir=vt.gen_sun(1))
    cam = vt.gen_camera(d, 5, 1920, 1080)
    st = vt.render_stats(ctx, w, cam, p)
    _, ref = oracle.render(ow, vt.default_palette(), cam, p, threads=THREADS)
    for k in ("primary_rays", "primary_hits", "shadow_rays", "shadow_hits", "mask_words", "coarse_words",
              "material_bytes", "record_bytes", "steps"):
        assert st[k] == ref[k], k


def test_config2_world_4k_with_bounce_rays_sampled_rows(vt, ctx, oracle):
    """Both benchmark cameras of the 4K cave frame, every 16th row (offset by
    the camera so the two cover different rows)."""
    import scenes
    desc, cams, params = scenes.config2()
    X, Y, Z = desc.dims
    w = vt.World(ctx, (X, Y, Z))
    try:
        w.generate(desc)                      # on the device, same bytes as the host generator
        mats = w.download_dense()
        ow = oracle.OracleWorld(mats)
        step = 16
        assert len(cams) == 2
        for ci, cam in enumerate(cams):
            gpu = vt.render_host(ctx, w, cam, params)
            ref, st = oracle.render(ow, vt.default_palette(), cam, params, threads=THREADS, row_step=step)
            rows = np.arange(0, cam.height, step)
            g = gpu.reshape(cam.height, cam.width)[rows].reshape(-1)
            r = ref.reshape(cam.height, cam.width)[rows].reshape(-1)
            compare(g, r)
            assert st["bounce_rays"] > 100000 and st["bounce_hits"] > 1000, ci
    finally:
        w.close()


def _batch_against_oracle(vt, ctx, oracle, picked, params, row_step):
    """One batch graph over the picked scenes' jobs; every row_step-th row of
    every job against the oracle.  Returns the rays checked."""
    worlds, jobs, owners = [], [], []
    try:
        for d, cams in picked:
            mats = vt.gen_world(d)
            w = vt.World(ctx, tuple(d.dims))
            w.upload_dense(mats)
            worlds.append(w)
            ow = oracle.OracleWorld(mats)
            for cam in cams:
                jobs.append((w, cam, ctx.alloc(cam.width * cam.height * 16)))
                owners.append(ow)
        batch = vt.Batch(ctx, jobs, params)
        batch.launch()
        ctx.sync()
        rays = 0
        for (w, cam, buf), ow in zip(jobs, owners):
            got = buf.download(np.zeros(cam.width * cam.height, vt.HIT_DTYPE))
            ref, st = oracle.render(ow, vt.default_palette(), cam, params, threads=THREADS, row_step=row_step)
            rows = np.arange(0, cam.height, row_step)
            compare(got.reshape(cam.height, cam.width)[rows].reshape(-1),
                    ref.reshape(cam.height, cam.width)[rows].reshape(-1))
            rays += st["primary_rays"] + st["shadow_rays"]
        batch.close()
        return rays
    finally:
        for _, _, buf in jobs:
            buf.free()
        for w in worlds:
            w.close()


def test_config3_large_scenes_batch_against_oracle(vt, ctx, oracle):
    """Every scene of the 64-scene batch workload above 300 voxels on a side
    (up to 512^3, where the chunk and brick jumps span farthest), all their
    cameras, as one batch graph: every 8th row of every job."""
    import scenes
    sc, params = scenes.config3()
    picked = [(d, cams) for d, cams in sc if d.dims[0] > 300]
    assert len(picked) >= 8 and max(d.dims[0] for d, _ in picked) > 450
    assert _batch_against_oracle(vt, ctx, oracle, picked, params, 8) > 2_000_000


def test_config3_batch_against_oracle_sampled_rows(vt, ctx, oracle):
    """The 64-scene batch workload's first scenes up to 300 voxels on a side
    (log-uniform cube worlds, 1-8 cameras each at 320x240 to 1920x1080), run
    as one batch graph: every 4th row of every job against the oracle, over a
    million rays in all."""
    import scenes
    sc, params = scenes.config3()
    picked = [(d, cams) for d, cams in sc if d.dims[0] <= 300][:8]
    assert _batch_against_oracle(vt, ctx, oracle, picked, params, 4) > 1_000_000


def test_config4_full_shading_step_against_fp64(vt, ctx, oracle):
    """The shading benchmark at full size: 256^3 world, 16 views of 512x512,
    targets rendered with the hidden palette and sun; one fused forward +
    backward over all views (vt_shade_backward_views) against the FP64
    gradient summed over the views (every element within 1e-4 relative, with
    the absolute floor of grad_close), and the forward image of every view
    against the FP64 colours."""
    from concurrent.futures import ThreadPoolExecutor
    import scenes
    desc, cams, (pal, alb, sun), (hpal, hsun) = scenes.config4()
    mats = vt.gen_world(desc)
    w = vt.World(ctx, tuple(desc.dims))
    bufs = []
    try:
        w.upload_dense(mats)
        n = cams[0].width * cams[0].height
        prim = vt.default_params(rays=vt.RAYS_PRIMARY, shade=vt.SHADE_NONE)
        hits = [ctx.alloc(n * 16) for _ in cams]
        targets = [ctx.alloc(n * 12) for _ in cams]
        rgbs = [ctx.alloc(n * 12) for _ in cams]
        bufs = hits + targets + rgbs
        for c, hb in zip(cams, hits):
            vt.render(ctx, w, c, prim, hb)
        hidden = vt.Shading(ctx, w, hpal, alb, hsun)
        for c, hb, tb in zip(cams, hits, targets):
            hidden.forward(c, hb, tb)
        hidden.close()
        sh = vt.Shading(ctx, w, pal, alb, sun)
        sh.zero_grad()
        sh.backward_views(cams, hits, targets)
        g = sh.grads()
        sh.forward_views(cams, hits, rgbs)
        ctx.sync()
        sh.close()
        recs = [hb.download(np.zeros(n, vt.HIT_DTYPE)) for hb in hits]
        tgts = [tb.download(np.zeros((n, 3), np.float32)) for tb in targets]
        imgs = [rb.download(np.zeros((n, 3), np.float32)) for rb in rgbs]
        ow = oracle.OracleWorld(mats)

        def ref(v):
            return oracle.shade_grad_f64(ow, cams[v], recs[v], pal, alb, sun, 0.2, 0.8, 512, tgts[v])

        loss, rpal, rsun, ralb, lit = 0.0, np.zeros((256, 3)), np.zeros(3), np.zeros(mats.size), 0
        apal, asun, aalb = np.zeros((256, 3)), np.zeros(3), np.zeros(mats.size)
        with ThreadPoolExecutor(max_workers=4) as ex:
            for img, r in zip(imgs, ex.map(ref, range(len(cams)))):
                assert np.abs(img - r["rgb"]).max() <= 1e-6
                loss += r["loss"]
                rpal += r["palette"]
                rsun += r["sun"]
                ralb += r["albedo"]
                apal += r["abs_palette"]
                asun += r["abs_sun"]
                aalb += r["abs_albedo"]
                lit += int((r["vis"] != 0).sum())
        assert g["loss"] == pytest.approx(loss, rel=1e-4)
        # element by element: 1e-4 relative, floor 1e-5 x the element's sum of |contributions|
        grad_close(g["palette"], rpal, apal, "palette")
        grad_close(g["sun"], rsun, asun, "sun")
        assert grad_close(g["albedo"], ralb, aalb, "albedo") > 100000
        assert lit > 100000
    finally:
        for b in bufs:
            b.free()
        w.close()
