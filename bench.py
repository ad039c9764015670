"""Benchmark: rays per second of the fused primary + shadow render path.

Workload (one step = one frame): a 512 x 256 x 512 voxel world in 32^3 chunks
(seeded value-noise fbm terrain + 200 trees), 1920 x 1080 primary rays plus
one shadow ray per hit toward a seeded sun, reference shading, max 512 steps
per ray; the step cycles over 8 seeded cameras.  The world is resident in HBM
before timing (the reference keeps it in persistently mapped buffers too);
L2 is flushed (256 MiB memset) between steps, outside the timed events.

    python bench.py [--gpus N --steps K --warmup W] [--impl ours|reference]

Rank 0 prints one JSON line.  --impl reference times the CPU oracle (a port of
the reference's traversal; the reference itself is GLSL behind OpenGL and has
no CPU implementation) on all host cores, on a bounded sample of each frame.
"""
from __future__ import annotations

import argparse
import ctypes as C
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "unnamed-voxel-tracer_gb300"

WORLD = (512, 256, 512)
IMAGE = (1920, 1080)
TREES = 200
SEED = 1
CAMERAS = 8
FLUSH_BYTES = 256 << 20


def _load(name: str, path: Path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def workload_config() -> dict:
    return {"workload": "512x256x512 voxel world (fbm terrain + 200 trees, 32^3 chunks), 1920x1080 primary + "
                        "1 shadow ray per hit, reference shading, max 512 steps, 8 seeded cameras",
            "world": list(WORLD), "image": list(IMAGE), "rays": "primary+shadow", "cameras": CAMERAS,
            "l2": "flushed between steps (256 MiB memset outside the timed events)",
            "parallelism": "replicas"}


def setup_scene(vt, rank: int):
    desc = vt.gen_desc(WORLD, seed=SEED, trees=TREES)
    mats = vt.gen_world(desc)
    cams = [vt.gen_camera(desc, s + CAMERAS * rank, IMAGE[0], IMAGE[1]) for s in range(CAMERAS)]
    params = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW, max_steps=512, shadow_max_steps=512,
                               sun_dir=vt.gen_sun(SEED))
    return desc, mats, cams, params


def read_peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def read_traffic():
    """DRAM bytes per launch of the render kernel from the committed ncu summary."""
    p = ROOT / "profiles" / "render_traffic.json"
    if not p.exists():
        return None, None
    try:
        d = json.loads(p.read_text())
        return float(d["dram_bytes_per_launch"]), d.get("note")
    except Exception:
        return None, None


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)], stdout=self.file,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.proc or not self.file:
            return None
        self.file.flush()
        rows = [r.split(", ") for r in Path(self.file.name).read_text().strip().splitlines() if r.strip()]
        try:
            os.unlink(self.file.name)
        except OSError:
            pass
        rows = [r for r in rows if len(r) >= 9]
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip().lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": float(rows[0][2]) if rows[0][2].replace(".", "").isdigit() else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_oracle_sample(vt, oracle_py, mats, cam, params, threads: int, target_s: float):
    """Rays/s of the CPU oracle on every row_step-th row of one frame, sized to
    take about target_s seconds.  Returns (rays_per_s, description)."""
    ow = oracle_py.OracleWorld(mats)
    pal = vt.default_palette()
    probe_step = 64
    t0 = time.perf_counter()
    _, st = oracle_py.render(ow, pal, cam, params, threads=threads, row_step=probe_step)
    dt = time.perf_counter() - t0
    rate = (st["primary_rays"] + st["shadow_rays"]) / max(dt, 1e-6)
    rays_per_row = (st["primary_rays"] + st["shadow_rays"]) / max(1, (cam.height + probe_step - 1) // probe_step)
    rows = max(threads, int(rate * target_s / max(rays_per_row, 1.0)))
    row_step = max(1, cam.height // rows)
    t0 = time.perf_counter()
    _, st = oracle_py.render(ow, pal, cam, params, threads=threads, row_step=row_step)
    dt = time.perf_counter() - t0
    rays = st["primary_rays"] + st["shadow_rays"]
    rows_done = (cam.height + row_step - 1) // row_step
    frame_rays = rays * cam.height / rows_done
    return rays / dt, (f"every {row_step}th row of a 1920x1080 frame ({st['primary_rays']} primary + "
                       f"{st['shadow_rays']} shadow rays, {dt:.1f} s)"), frame_rays


def run_reference(args, rank: int, world: int) -> None:
    if rank != 0:
        return
    sys.path.insert(0, str(PKG))
    _load("vt_build", PKG / "build.py").build()
    import vt
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle_py
    _, mats, cams, params = setup_scene(vt, 0)
    threads = os.cpu_count() or 1
    per_step = max(2.0, 20.0 / max(1, args.steps + args.warmup))
    for i in range(args.warmup):
        cpu_oracle_sample(vt, oracle_py, mats, cams[i % CAMERAS], params, threads, per_step)
    rays, secs, descs = 0.0, 0.0, []
    for i in range(args.steps):
        r, dsc, frame_rays = cpu_oracle_sample(vt, oracle_py, mats, cams[i % CAMERAS], params, threads, per_step)
        rays += frame_rays
        secs += frame_rays / r
        descs.append(dsc)
    value = rays / secs / 1e9
    line = {"impl": "reference", "metric": "Grays/s", "value": value, "unit": "Grays/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(),
            "cpu_baseline": {"value": value, "unit": "Grays/s", "cores": threads, "kind": "port",
                             "sample": descs[0]},
            "e2e": {"value": value, "unit": "Grays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def aggregate(torch, dist, world: int, device, rays: float, ms: float, e2e_s: float) -> tuple[float, float, float]:
    """Whole-job totals of a replica run: rays summed over ranks, device and
    end-to-end times maxed over ranks (the job ends with its slowest rank)."""
    if world == 1:
        return rays, ms, e2e_s
    r = torch.tensor([rays], dtype=torch.float64, device=device)
    t = torch.tensor([ms, e2e_s], dtype=torch.float64, device=device)
    dist.all_reduce(r, op=dist.ReduceOp.SUM)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(r[0]), float(t[0]), float(t[1])


def _timed(torch, fn, reps: int) -> float:
    """Mean ms of fn() over reps runs, CUDA events on the current stream."""
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    s.record()
    for _ in range(reps):
        fn()
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / reps


def measure_config2(vt, scenes, ctx, torch, flush) -> dict:
    """2048x256x2048 world with caves (1 GiB of materials, 128 MiB of mask
    words: at the L2 size), 3840x2160 primary + shadow + bounce rays."""
    desc, cams, params = scenes.config2()
    w = vt.World(ctx, tuple(desc.dims))
    w.upload_dense(vt.gen_world(desc))
    out = ctx.alloc(cams[0].width * cams[0].height * 16)
    sh = torch.cuda.current_stream().cuda_stream
    stats = [vt.render_stats(ctx, w, c, params, sh) for c in cams]
    rays = [s["primary_rays"] + s["shadow_rays"] + s["bounce_rays"] for s in stats]
    abytes = [8 * s["mask_words"] + 8 * s["coarse_words"] + s["material_bytes"] + s["record_bytes"] for s in stats]
    ms = []
    for i, c in enumerate(cams):
        def frame():
            ctx.check(ctx.lib.vt_render(ctx.handle, w.handle, C.byref(c), C.byref(params), out.ptr, sh))
        frame()
        flush.zero_()
        ms.append(_timed(torch, frame, 1))
    w.close()
    out.free()
    t = sum(ms) * 1e-3
    return {"workload": "2048x256x2048 world + caves, 3840x2160, primary + shadow + 1 cosine bounce per hit",
            "grays_per_s": sum(rays) / t / 1e9, "ms_per_frame": sum(ms) / len(ms),
            "rays_per_frame": sum(rays) / len(rays), "algorithmic_gbs": sum(abytes) / t / 1e9,
            "l2": "flushed before each frame"}


def measure_config3(vt, scenes, ctx, torch) -> dict:
    """64 cube scenes (edge log-uniform in [32, 512]) x 1-8 cameras: one
    CUDA-graph launch of the batch vs one vt_render launch per camera.  The
    default batch graph holds the per-camera launches on 8 concurrent chains;
    the queue shape (one persistent kernel over 16x16 units) is timed too."""
    sc, params = scenes.config3()
    worlds, jobs = [], []
    for desc, cams in sc:
        w = vt.World(ctx, tuple(desc.dims))
        w.upload_dense(vt.gen_world(desc))
        worlds.append(w)
        for c in cams:
            jobs.append((w, c, ctx.alloc(c.width * c.height * 16)))
    sh = torch.cuda.current_stream().cuda_stream

    def per_scene():
        for w, c, buf in jobs:
            ctx.check(ctx.lib.vt_render(ctx.handle, w.handle, C.byref(c), C.byref(params), buf.ptr, sh))

    batch = vt.Batch(ctx, jobs, params)
    per_scene()
    batch.launch(sh)
    t_scene = _timed(torch, per_scene, 3)
    t_batch = _timed(torch, lambda: batch.launch(sh), 3)
    pixels = batch.info()["pixels"]
    batch.close()
    ctx.set_tuning(kernel=vt.KERNEL_QUEUE)
    qbatch = vt.Batch(ctx, jobs, params)
    qbatch.launch(sh)
    ctx.set_tuning()
    t_queue = _timed(torch, lambda: qbatch.launch(sh), 3)
    qbatch.close()
    for _, _, buf in jobs:
        buf.free()
    for w in worlds:
        w.close()
    return {"workload": f"{len(sc)} scenes, {len(jobs)} cameras, {pixels / 1e6:.1f} Mpixels, primary + shadow",
            "batched_gpix_per_s": pixels / (t_batch * 1e-3) / 1e9,
            "per_scene_gpix_per_s": pixels / (t_scene * 1e-3) / 1e9,
            "batched_ms": t_batch, "per_scene_ms": t_scene, "speedup": t_scene / t_batch,
            "batched_queue_gpix_per_s": pixels / (t_queue * 1e-3) / 1e9,
            "launches_per_scene_path": len(jobs)}


def measure_mode_r(vt, ctx, torch, mats, cams, flush) -> dict:
    """The reference's own algorithm on the GPU: the same world in the
    reference's format (64^3 chunk table, 8^3 u32 bricks, 8 sub-voxel models
    of 8^3 RGBA8) and the same cameras, one vt_render_reference frame each
    (traceMap stepping one voxel or sub-voxel per iteration, 192 iterations
    for primary and 48 for shadow rays, map.glsl:83-168, secondary.comp.glsl)."""
    import brickmap
    sys.path.insert(0, str(ROOT / "tests"))
    import refworld   # the seeded sub-voxel models of the tests
    rng = np.random.default_rng(SEED)
    chunks, data = brickmap.build_map(mats, np.arange(256, dtype=np.uint32) % 8)
    bm = vt.Brickmap(ctx)
    bm.upload(chunks, data)
    bm.set_atlas(brickmap.build_atlas(refworld.random_models(rng, 8)), 8)
    out = ctx.alloc(IMAGE[0] * IMAGE[1] * 32)
    sh = torch.cuda.current_stream().cuda_stream

    def frame(i):
        ctx.check(ctx.lib.vt_render_reference(ctx.handle, bm.handle, C.byref(cams[i % len(cams)]), out.ptr, sh))

    for i in range(3):
        frame(i)
    ms = 0.0
    for i in range(16):
        flush.zero_()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        frame(i)
        e.record()
        torch.cuda.synchronize()
        ms += s.elapsed_time(e) / 16
    bm.close()
    out.free()
    return {"workload": "the 512x256x512 world in the reference's format with 8 sub-voxel models, the 8 bench "
                        "cameras, 1920x1080, the reference's frame (primary + shadow + composite)",
            "gpix_per_s": IMAGE[0] * IMAGE[1] / (ms * 1e-3) / 1e9, "ms_per_frame": ms,
            "note": "the reference's algorithm restated bit-exactly on the GPU; L2 flushed before each frame, "
                    "outside the timed events"}


def measure_config4(vt, scenes, ctx, torch) -> dict:
    """256^3 world, 16 views at 512x512: one optimisation step = fused
    forward + backward of the shading (shadow rays recomputed) over all views,
    one vt_shade_backward_views call."""
    desc, cams, (pal, alb, sun), (hpal, hsun) = scenes.config4()
    w = vt.World(ctx, tuple(desc.dims))
    w.upload_dense(vt.gen_world(desc))
    prim = vt.default_params(rays=vt.RAYS_PRIMARY, shade=vt.SHADE_NONE)
    n = cams[0].width * cams[0].height
    hits = [ctx.alloc(n * 16) for _ in cams]
    for c, hb in zip(cams, hits):
        vt.render(ctx, w, c, prim, hb)
    targets = [ctx.alloc(n * 12) for _ in cams]
    hidden = vt.Shading(ctx, w, hpal, alb, hsun)
    for c, hb, tb in zip(cams, hits, targets):
        hidden.forward(c, hb, tb)
    hidden.close()
    sh_ = vt.Shading(ctx, w, pal, alb, sun)
    rgbs = [ctx.alloc(n * 12) for _ in cams]

    def step():
        sh_.zero_grad_async()
        sh_.backward_views(cams, hits, targets)

    def forward():
        sh_.forward_views(cams, hits, rgbs)

    step()
    t_step = _timed(torch, step, 5)
    t_fwd = _timed(torch, forward, 5)
    loss = sh_.grads()["loss"]
    sh_.close()
    for b in hits + targets + rgbs:
        b.free()
    w.close()
    return {"workload": "256^3 world, 16 views at 512x512, Lambert + shadowed sun, L2 image loss",
            "fwd_bwd_ms_per_iter": t_step, "fwd_ms_per_iter": t_fwd, "loss": loss}


def measure_l2_gbs(torch, dev) -> float:
    """Read+write GB/s of a 24 MiB copy held in L2 (many passes)."""
    a = torch.empty(24 << 20, dtype=torch.uint8, device=dev)
    b = torch.empty_like(a)
    for _ in range(10):
        b.copy_(a)
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    s.record()
    n = 200
    for _ in range(n):
        b.copy_(a)
    e.record()
    torch.cuda.synchronize()
    return 2 * a.numel() * n / (s.elapsed_time(e) * 1e-3) / 1e9


def run_ours(args, rank: int, world: int, local_rank: int) -> None:
    import torch
    import torch.distributed as dist

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    sys.path.insert(0, str(PKG))
    _load("vt_build", PKG / "build.py").build()
    import vt

    ctx = vt.Context(local_rank)
    _, mats, cams, params = setup_scene(vt, rank)
    wobj = vt.World(ctx, WORLD)
    wobj.upload_dense(mats)
    ctx.sync()
    out = torch.empty(IMAGE[0] * IMAGE[1] * 16, dtype=torch.uint8, device=dev)
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream

    # algorithmic bytes and ray counts per camera (instrumented kernel, untimed)
    stats = [vt.render_stats(ctx, wobj, c, params, sh) for c in cams]
    rays = [s["primary_rays"] + s["shadow_rays"] for s in stats]
    abytes = [8 * s["mask_words"] + 8 * s["coarse_words"] + s["material_bytes"] + s["record_bytes"] for s in stats]

    def frame(i):
        ctx.check(ctx.lib.vt_render(ctx.handle, wobj.handle, C.byref(cams[i % CAMERAS]), C.byref(params),
                                    out.data_ptr(), sh))

    for i in range(args.warmup):
        flush.zero_()
        frame(i)
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clk:
        for i in range(args.steps):
            flush.zero_()
            starts[i].record(stream)
            frame(i)
            ends[i].record(stream)
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
    kernel_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = sum(kernel_ms)
    total_rays = sum(rays[i % CAMERAS] for i in range(args.steps))
    total_bytes = sum(abytes[i % CAMERAS] for i in range(args.steps))
    ctx.sync(sh)

    # end to end through the C ABI with host output (pinned), copies inside
    hbuf = C.c_void_p()
    nbytes = IMAGE[0] * IMAGE[1] * 16
    ctx.check(ctx.lib.vt_host_alloc_pinned(ctx.handle, nbytes, C.byref(hbuf)))
    e2e_s = 0.0
    for i in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.check(ctx.lib.vt_render_host(ctx.handle, wobj.handle, C.byref(cams[i % CAMERAS]), C.byref(params),
                                         hbuf.value))
        if i >= args.warmup:
            e2e_s += time.perf_counter() - t0
    ctx.lib.vt_host_free_pinned(ctx.handle, hbuf)

    job_rays, total_ms, e2e_s = aggregate(torch, dist, world, dev, total_rays, total_ms, e2e_s)
    value = job_rays / (total_ms * 1e-3) / 1e9
    e2e_value = job_rays / e2e_s / 1e9

    if rank != 0:
        return
    peak, peak_kind = read_peaks()
    achieved = total_bytes / (total_ms * 1e-3) / 1e9
    traffic, traffic_note = read_traffic()
    l2 = measure_l2_gbs(torch, dev)
    cpu = None
    if world == 1:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle_py
        threads = os.cpu_count() or 1
        rays_c, secs_c = 0.0, 0.0
        for cam in cams:   # the bench's 8 cameras, each sampled to ~1.5 s (a whole frame if it is faster)
            r, _, fr = cpu_oracle_sample(vt, oracle_py, mats, cam, params, threads, 12.0 / len(cams))
            rays_c += fr
            secs_c += fr / r
        cpu = {"value": rays_c / secs_c / 1e9, "unit": "Grays/s", "cores": threads, "kind": "port",
               "sample": f"the 8 bench cameras at 1920x1080, each on every k-th row sized to ~1.5 s of CPU work "
                         f"(all rows when a frame takes less); {secs_c:.1f} s in total, rates extrapolated per frame"}
    name, sms = ctx.device_info()
    # the other configurations, measured once each (not part of the timed steps)
    extra = {}
    if world == 1 and not args.headline_only:
        import scenes
        wobj.close()
        for key, fn in (("mode_r", lambda: measure_mode_r(vt, ctx, torch, mats, cams, flush)),
                        ("config2", lambda: measure_config2(vt, scenes, ctx, torch, flush)),
                        ("config3", lambda: measure_config3(vt, scenes, ctx, torch)),
                        ("config4", lambda: measure_config4(vt, scenes, ctx, torch))):
            try:
                extra[key] = fn()
            except Exception as exc:  # report, keep the headline line
                extra[key] = {"error": f"{type(exc).__name__}: {exc}"}
        wobj = None
    line = {
        "metric": "Grays/s", "value": value, "unit": "Grays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": workload_config(),
        "gpu_launches": args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_kind": f"{peak_kind} hbm_gbs",
                     "algorithmic_bytes_per_step": total_bytes / args.steps, "traffic_note": traffic_note},
        "roofline_l2": {"achieved": achieved, "peak": l2, "unit": "GB/s", "frac": achieved / l2,
                        "peak_kind": "24 MiB device copy held in L2, read+write bytes, this run"},
        "rays_per_step": job_rays / args.steps,
        "per_ray": {k: sum(s[k] for s in stats) / sum(rays) for k in ("steps", "iterations", "mask_words",
                                                                       "coarse_words")},
        # unit crossings per second (a jump over an empty box counts every crossing it skips)
        "steps_per_s": value * 1e9 * sum(s["steps"] for s in stats) / sum(rays),
        "e2e": {"value": e2e_value, "unit": "Grays/s", "h2d_bytes_per_step": C.sizeof(vt.Camera_t) + C.sizeof(vt.Params_t),
                "d2h_bytes_per_step": nbytes,
                "note": "vt_render_host into pinned host memory: camera and params travel in the launch; the kernel writes the records across the host link"},
        "cpu_baseline": cpu, "clocks": clk.summary(), "device": {"name": name, "sms": sms},
        **extra,
    }
    print(json.dumps(line), flush=True)
    if wobj is not None:
        wobj.close()
    ctx.close()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--headline-only", action="store_true",
                    help="skip the config 2/3/4 measurements that follow the headline")
    ap.add_argument("--only", choices=["config2", "config3", "config4"],
                    help="run just one of the other configurations and print its result (for profiling)")
    args = ap.parse_args()
    if args.only:
        import torch
        sys.path.insert(0, str(PKG))
        _load("vt_build", PKG / "build.py").build()
        import scenes
        import vt
        ctx = vt.Context(0)
        if args.only == "config2":
            res = measure_config2(vt, scenes, ctx, torch, torch.empty(FLUSH_BYTES, dtype=torch.uint8, device="cuda"))
        elif args.only == "config3":
            res = measure_config3(vt, scenes, ctx, torch)
        else:
            res = measure_config4(vt, scenes, ctx, torch)
        print(json.dumps({"only": args.only, **res}), flush=True)
        ctx.close()
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
