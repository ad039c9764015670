"""Benchmark: rays per second of the fused primary + shadow render path.

Workload (one step = one frame): a 512 x 256 x 512 voxel world in 32^3 chunks
(seeded value-noise fbm terrain + 200 trees), 1920 x 1080 primary rays plus
one shadow ray per hit toward a seeded sun, reference shading, max 512 steps
per ray; the step cycles over 8 seeded cameras.  The world is resident in HBM
before timing (the reference keeps it in persistently mapped buffers too);
L2 is flushed (256 MiB memset) between steps, outside the timed events.

    python bench.py [--gpus N --steps K --warmup W] [--impl ours|reference]

Rank 0 prints one JSON line.  After the headline it measures the other
workloads once each (small plain scene, the 4K cave world with bounce rays,
the 64-scene batch, the shading adjoint, the reference's own algorithm on the
GPU), each with its roofline and a CPU baseline.

--impl reference times the CPU oracle (a port of the reference's traversal;
the reference itself is GLSL behind OpenGL and has no CPU implementation) on
all host cores, on a bounded sample of each frame; it builds its scene with
the oracle's own generator and never loads the GPU library.
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
L2_PROBE_BYTES = 24 << 20


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


def setup_scene(gen, rank: int):
    """The headline scene from a generator module: the library's (vt) or the
    oracle's restatement (oracle_py); both give the same bytes."""
    desc = gen.gen_desc(WORLD, seed=SEED, trees=TREES)
    mats = gen.gen_world(desc)
    cams = [gen.gen_camera(desc, s + CAMERAS * rank, IMAGE[0], IMAGE[1]) for s in range(CAMERAS)]
    params = gen.default_params(rays=1 | 2, max_steps=512, shadow_max_steps=512, sun_dir=gen.gen_sun(SEED))
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


def roofline(abytes: float, seconds: float, peak: float, peak_kind: str, unit_note: str) -> dict:
    """Algorithmic bytes of one step over its kernel time, against the
    measured HBM copy rate."""
    achieved = abytes / seconds / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_kind": f"{peak_kind} hbm_gbs", "algorithmic_bytes_per_step": abytes, "bytes": unit_note}


RAY_BYTES = "8 x (brick words + chunk words consulted) + 1 per material read on a hit + 16 per record"


def ray_bytes(stats: dict) -> float:
    return 8.0 * stats["mask_words"] + 8.0 * stats["coarse_words"] + stats["material_bytes"] + stats["record_bytes"]


# ---------------------------------------------------------------- clocks
class Clocks:
    """SM clock and clock-event reasons through NVML (the driver's library,
    read-only queries), sampled where the caller asks: once per timed step,
    while that step's kernel runs.  Falls back to an nvidia-smi process
    sampling every 100 ms over the whole timed phase."""
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}
    SMI = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, cuda_index: int):
        self.samples, self.source, self.nv, self.h = [], None, None, C.c_void_p()
        self.proc = self.file = None
        self.max_mhz = None
        cvd = os.environ.get("CUDA_VISIBLE_DEVICES", "")
        try:
            idx = int(cvd.split(",")[cuda_index]) if cvd else cuda_index
        except (ValueError, IndexError):
            idx = cuda_index
        self.idx = idx
        try:
            nv = C.CDLL("libnvidia-ml.so.1")
            if nv.nvmlInit_v2() != 0:
                raise OSError("nvmlInit")
            count = C.c_uint()
            nv.nvmlDeviceGetCount_v2(C.byref(count))
            if count.value == 1:
                idx = 0
            if nv.nvmlDeviceGetHandleByIndex_v2(C.c_uint(idx), C.byref(self.h)) != 0:
                raise OSError("nvmlDeviceGetHandleByIndex")
            self.reasons_fn = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                nv.nvmlDeviceGetCurrentClocksThrottleReasons
            mx = C.c_uint()
            if nv.nvmlDeviceGetMaxClockInfo(self.h, 1, C.byref(mx)) == 0:   # NVML_CLOCK_SM
                self.max_mhz = float(mx.value)
            self.nv, self.source = nv, "nvml, one sample per timed step while it runs"
        except (OSError, AttributeError):
            self.nv = None

    def start(self):
        if self.nv is None:
            try:
                self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
                q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
                     "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                     "clocks_event_reasons.sw_power_cap")
                self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                              "-lms", "100", "-i", str(self.idx)], stdout=self.file,
                                             stderr=subprocess.DEVNULL)
                self.source = "nvidia-smi every 100 ms around the timed phase"
                time.sleep(0.3)
            except OSError:
                self.proc = None
        return self

    def sample(self):
        if self.nv is None:
            return
        mhz, reasons = C.c_uint(), C.c_ulonglong()
        if self.nv.nvmlDeviceGetClockInfo(self.h, 1, C.byref(mhz)) == 0 and \
                self.reasons_fn(self.h, C.byref(reasons)) == 0:
            self.samples.append((float(mhz.value), int(reasons.value)))

    def stop(self):
        if not self.proc:
            return
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        for row in Path(self.file.name).read_text().splitlines():
            r = [x.strip() for x in row.split(",")]
            if len(r) >= 6 and r[0].replace(".", "").isdigit():
                self.samples.append((float(r[0]), sum(1 << i for i in range(4) if r[2 + i].lower() == "active")))
                if r[1].replace(".", "").isdigit():
                    self.max_mhz = float(r[1])
        os.unlink(self.file.name)

    def summary(self):
        if not self.samples:
            return None
        if self.nv is not None:
            seen = sorted({name for _, bits in self.samples for b, name in self.REASONS.items() if bits & b})
        else:
            seen = sorted({self.SMI[i] for _, bits in self.samples for i in range(4) if bits >> i & 1})
        return {"sm_mhz": statistics.median(m for m, _ in self.samples), "sm_max_mhz": self.max_mhz,
                "reasons": seen, "samples": len(self.samples), "source": self.source}


# ----------------------------------------------------------- CPU baselines
def cpu_oracle_sample(oracle_py, ow, pal, cam, params, threads: int, target_s: float):
    """Rays/s of the CPU oracle (unit-step walk) on every k-th row of one
    frame, k sized so that the sample takes about target_s seconds.
    Returns (rays_per_s, description, rays of the whole frame)."""
    probe_step = 64
    kinds = ("primary_rays", "shadow_rays", "bounce_rays")
    t0 = time.perf_counter()
    _, st = oracle_py.render(ow, pal, cam, params, threads=threads, row_step=probe_step)
    dt = time.perf_counter() - t0
    rate = sum(st[k] for k in kinds) / max(dt, 1e-6)
    rays_per_row = sum(st[k] for k in kinds) / max(1, (cam.height + probe_step - 1) // probe_step)
    rows = max(threads, int(rate * target_s / max(rays_per_row, 1.0)))
    row_step = max(1, cam.height // rows)
    t0 = time.perf_counter()
    _, st = oracle_py.render(ow, pal, cam, params, threads=threads, row_step=row_step)
    dt = time.perf_counter() - t0
    rays = sum(st[k] for k in kinds)
    rows_done = (cam.height + row_step - 1) // row_step
    frame_rays = rays * cam.height / rows_done
    return rays / dt, (f"every {row_step}th row of a {cam.width}x{cam.height} frame ({rays} rays, {dt:.1f} s)"), \
        frame_rays


def host_walker():
    """The production traversal (trace_p.cuh) compiled for the host cores
    (tests/host/trace_host.cpp), or None where it cannot be built."""
    src = ROOT / "tests" / "host" / "trace_host.cpp"
    out = ROOT / "tests" / "host" / "_build" / "libtrace_host.so"
    deps = [src, PKG / "csrc" / "trace_p.cuh", PKG / "csrc" / "vt_internal.h"]
    inc = next((p for p in ("/usr/local/cuda/include", "/usr/local/cuda/targets/x86_64-linux/include",
                            "/usr/local/cuda/targets/sbsa-linux/include") if (Path(p) / "cuda_runtime.h").exists()),
               None)
    try:
        if not out.exists() or any(d.stat().st_mtime > out.stat().st_mtime for d in deps):
            if inc is None:
                return None
            out.parent.mkdir(exist_ok=True)
            subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", "-I",
                            inc, str(src), "-o", str(out)], check=True, capture_output=True)
        lib = C.CDLL(str(out))
    except (OSError, subprocess.CalledProcessError):
        return None
    lib.ht_world_new.restype = C.c_void_p
    lib.ht_world_new.argtypes = [C.POINTER(C.c_int32), C.c_void_p]
    lib.ht_world_free.argtypes = [C.c_void_p]
    lib.ht_frame_mt.restype = C.c_int64
    lib.ht_frame_mt.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.POINTER(C.c_float),
                                C.c_int32, C.c_int32, C.POINTER(C.c_int64)]
    return lib


def cpu_skipping_walk(oracle_py, mats, cams, params, threads: int, row_step: int = 4):
    """Rays/s of this library's own skipping walk (chunk and brick jumps) on
    the host cores, primary + shadow rays of every row_step-th row of each
    camera: the same algorithm as the GPU kernel, so that GPU over CPU
    compares hardware rather than algorithms."""
    lib = host_walker()
    if lib is None:
        return None
    Z, Y, X = mats.shape
    hw = lib.ht_world_new((C.c_int32 * 3)(X, Y, Z), np.ascontiguousarray(mats).ctypes.data)
    try:
        rays, secs = 0, 0.0
        sun = (C.c_float * 3)(*params.sun_dir)
        for cam in cams:
            o, d = oracle_py.primary_rays(cam, row_step)
            dark = C.c_int64()
            t0 = time.perf_counter()
            rays += lib.ht_frame_mt(hw, o.ctypes.data, d.ctypes.data, o.shape[0], params.max_steps, sun,
                                    params.shadow_max_steps, threads, C.byref(dark))
            secs += time.perf_counter() - t0
    finally:
        lib.ht_world_free(hw)
    return {"value": rays / secs / 1e9, "unit": "Grays/s", "cores": threads, "kind": "port",
            "sample": f"this library's skipping walk (chunk and brick jumps, trace_p.cuh built for the host), "
                      f"primary + shadow rays of every {row_step}th row of the {len(cams)} cameras "
                      f"({rays} rays, {secs:.1f} s)"}


# -------------------------------------------------------------- GPU legs
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


def _timed_flushed(torch, fn, reps: int, flush) -> float:
    """Mean ms of fn() over reps runs, each after an L2 flush and timed alone."""
    ms = 0.0
    for _ in range(reps):
        flush.zero_()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        fn()
        e.record()
        torch.cuda.synchronize()
        ms += s.elapsed_time(e)
    return ms / reps


def measure_config1_frames(vt, ctx, torch, flush) -> dict:
    """The headline frames alone (the 512x256x512 world, its 8 cameras at
    1920x1080, primary + shadow): 2 warm-up frames, then the 8 cameras once
    each after an L2 flush.  For profiling a tuning (--only config1 --tuning)."""
    _, mats, cams, params = setup_scene(vt, 0)
    w = vt.World(ctx, WORLD)
    w.upload_dense(mats)
    out = ctx.alloc(IMAGE[0] * IMAGE[1] * 16)
    sh = torch.cuda.current_stream().cuda_stream
    ms = []
    for i in range(2 + CAMERAS):
        def frame():
            ctx.check(ctx.lib.vt_render(ctx.handle, w.handle, C.byref(cams[i % CAMERAS]), C.byref(params), out.ptr,
                                        sh))
        if i < 2:
            frame()
        else:
            ms.append(_timed_flushed(torch, frame, 1, flush))
    w.close()
    out.free()
    return {"workload": workload_config()["workload"], "ms_per_frame": sum(ms) / len(ms), "tuning": ctx.get_tuning()}


def measure_config0(vt, scenes, ctx, torch, flush, peak, peak_kind, oracle_py, autotune: bool = True) -> dict:
    """128^3 terrain, 640x360 primary rays (max 512 steps): the small plain
    scene that the CPU oracle also renders whole."""
    desc, cams, params = scenes.config0()
    cam = cams[0]
    mats = vt.gen_world(desc)
    w = vt.World(ctx, tuple(desc.dims))
    w.upload_dense(mats)
    out = ctx.alloc(cam.width * cam.height * 16)
    sh = torch.cuda.current_stream().cuda_stream
    st = vt.render_stats(ctx, w, cam, params, sh)
    before = ctx.get_tuning()
    if autotune:
        tuning, _ = ctx.autotune(w, cam, params, reps=20)   # the library's own choice for this frame
    else:
        tuning = before

    def frame():
        ctx.check(ctx.lib.vt_render(ctx.handle, w.handle, C.byref(cam), C.byref(params), out.ptr, sh))

    for _ in range(3):
        frame()
    ms = _timed_flushed(torch, frame, 50, flush)
    ctx.set_tuning(**before)
    w.close()
    out.free()
    rays = st["primary_rays"]
    threads = os.cpu_count() or 1
    ow = oracle_py.OracleWorld(mats)
    t0 = time.perf_counter()
    _, cst = oracle_py.render(ow, vt.default_palette(), cam, params, threads=threads)
    dt = time.perf_counter() - t0
    return {"workload": "128^3 terrain (fbm, water), 640x360 primary rays, max 512 steps",
            "grays_per_s": rays / (ms * 1e-3) / 1e9, "ms_per_frame": ms, "rays_per_frame": rays,
            "l2": "flushed before each frame",
            "tuning": {"by": "vt_autotune on this frame" if autotune else "given", **tuning},
            "roofline": roofline(ray_bytes(st), ms * 1e-3, peak, peak_kind, RAY_BYTES),
            "cpu_baseline": {"value": cst["primary_rays"] / dt / 1e9, "unit": "Grays/s", "cores": threads,
                             "kind": "port", "sample": f"the whole frame ({cst['primary_rays']} rays, {dt:.2f} s)"}}


def measure_config2(vt, scenes, ctx, torch, flush, peak, peak_kind, oracle_py, autotune: bool = True) -> dict:
    """2048x256x2048 world with caves (1 GiB of materials, 128 MiB of mask
    words), 3840x2160 primary + shadow + bounce rays."""
    desc, cams, params = scenes.config2()
    w = vt.World(ctx, tuple(desc.dims))
    w.generate(desc)
    out = ctx.alloc(cams[0].width * cams[0].height * 16)
    sh = torch.cuda.current_stream().cuda_stream
    stats = [vt.render_stats(ctx, w, c, params, sh) for c in cams]
    rays = [s["primary_rays"] + s["shadow_rays"] + s["bounce_rays"] for s in stats]
    before = ctx.get_tuning()
    if autotune:
        tuning, _ = ctx.autotune(w, cams[0], params, reps=2)   # the library's own choice for this frame size
    else:
        tuning = before
    ms = []
    for c in cams:
        def frame():
            ctx.check(ctx.lib.vt_render(ctx.handle, w.handle, C.byref(c), C.byref(params), out.ptr, sh))
        frame()
        ms.append(_timed_flushed(torch, frame, 3, flush))
    ctx.set_tuning(**before)
    mats = w.download_dense()
    w.close()
    out.free()
    t = sum(ms) * 1e-3
    threads = os.cpu_count() or 1
    r, dsc, _ = cpu_oracle_sample(oracle_py, oracle_py.OracleWorld(mats), vt.default_palette(), cams[0], params,
                                  threads, 4.0)
    del mats
    return {"workload": "2048x256x2048 world + caves, 3840x2160, primary + shadow + 1 cosine bounce per hit",
            "grays_per_s": sum(rays) / t / 1e9, "ms_per_frame": sum(ms) / len(ms),
            "rays_per_frame": sum(rays) / len(rays), "l2": "flushed before each frame (the mask alone is 128 MiB)",
            "tuning": {"by": "vt_autotune on camera 0's frame" if autotune else "given", **tuning},
            "roofline": roofline(sum(ray_bytes(s) for s in stats) / len(stats), t / len(stats), peak, peak_kind,
                                 RAY_BYTES + ", bounce rays included"),
            "cpu_baseline": {"value": r / 1e9, "unit": "Grays/s", "cores": threads, "kind": "port",
                             "sample": "camera 0: " + dsc}}


def launch_floor(torch, n: int) -> dict:
    """Fixed costs of the launch structures, measured with trivial kernels
    (one-element adds) in CUDA graphs: n launches in sequence on one chain,
    and n launches spread over 8 concurrent chains."""
    def graph_of(chains: int) -> float:
        x = torch.zeros(chains, device="cuda")
        streams = [torch.cuda.Stream() for _ in range(chains)]
        g = torch.cuda.CUDAGraph()
        cap = torch.cuda.Stream()
        cap.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(cap):
            with torch.cuda.graph(g, stream=cap):
                cur = torch.cuda.current_stream()
                for s in streams:
                    s.wait_stream(cur)
                for j in range(n):
                    with torch.cuda.stream(streams[j % chains]):
                        x[j % chains:j % chains + 1].add_(1.0)
                for s in streams:
                    cur.wait_stream(s)
        torch.cuda.synchronize()
        return _timed(torch, g.replay, 20)
    return {"trivial_graph_one_chain_ms": graph_of(1), "trivial_graph_8_chains_ms": graph_of(8), "launches": n}


def measure_config3(vt, scenes, ctx, torch, peak, peak_kind, oracle_py) -> dict:
    """64 cube scenes (edge log-uniform in [32, 512]) x 1-8 cameras: one
    CUDA-graph launch of the batch vs one vt_render launch per camera.  The
    default batch graph holds one launch per world (all its cameras); the
    per-job shape (one launch per camera on 8 concurrent chains) and the
    queue shape (one persistent kernel over 16x16 units) are timed too."""
    sc, params = scenes.config3()
    worlds, jobs = [], []
    for desc, cams in sc:
        w = vt.World(ctx, tuple(desc.dims))
        w.generate(desc)
        worlds.append((w, desc))
        for c in cams:
            jobs.append((w, c, ctx.alloc(c.width * c.height * 16)))
    sh = torch.cuda.current_stream().cuda_stream

    def per_scene():
        for w, c, buf in jobs:
            ctx.check(ctx.lib.vt_render(ctx.handle, w.handle, C.byref(c), C.byref(params), buf.ptr, sh))

    def shape_ms(kernel: int) -> float:
        ctx.set_tuning(kernel=kernel)
        b = vt.Batch(ctx, jobs, params)
        b.launch(sh)                     # captured with this tuning
        ctx.set_tuning()
        ms = _timed(torch, lambda: b.launch(sh), 3)
        b.close()
        return ms

    per_scene()
    t_scene = _timed(torch, per_scene, 3)
    t_batch = shape_ms(vt.KERNEL_TILE)
    t_per_job = shape_ms(vt.KERNEL_PER_JOB)
    t_queue = shape_ms(vt.KERNEL_QUEUE)
    pixels = sum(c.width * c.height for _, c, _ in jobs)
    abytes, rays = 0.0, 0
    for w, c, _ in jobs:
        s = vt.render_stats(ctx, w, c, params, sh)
        abytes += ray_bytes(s)
        rays += s["primary_rays"] + s["shadow_rays"]
    floor = launch_floor(torch, len(jobs))
    # CPU: the oracle on sampled rows of the first jobs, about 4 s
    threads = os.cpu_count() or 1
    crays, csecs, used = 0.0, 0.0, 0
    cur = None
    for w, c, _ in jobs:
        if csecs > 4.0:
            break
        if cur is None or cur[0] is not w:
            desc = next(d for ww, d in worlds if ww is w)
            cur = (w, oracle_py.OracleWorld(vt.gen_world(desc)))
        r, _, fr = cpu_oracle_sample(oracle_py, cur[1], vt.default_palette(), c, params, threads, 0.5)
        crays += fr
        csecs += fr / r
        used += 1
    for _, _, buf in jobs:
        buf.free()
    for w, _ in worlds:
        w.close()
    return {"workload": f"{len(sc)} scenes, {len(jobs)} cameras, {pixels / 1e6:.1f} Mpixels, primary + shadow",
            "batched_gpix_per_s": pixels / (t_batch * 1e-3) / 1e9,
            "per_scene_gpix_per_s": pixels / (t_scene * 1e-3) / 1e9,
            "batched_grays_per_s": rays / (t_batch * 1e-3) / 1e9,
            "batched_ms": t_batch, "per_scene_ms": t_scene, "speedup": t_scene / t_batch,
            "batched_per_job_gpix_per_s": pixels / (t_per_job * 1e-3) / 1e9, "batched_per_job_ms": t_per_job,
            "batched_queue_gpix_per_s": pixels / (t_queue * 1e-3) / 1e9, "batched_queue_ms": t_queue,
            "launches_per_scene_path": len(jobs), "launch_floor": floor,
            "roofline": roofline(abytes, t_batch * 1e-3, peak, peak_kind, RAY_BYTES + ", all jobs of the batch"),
            "cpu_baseline": {"value": crays / csecs / 1e9, "unit": "Grays/s", "cores": threads, "kind": "port",
                             "sample": f"sampled rows of the first {used} jobs ({csecs:.1f} s extrapolated "
                                       f"to whole frames)"}}


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


def measure_config4(vt, scenes, ctx, torch, peak, peak_kind, oracle_py) -> dict:
    """256^3 world, 16 views at 512x512: one optimisation step = fused
    forward + backward of the shading (shadow rays recomputed) over all views,
    one vt_shade_backward_views call."""
    desc, cams, (pal, alb, sun), (hpal, hsun) = scenes.config4()
    mats = vt.gen_world(desc)
    w = vt.World(ctx, tuple(desc.dims))
    w.upload_dense(mats)
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
    # algorithmic bytes of one step: per pixel the 16-byte record and the
    # 12-byte target; per hit the 4-byte albedo read, 12 + 4 bytes of
    # palette and albedo gradient, and the recomputed shadow ray's words
    stream = torch.cuda.current_stream().cuda_stream
    both = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW, sun_dir=[float(v) for v in sun])
    px, hitn, shadow_words = 0, 0, 0
    for c in cams:
        a = vt.render_stats(ctx, w, c, prim, stream)
        b = vt.render_stats(ctx, w, c, both, stream)
        px += c.width * c.height
        hitn += a["primary_hits"]
        shadow_words += (b["mask_words"] + b["coarse_words"]) - (a["mask_words"] + a["coarse_words"])
    abytes = 28.0 * px + 20.0 * hitn + 8.0 * shadow_words
    # CPU: the FP64 oracle gradient (the adjoint's checker) of 8 views, one thread per view
    views = 8
    recs = [hb.download(np.zeros(n, vt.HIT_DTYPE)) for hb in hits[:views]]
    tgts = [tb.download(np.zeros((n, 3), np.float32)) for tb in targets[:views]]
    for b in hits + targets + rgbs:
        b.free()
    w.close()
    from concurrent.futures import ThreadPoolExecutor
    ow = oracle_py.OracleWorld(mats)
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=views) as ex:
        list(ex.map(lambda v: oracle_py.shade_grad_f64(ow, cams[v], recs[v], pal, alb, sun, 0.2, 0.8, 512, tgts[v]),
                    range(views)))
    cpu_s = time.perf_counter() - t0
    return {"workload": "256^3 world, 16 views at 512x512, Lambert + shadowed sun, L2 image loss",
            "fwd_bwd_ms_per_iter": t_step, "fwd_ms_per_iter": t_fwd, "loss": loss,
            "roofline": roofline(abytes, t_step * 1e-3, peak, peak_kind,
                                 "per pixel 16 (record) + 12 (target); per hit 4 (albedo) + 16 (palette and albedo "
                                 "gradient) + 8 x the recomputed shadow ray's brick and chunk words"),
            "cpu_baseline": {"value": cpu_s * 1e3 * len(cams) / views, "unit": "ms per fwd+bwd iteration",
                             "higher_is_better": False, "cores": views, "kind": "port",
                             "sample": f"the FP64 oracle gradient of {views} of the {len(cams)} views, one thread "
                                       f"each ({cpu_s:.1f} s), scaled to {len(cams)} views"}}


# -------------------------------------------------------------- the arms
def run_reference(args, rank: int, world: int) -> None:
    """The reference's traversal on the CPU (the oracle port: the reference
    itself is GLSL behind OpenGL), on all host cores, sampled per frame.  Its
    scene comes from the oracle's generator: no GPU library is loaded."""
    if rank != 0:
        return
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle_py
    _, mats, cams, params = setup_scene(oracle_py, 0)
    threads = os.cpu_count() or 1
    ow = oracle_py.OracleWorld(mats)
    pal = oracle_py.default_palette()
    per_step = max(2.0, 20.0 / max(1, args.steps + args.warmup))
    for i in range(args.warmup):
        cpu_oracle_sample(oracle_py, ow, pal, cams[i % CAMERAS], params, threads, per_step)
    rays, secs, descs = 0.0, 0.0, []
    for i in range(args.steps):
        r, dsc, frame_rays = cpu_oracle_sample(oracle_py, ow, pal, cams[i % CAMERAS], params, threads, per_step)
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
    abytes = [ray_bytes(s) for s in stats]

    def frame(i):
        ctx.check(ctx.lib.vt_render(ctx.handle, wobj.handle, C.byref(cams[i % CAMERAS]), C.byref(params),
                                    out.data_ptr(), sh))

    for i in range(args.warmup):
        flush.zero_()
        frame(i)
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clk = Clocks(local_rank).start()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    for i in range(args.steps):
        flush.zero_()
        starts[i].record(stream)
        frame(i)
        ends[i].record(stream)
        clk.sample()        # while this step's flush and frame run
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clk.stop()
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
    l2 = ctx.read_bandwidth(L2_PROBE_BYTES, 400)
    hbm_read = ctx.read_bandwidth(4 << 30, 4)
    cpu = None
    extra = {}
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle_py
    if world == 1:
        threads = os.cpu_count() or 1
        ow = oracle_py.OracleWorld(mats)
        pal = vt.default_palette()
        rays_c, secs_c = 0.0, 0.0
        for cam in cams:   # the bench's 8 cameras, each sampled to ~1 s (a whole frame if it is faster)
            r, _, fr = cpu_oracle_sample(oracle_py, ow, pal, cam, params, threads, 8.0 / len(cams))
            rays_c += fr
            secs_c += fr / r
        del ow
        cpu = {"value": rays_c / secs_c / 1e9, "unit": "Grays/s", "cores": threads, "kind": "port",
               "sample": f"the unit-step oracle on the 8 bench cameras at 1920x1080, each on every k-th row sized "
                         f"to ~1 s of CPU work; {secs_c:.1f} s in total, rates extrapolated per frame",
               "skipping_walk": cpu_skipping_walk(oracle_py, mats, cams, params, threads)}
    name, sms = ctx.device_info()
    # the other configurations, measured once each (not part of the timed steps)
    if world == 1 and not args.headline_only:
        import scenes
        wobj.close()
        wobj = None
        for key, fn in (("config0", lambda: measure_config0(vt, scenes, ctx, torch, flush, peak, peak_kind,
                                                             oracle_py)),
                        ("mode_r", lambda: measure_mode_r(vt, ctx, torch, mats, cams, flush)),
                        ("config2", lambda: measure_config2(vt, scenes, ctx, torch, flush, peak, peak_kind,
                                                            oracle_py)),
                        ("config3", lambda: measure_config3(vt, scenes, ctx, torch, peak, peak_kind, oracle_py)),
                        ("config4", lambda: measure_config4(vt, scenes, ctx, torch, peak, peak_kind, oracle_py))):
            try:
                extra[key] = fn()
            except Exception as exc:  # report, keep the headline line
                extra[key] = {"error": f"{type(exc).__name__}: {exc}"}
    line = {
        "metric": "Grays/s", "value": value, "unit": "Grays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": workload_config(),
        "gpu_launches": args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_kind": f"{peak_kind} hbm_gbs",
                     "algorithmic_bytes_per_step": total_bytes / args.steps, "bytes": RAY_BYTES,
                     "traffic_note": traffic_note},
        "roofline_l2": {"achieved": achieved, "peak": l2, "unit": "GB/s", "frac": achieved / l2,
                        "peak_kind": "this run: the library's read probe (vt_probe_read_bandwidth), 16-byte "
                                     "L2-only loads over a 24 MiB buffer, 400 passes in one launch",
                        "hbm_read_gbs": hbm_read},
        "rays_per_step": job_rays / args.steps,
        "per_ray": {k: sum(s[k] for s in stats) / sum(rays) for k in ("steps", "iterations", "mask_words",
                                                                       "coarse_words")},
        # unit crossings per second (a jump over an empty box counts every crossing it skips)
        "steps_per_s": value * 1e9 * sum(s["steps"] for s in stats) / sum(rays),
        "e2e": {"value": e2e_value, "unit": "Grays/s",
                "h2d_bytes_per_step": C.sizeof(vt.Camera_t) + C.sizeof(vt.Params_t), "d2h_bytes_per_step": nbytes,
                "note": "vt_render_host into pinned host memory: camera and params travel in the launch; the kernel "
                        "writes the records across the host link"},
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
                    help="skip the other workloads' measurements that follow the headline")
    ap.add_argument("--only", choices=["config0", "config1", "config2", "config3", "config4"],
                    help="run just one workload and print its result (for profiling)")
    ap.add_argument("--tuning", default="",
                    help="with --only: vt_tuning fields for the context, e.g. share_bricks=1,l2_persist=1 "
                         "(--only runs never autotune)")
    args = ap.parse_args()
    if args.only:
        import torch
        sys.path.insert(0, str(PKG))
        sys.path.insert(0, str(ROOT / "oracle"))
        _load("vt_build", PKG / "build.py").build()
        import oracle_py
        import scenes
        import vt
        ctx = vt.Context(0)
        if args.tuning:
            ctx.set_tuning(**{k: int(v) for k, v in (kv.split("=") for kv in args.tuning.split(","))})
        peak, kind = read_peaks()
        flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device="cuda")
        fixed = True   # profiling: the given tuning (or the default) as it is, launch order fixed
        fn = {"config0": lambda: measure_config0(vt, scenes, ctx, torch, flush, peak, kind, oracle_py, not fixed),
              "config1": lambda: measure_config1_frames(vt, ctx, torch, flush),
              "config2": lambda: measure_config2(vt, scenes, ctx, torch, flush, peak, kind, oracle_py, not fixed),
              "config3": lambda: measure_config3(vt, scenes, ctx, torch, peak, kind, oracle_py),
              "config4": lambda: measure_config4(vt, scenes, ctx, torch, peak, kind, oracle_py)}[args.only]
        print(json.dumps({"only": args.only, **fn()}), flush=True)
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
