"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loaded by tests/, __graft_entry__.smoke() and the CPU-baseline legs of
bench.py, as the checker and as the timed CPU baseline.  Nothing in the
library path imports it.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent / "unnamed-voxel-tracer_gb300"))
import vt  # noqa: E402  (struct layouts of include/vt.h)

import importlib.util  # noqa: E402

_spec = importlib.util.spec_from_file_location("vt_oracle_build", HERE / "build.py")
_build = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(_build)


class VtoWorld_t(C.Structure):
    _fields_ = [("dims", C.c_int32 * 3), ("mats", C.c_void_p), ("chunk_occ", C.c_void_p), ("chunks", C.c_int32 * 3),
                ("entities", C.c_void_p), ("n_entities", C.c_int32)]


class VtoTrace_t(C.Structure):
    _fields_ = [("hit", C.c_int32), ("voxel", C.c_uint32), ("cell", C.c_int32 * 3), ("t", C.c_float),
                ("face", C.c_int32), ("axis", C.c_int32), ("material", C.c_uint8), ("steps", C.c_int32),
                ("mask_words", C.c_uint64), ("coarse_words", C.c_uint64)]


class VtoRefWorld_t(C.Structure):
    _fields_ = [("chunks", C.c_void_p), ("data", C.c_void_p), ("ndata", C.c_uint64), ("atlas", C.c_void_p)]


class VtoRefHit_t(C.Structure):
    _fields_ = [("data", C.c_uint32), ("hit_pos", C.c_float * 3), ("normal", C.c_float * 3),
                ("iterations", C.c_int32)]


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        lib = C.CDLL(str(_build.build()))
        P = C.c_void_p
        lib.vto_world_init.argtypes = [C.POINTER(VtoWorld_t), C.POINTER(C.c_int32), P]
        lib.vto_world_init.restype = C.c_int32
        lib.vto_world_free.argtypes = [C.POINTER(VtoWorld_t)]
        lib.vto_trace_p.argtypes = [C.POINTER(VtoWorld_t), C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int32,
                                    C.POINTER(VtoTrace_t)]
        lib.vto_render.argtypes = [C.POINTER(VtoWorld_t), P, C.POINTER(vt.Camera_t), C.POINTER(vt.Params_t), P,
                                   C.c_int32, C.POINTER(vt.Stats_t)]
        lib.vto_render.restype = C.c_int32
        lib.vto_render_sampled.argtypes = [C.POINTER(VtoWorld_t), P, C.POINTER(vt.Camera_t),
                                           C.POINTER(vt.Params_t), P, C.c_int32, C.c_int32, C.POINTER(vt.Stats_t)]
        lib.vto_render_sampled.restype = C.c_int32
        lib.vto_trace_rays.argtypes = [C.POINTER(VtoWorld_t), P, P, C.c_int32, C.c_int32, P]
        lib.vto_sinf.argtypes = [C.c_float]
        lib.vto_sinf.restype = C.c_float
        lib.vto_cosf.argtypes = [C.c_float]
        lib.vto_cosf.restype = C.c_float
        lib.vto_tracemap.argtypes = [C.POINTER(VtoRefWorld_t), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                     C.c_int32, C.POINTER(VtoRefHit_t)]
        lib.vto_primary_r.argtypes = [C.POINTER(VtoRefWorld_t), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                      C.c_float, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32,
                                      C.POINTER(C.c_float), C.POINTER(VtoRefHit_t)]
        lib.vto_shade_grad_f64.argtypes = [C.POINTER(VtoWorld_t), C.POINTER(vt.Camera_t), P, P, P,
                                           C.POINTER(C.c_double), C.c_double, C.c_double, C.c_int32, P, P, P, P,
                                           P, P, P, C.POINTER(C.c_double), P, P, C.POINTER(C.c_double)]
        lib.vto_shade_grad_f64.restype = C.c_int32
        lib.vto_trace_entities.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_float,
                                           C.POINTER(VtoRefHit_t)]
        lib.vto_sky_ref.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float)]
        lib.vto_render_reference.argtypes = [C.POINTER(VtoRefWorld_t), C.POINTER(C.c_float),
                                             C.POINTER(C.c_float), C.c_float, C.c_int32, C.c_int32, P]
        lib.vto_edit_r.argtypes = [C.POINTER(VtoRefWorld_t), P, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                   C.c_int32, C.POINTER(VtoRefHit_t)]
        lib.vto_pick_p.argtypes = [C.POINTER(VtoWorld_t), C.POINTER(vt.Camera_t), C.c_int32, C.c_int32,
                                   C.POINTER(VtoTrace_t), C.POINTER(C.c_int32)]
        lib.vto_primary_rays.argtypes = [C.POINTER(vt.Camera_t), C.c_int32, P, P]
        lib.vto_primary_rays.restype = None
        G = C.POINTER(vt.GenDesc_t)
        lib.vto_gen_desc_init.argtypes = [G, C.c_int32, C.c_int32, C.c_int32, C.c_float, C.c_uint64]
        lib.vto_gen_desc_init.restype = None
        lib.vto_gen_world.argtypes = [G, P, C.c_size_t, C.c_int32]
        lib.vto_gen_world.restype = C.c_int32
        lib.vto_gen_height.argtypes = [G, C.c_int32, C.c_int32]
        lib.vto_gen_height.restype = C.c_int32
        lib.vto_gen_camera.argtypes = [G, C.c_uint64, C.c_int32, C.c_int32, C.POINTER(vt.Camera_t)]
        lib.vto_gen_camera.restype = C.c_int32
        lib.vto_default_palette.argtypes = [P]
        lib.vto_default_palette.restype = None
        lib.vto_gen_sun.argtypes = [C.c_uint64, C.POINTER(C.c_float)]
        lib.vto_gen_sun.restype = None
        _lib = lib
    return _lib


def primary_rays(cam, row_step: int = 1):
    """(origins, dirs) of the primary rays of every row_step-th row, (n, 3) float32."""
    rows = (cam.height + row_step - 1) // row_step
    o = np.zeros((rows * cam.width, 3), np.float32)
    d = np.zeros((rows * cam.width, 3), np.float32)
    load().vto_primary_rays(C.byref(cam), int(row_step), o.ctypes.data, d.ctypes.data)
    return o, d


# ------------------------------------------------ seeded scenes (vt_oracle_gen.c)
# The same scenes as the library's vt.gen_* helpers, without loading libvt.so.
def gen_desc(dims, scale: float = 1.0, seed: int = 0, trees: int = 0, caves: bool = False):
    d = vt.GenDesc_t()
    load().vto_gen_desc_init(C.byref(d), int(dims[0]), int(dims[1]), int(dims[2]), float(scale), int(seed))
    d.trees = int(trees)
    d.caves = 1 if caves else 0
    return d


def gen_world(desc, threads: int = 0) -> np.ndarray:
    X, Y, Z = desc.dims
    out = np.zeros((Z, Y, X), dtype=np.uint8)
    import os
    if load().vto_gen_world(C.byref(desc), out.ctypes.data, out.nbytes, threads or (os.cpu_count() or 1)) != 0:
        raise ValueError("bad generator description")
    return out


def gen_camera(desc, seed: int, width: int, height: int):
    cam = vt.Camera_t()
    if load().vto_gen_camera(C.byref(desc), int(seed), int(width), int(height), C.byref(cam)) != 0:
        raise ValueError("bad camera arguments")
    return cam


def gen_sun(seed: int):
    out = (C.c_float * 3)()
    load().vto_gen_sun(int(seed), out)
    return [float(v) for v in out]


def default_palette() -> np.ndarray:
    pal = np.zeros(256, np.uint32)
    load().vto_default_palette(pal.ctypes.data)
    return pal


def default_params(**kw):
    """vt_params_default's values (the reference's SUN_DIR, camera.glsl:8), as
    a vt.Params_t, with fields overridden by keyword."""
    p = vt.Params_t()
    p.max_steps, p.shadow_max_steps, p.bounce_max_steps = 512, 512, 256
    p.rays, p.shade, p.flags, p.seed = vt.RAYS_PRIMARY | vt.RAYS_SHADOW, vt.SHADE_REFERENCE, \
        vt.FLAG_CROSSHAIR | vt.FLAG_VIGNETTE, 0
    p.sun_dir = (C.c_float * 3)(7.52185881e-01, 6.58950984e-01, 7.52185881e-01)
    p.ambient, p.diffuse, p.bounce_weight = 0.2, 0.8, 0.3
    for k, v in kw.items():
        if k == "sun_dir":
            p.sun_dir = (C.c_float * 3)(*v)
        else:
            setattr(p, k, v)
    return p


class OracleWorld:
    """A dense mode-P world (uint8 array [z, y, x]) seen by the oracle."""

    def __init__(self, mats: np.ndarray, entities: np.ndarray | None = None):
        self.mats = np.ascontiguousarray(mats, dtype=np.uint8)
        Z, Y, X = self.mats.shape
        self.dims = (X, Y, Z)
        self.w = VtoWorld_t()
        dims = (C.c_int32 * 3)(X, Y, Z)
        if load().vto_world_init(C.byref(self.w), dims, self.mats.ctypes.data) != 0:
            raise MemoryError("oracle world init failed")
        if entities is not None:
            self.entities = np.ascontiguousarray(entities, dtype=np.float32).reshape(-1, 6)
            self.w.entities = self.entities.ctypes.data
            self.w.n_entities = self.entities.shape[0]

    def __del__(self):
        if _lib is not None and getattr(self, "w", None) is not None:
            _lib.vto_world_free(C.byref(self.w))
            self.w = None


def render(world: OracleWorld, palette: np.ndarray, cam, params, threads: int = 1, row_step: int = 1):
    """Returns (records[H*W] as vt.HIT_DTYPE, stats dict).  With row_step > 1
    only rows 0, row_step, 2*row_step, ... are rendered (others stay zero)."""
    lib = load()
    out = np.zeros(cam.width * cam.height, dtype=vt.HIT_DTYPE)
    pal = np.ascontiguousarray(palette, dtype=np.uint32)
    st = vt.Stats_t()
    rc = lib.vto_render_sampled(C.byref(world.w), pal.ctypes.data, C.byref(cam), C.byref(params),
                                out.ctypes.data, threads, row_step, C.byref(st))
    if rc != 0:
        raise RuntimeError("oracle render failed")
    return out, st.as_dict()


def trace_rays(world: OracleWorld, origins: np.ndarray, dirs: np.ndarray, max_steps: int) -> np.ndarray:
    origins = np.ascontiguousarray(origins, dtype=np.float32).reshape(-1, 3)
    dirs = np.ascontiguousarray(dirs, dtype=np.float32).reshape(-1, 3)
    out = np.zeros(origins.shape[0], dtype=vt.HIT_DTYPE)
    load().vto_trace_rays(C.byref(world.w), origins.ctypes.data, dirs.ctypes.data, origins.shape[0], max_steps,
                          out.ctypes.data)
    return out


def trace_one(world: OracleWorld, o, d, max_steps: int) -> VtoTrace_t:
    tr = VtoTrace_t()
    load().vto_trace_p(C.byref(world.w), (C.c_float * 3)(*o), (C.c_float * 3)(*d), max_steps, C.byref(tr))
    return tr


class OracleRefWorld:
    """The reference's world format: 64^3 chunk table, u32 bricks, 256^3 atlas."""

    def __init__(self, chunks: np.ndarray, data: np.ndarray, atlas: np.ndarray):
        self.chunks = np.ascontiguousarray(chunks, dtype=np.uint32)
        self.data = np.ascontiguousarray(data, dtype=np.uint32)
        self.atlas = np.ascontiguousarray(atlas, dtype=np.uint32)
        assert self.chunks.size == 64 ** 3 and self.atlas.size == 256 ** 3
        self.w = VtoRefWorld_t(self.chunks.ctypes.data, self.data.ctypes.data, self.data.size, self.atlas.ctypes.data)


def tracemap(world: OracleRefWorld, o, d, max_steps: int) -> VtoRefHit_t:
    h = VtoRefHit_t()
    load().vto_tracemap(C.byref(world.w), (C.c_float * 3)(*o), (C.c_float * 3)(*d), max_steps, C.byref(h))
    return h


def edit_r(world: OracleRefWorld, cam, edit_mode: int) -> VtoRefHit_t:
    """The editing pass on the reference world; writes into world.data."""
    h = VtoRefHit_t()
    load().vto_edit_r(C.byref(world.w), world.data.ctypes.data, (C.c_float * 4)(*cam.pos),
                      (C.c_float * 16)(*cam.view), edit_mode, C.byref(h))
    return h


def pick_p(world: OracleWorld, cam, max_steps: int, edit_mode: int = -1):
    """(trace, target {x, y, z, valid}) of the mode-P pick ray."""
    tr = VtoTrace_t()
    tgt = (C.c_int32 * 4)()
    load().vto_pick_p(C.byref(world.w), C.byref(cam), max_steps, edit_mode, C.byref(tr), tgt)
    return tr, list(tgt)


def shade_grad_f64(world: OracleWorld, cam, hits: np.ndarray, palette, albedo, sun, ambient: float, diffuse: float,
                   shadow_max_steps: int, target: np.ndarray | None = None, vis_in: np.ndarray | None = None) -> dict:
    """FP64 Lambert shading of one view and the exact gradient of
    L = sum (c - target)^2 over the fixed hit set (records from render)."""
    n = cam.width * cam.height
    X, Y, Z = world.dims
    pal = np.ascontiguousarray(palette, np.float64).reshape(768)
    alb = None if albedo is None else np.ascontiguousarray(albedo, np.float64).reshape(-1)
    hits = np.ascontiguousarray(hits)
    rgb = np.zeros(n * 3, np.float64)
    vis = np.zeros(n, np.uint8)
    loss = np.zeros(1, np.float64)
    g_pal = np.zeros(768, np.float64)
    g_alb = np.zeros(X * Y * Z, np.float64) if alb is not None else None
    g_sun = (C.c_double * 3)()
    a_pal = np.zeros(768, np.float64)
    a_alb = np.zeros(X * Y * Z, np.float64) if alb is not None else None
    a_sun = (C.c_double * 3)()
    tgt = None if target is None else np.ascontiguousarray(target, np.float32).reshape(-1)
    vin = None if vis_in is None else np.ascontiguousarray(vis_in, np.uint8).reshape(-1)
    rc = load().vto_shade_grad_f64(
        C.byref(world.w), C.byref(cam), hits.ctypes.data, pal.ctypes.data,
        alb.ctypes.data if alb is not None else None, (C.c_double * 3)(*sun), ambient, diffuse, shadow_max_steps,
        tgt.ctypes.data if tgt is not None else None, vin.ctypes.data if vin is not None else None, vis.ctypes.data,
        rgb.ctypes.data, loss.ctypes.data, g_pal.ctypes.data, g_alb.ctypes.data if g_alb is not None else None,
        g_sun, a_pal.ctypes.data, a_alb.ctypes.data if a_alb is not None else None, a_sun)
    if rc != 0:
        raise ValueError("bad shading arguments")
    # abs_*: per gradient element, the sum of |per-pixel contribution|
    return {"rgb": rgb.reshape(n, 3), "vis": vis, "loss": float(loss[0]), "palette": g_pal.reshape(256, 3),
            "albedo": g_alb, "sun": np.array(list(g_sun)), "abs_palette": a_pal.reshape(256, 3),
            "abs_albedo": a_alb, "abs_sun": np.array(list(a_sun))}


def render_reference(world: OracleRefWorld, cam) -> np.ndarray:
    """The reference's frame (primary + secondary + blit), vt.REF_PIXEL_DTYPE records."""
    out = np.zeros(cam.width * cam.height, dtype=vt.REF_PIXEL_DTYPE)
    load().vto_render_reference(C.byref(world.w), (C.c_float * 4)(*cam.pos), (C.c_float * 16)(*cam.view), cam.fov,
                                cam.width, cam.height, out.ctypes.data)
    return out


def trace_entities(o, d, max_distance: float) -> VtoRefHit_t:
    h = VtoRefHit_t()
    load().vto_trace_entities((C.c_float * 3)(*o), (C.c_float * 3)(*d), max_distance, C.byref(h))
    return h


def sky_ref(rd):
    out = (C.c_float * 4)()
    load().vto_sky_ref((C.c_float * 3)(*rd), out)
    return list(out)


def primary_r(world: OracleRefWorld, cam_pos, view, fov: float, px: int, py: int, width: int, height: int,
              max_steps: int = 192):
    """The reference's primary ray (primary.comp.glsl:31-43): (direction, hit)."""
    h = VtoRefHit_t()
    d = (C.c_float * 3)()
    load().vto_primary_r(C.byref(world.w), (C.c_float * 4)(*cam_pos), (C.c_float * 16)(*view), fov, px, py, width,
                         height, max_steps, d, C.byref(h))
    return [d[0], d[1], d[2]], h


# ---- the reference's own shader code compiled as C++ (oracle/_ref/libref.so),
# available where the reference sources are (built by oracle/build_ref.py)
REF_LIB = HERE / "_ref" / "libref.so"
_ref = None


def load_ref():
    """The compiled reference shaders, or None where they cannot be built."""
    global _ref
    if _ref is None:
        spec = importlib.util.spec_from_file_location("vt_ref_build", HERE / "build_ref.py")
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        if mod.build_if_available() is None or not REF_LIB.exists():
            return None
        lib = C.CDLL(str(REF_LIB))
        P, F = C.c_void_p, C.POINTER(C.c_float)
        lib.ref_set_world.argtypes = [P, P, P]
        lib.ref_trace_map.argtypes = [F, F, C.c_int32, C.POINTER(C.c_uint32), F, F]
        lib.ref_trace_entities.argtypes = [F, F, C.c_float, C.POINTER(C.c_uint32), F, F]
        lib.ref_sky.argtypes = [F, F, F]
        lib.ref_primary.argtypes = [F, F, C.c_float, C.c_int32, C.c_int32, C.c_int32, C.c_int32, F,
                                    C.POINTER(C.c_uint32), F, F]
        lib.ref_pick.argtypes = [F, F, C.POINTER(C.c_uint32), F, F]
        lib.ref_set_voxel.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_uint32]
        _ref = lib
    return _ref
