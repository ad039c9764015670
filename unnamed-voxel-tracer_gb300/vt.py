"""Python host for libvt (include/vt.h) over ctypes.

Mirrors the reference engine's render-path API so that a host written against
the reference reads the same here:

    reference (Zig)                                   here
    VoxelBrickmap(dim, ch).init/set/get/clear          World(ctx, dims).set/get/clear/upload_dense/upload_chunk
        src/engine/voxel.zig:25-82
    Camera.set_pos/rotate/as_uniform_data              Camera(...).set_pos/rotate/as_uniform_data
        src/engine/graphics/camera.zig:5-44
    Game.render (primary + secondary + blit)           render(ctx, world, camera, params, out)
        src/game.zig:232-256

Every call goes to the CUDA library; there is no CPU path.  A missing or
unloadable libvt.so raises immediately.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "lib" / "libvt.so"

# ---------------------------------------------------------------- constants
VT_OK = 0
VT_ERR_OOM = 2
STATUS_NAMES = {0: "VT_OK", 1: "VT_ERR_ARG", 2: "VT_ERR_OOM", 3: "VT_ERR_CUDA", 4: "VT_ERR_DEVICE_OOB",
                5: "VT_ERR_TIMEOUT", 6: "VT_ERR_NO_DEVICE", 7: "VT_ERR_FORMAT", 8: "VT_ERR_STATE"}
RAYS_PRIMARY, RAYS_SHADOW, RAYS_BOUNCE = 1, 2, 4
SHADE_NONE, SHADE_REFERENCE, SHADE_LAMBERT = 0, 1, 2
FLAG_CROSSHAIR, FLAG_VIGNETTE, FLAG_CHECKED = 1, 2, 4
KERNEL_TILE, KERNEL_QUEUE, KERNEL_PER_JOB = 0, 1, 2
HIT_PRIMARY, HIT_SHADOWED, HIT_BOUNCE, HIT_ENTITY = 1, 2, 4, 8


class Camera_t(C.Structure):
    _fields_ = [("pos", C.c_float * 4), ("view", C.c_float * 16), ("fov", C.c_float),
                ("tan_half_fov", C.c_float), ("width", C.c_int32), ("height", C.c_int32)]


class Params_t(C.Structure):
    _fields_ = [("max_steps", C.c_int32), ("shadow_max_steps", C.c_int32), ("bounce_max_steps", C.c_int32),
                ("rays", C.c_uint32), ("shade", C.c_uint32), ("flags", C.c_uint32), ("seed", C.c_uint32),
                ("sun_dir", C.c_float * 3), ("ambient", C.c_float), ("diffuse", C.c_float),
                ("bounce_weight", C.c_float)]


class Stats_t(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in (
        "primary_rays", "primary_hits", "shadow_rays", "shadow_hits", "bounce_rays", "bounce_hits",
        "mask_words", "coarse_words", "material_bytes", "record_bytes", "steps", "iterations")]

    def as_dict(self) -> dict:
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


class Tuning_t(C.Structure):
    _fields_ = [("kernel", C.c_int32), ("warp_tile_w", C.c_int32), ("occupancy", C.c_int32), ("batch", C.c_int32),
                ("share_bricks", C.c_int32), ("l2_persist", C.c_int32), ("bounce_refill", C.c_int32),
                ("bounce_walk", C.c_int32), ("bounce_sort", C.c_int32)]

    def as_dict(self) -> dict:
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


class ShadeInputs_t(C.Structure):
    _fields_ = [("d_palette", C.c_void_p), ("d_albedo", C.c_void_p), ("sun", C.c_float * 3),
                ("ambient", C.c_float), ("diffuse", C.c_float), ("shadow_max_steps", C.c_int32)]


class Job_t(C.Structure):
    _fields_ = [("world", C.c_void_p), ("camera", Camera_t), ("d_out", C.c_void_p)]


class WorldDesc_t(C.Structure):
    _fields_ = [("dims", C.c_int32 * 3)]


class WorldInfo_t(C.Structure):
    _fields_ = [("dims", C.c_int32 * 3), ("chunks", C.c_int32 * 3), ("mask_bytes", C.c_uint64),
                ("material_bytes", C.c_uint64), ("coarse_bytes", C.c_uint64), ("d_mask", C.c_void_p),
                ("d_materials", C.c_void_p), ("d_coarse", C.c_void_p)]


class GenDesc_t(C.Structure):
    _fields_ = [("dims", C.c_int32 * 3), ("base_height", C.c_float), ("amplitude", C.c_float),
                ("period", C.c_float), ("water_level", C.c_float), ("camera_height", C.c_float),
                ("octaves", C.c_int32), ("trees", C.c_int32), ("caves", C.c_int32),
                ("cave_threshold", C.c_float), ("cave_period", C.c_float), ("seed", C.c_uint64)]


# numpy view of vt_hit (16 bytes)
HIT_DTYPE = np.dtype([("voxel", "<u4"), ("t", "<f4"), ("rgba", "<u4"), ("face", "u1"), ("material", "u1"),
                      ("flags", "u1"), ("pad", "u1")])
assert HIT_DTYPE.itemsize == 16

_P = C.c_void_p
_S = C.c_int32
_SIGNATURES = {
    "vt_abi_version": (C.c_int32, []),
    "vt_status_string": (C.c_char_p, [_S]),
    "vt_ctx_create": (_S, [C.c_int32, C.POINTER(_P)]),
    "vt_ctx_destroy": (_S, [_P]),
    "vt_last_error_string": (C.c_char_p, [_P]),
    "vt_sync": (_S, [_P, _P]),
    "vt_wait": (_S, [_P, _P, C.c_int64]),
    "vt_debug_fail_alloc": (None, [C.c_int64]),
    "vt_debug_alloc_counts": (None, [C.POINTER(C.c_uint64), C.POINTER(C.c_int64)]),
    "vt_device_info": (_S, [_P, C.c_char_p, C.c_int32, C.POINTER(C.c_int32)]),
    "vt_device_alloc": (_S, [_P, C.c_size_t, C.POINTER(_P)]),
    "vt_device_free": (_S, [_P, _P]),
    "vt_host_alloc_pinned": (_S, [_P, C.c_size_t, C.POINTER(_P)]),
    "vt_host_free_pinned": (_S, [_P, _P]),
    "vt_memcpy_h2d": (_S, [_P, _P, _P, C.c_size_t, _P]),
    "vt_memcpy_d2h": (_S, [_P, _P, _P, C.c_size_t, _P]),
    "vt_memset_d": (_S, [_P, _P, C.c_int32, C.c_size_t, _P]),
    "vt_stream_create": (_S, [_P, C.POINTER(_P)]),
    "vt_stream_destroy": (_S, [_P, _P]),
    "vt_world_create": (_S, [_P, C.POINTER(WorldDesc_t), C.POINTER(_P)]),
    "vt_world_destroy": (_S, [_P]),
    "vt_world_clear": (_S, [_P, _P]),
    "vt_world_upload_dense": (_S, [_P, _P, C.c_size_t, _P]),
    "vt_world_upload_chunk": (_S, [_P, C.c_int32, C.c_int32, C.c_int32, _P, _P]),
    "vt_world_set_voxel": (_S, [_P, C.c_int32, C.c_int32, C.c_int32, C.c_uint8, _P]),
    "vt_world_get_voxel": (_S, [_P, C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_uint8)]),
    "vt_world_download_dense": (_S, [_P, _P, C.c_size_t, _P]),
    "vt_world_set_entities": (_S, [_P, _P, C.c_int32]),
    "vt_world_set_palette": (_S, [_P, _P]),
    "vt_world_get_info": (_S, [_P, C.POINTER(WorldInfo_t)]),
    "vt_camera_look": (_S, [C.POINTER(C.c_float), C.c_float, C.c_float, C.c_float, C.c_int32, C.c_int32,
                            C.POINTER(Camera_t)]),
    "vt_params_default": (None, [C.POINTER(Params_t)]),
    "vt_render": (_S, [_P, _P, C.POINTER(Camera_t), C.POINTER(Params_t), _P, _P]),
    "vt_render_host": (_S, [_P, _P, C.POINTER(Camera_t), C.POINTER(Params_t), _P]),
    "vt_render_host_static": (_S, [_P, _P, C.POINTER(Camera_t), C.POINTER(Params_t), _P]),
    "vt_render_stats": (_S, [_P, _P, C.POINTER(Camera_t), C.POINTER(Params_t), C.POINTER(Stats_t), _P]),
    "vt_trace_rays": (_S, [_P, _P, _P, _P, C.c_int32, C.c_int32, _P, _P]),
    "vt_shade_forward": (_S, [_P, _P, C.POINTER(Camera_t), _P, C.POINTER(ShadeInputs_t), _P, _P, _P, _P]),
    "vt_shade_backward": (_S, [_P, _P, C.POINTER(Camera_t), _P, C.POINTER(ShadeInputs_t), _P, _P, _P, _P, _P, _P]),
    "vt_shade_forward_views": (_S, [_P, _P, C.c_int32, C.POINTER(Camera_t), _P, C.POINTER(ShadeInputs_t), _P, _P]),
    "vt_shade_backward_views": (_S, [_P, _P, C.c_int32, C.POINTER(Camera_t), _P, C.POINTER(ShadeInputs_t), _P, _P,
                                     _P, _P, _P, _P]),
    "vt_brickmap_create": (_S, [_P, C.POINTER(_P)]),
    "vt_brickmap_destroy": (_S, [_P]),
    "vt_brickmap_upload": (_S, [_P, _P, _P, C.c_size_t]),
    "vt_brickmap_set_model": (_S, [_P, C.c_int32, _P]),
    "vt_brickmap_load_vox": (_S, [_P, _P, C.c_size_t, C.POINTER(C.c_int32)]),
    "vt_vox_decode": (_S, [_P, C.c_size_t, _P, C.c_int32, C.POINTER(C.c_int32)]),
    "vt_trace_map": (_S, [_P, _P, _P, _P, C.c_int32, C.c_int32, _P, _P]),
    "vt_render_reference": (_S, [_P, _P, C.POINTER(Camera_t), _P, _P]),
    "vt_brickmap_edit": (_S, [_P, _P, C.POINTER(Camera_t), C.c_int32, _P, _P]),
    "vt_brickmap_download": (_S, [_P, _P, _P, C.c_size_t]),
    "vt_pick": (_S, [_P, _P, C.POINTER(Camera_t), C.c_int32, _P]),
    "vt_edit": (_S, [_P, _P, C.POINTER(Camera_t), C.c_int32, C.c_int32, _P, _P]),
    "vt_world_download_distances": (_S, [_P, _P, C.c_size_t, _P, C.c_size_t]),
    "vt_batch_create": (_S, [_P, C.POINTER(Job_t), C.c_int32, C.POINTER(Params_t), C.POINTER(_P)]),
    "vt_batch_launch": (_S, [_P, _P]),
    "vt_batch_destroy": (_S, [_P]),
    "vt_batch_info": (_S, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_int32), C.POINTER(C.c_uint32)]),
    "vt_batch_autotune": (_S, [_P, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_float)]),
    "vt_probe_read_bandwidth": (_S, [_P, C.c_uint64, C.c_int32, C.POINTER(C.c_float)]),
    "vt_set_tuning": (_S, [_P, C.POINTER(Tuning_t)]),
    "vt_get_tuning": (_S, [_P, C.POINTER(Tuning_t)]),
    "vt_autotune": (_S, [_P, _P, C.POINTER(Camera_t), C.POINTER(Params_t), C.c_int32, C.c_char_p,
                         C.POINTER(Tuning_t), C.POINTER(C.c_float)]),
    "vt_gen_desc_init": (None, [C.POINTER(GenDesc_t), C.c_int32, C.c_int32, C.c_int32, C.c_float, C.c_uint64]),
    "vt_gen_world": (_S, [C.POINTER(GenDesc_t), _P, C.c_size_t, C.c_int32]),
    "vt_gen_height": (C.c_int32, [C.POINTER(GenDesc_t), C.c_int32, C.c_int32]),
    "vt_procgen_reference": (_S, [C.c_int32, C.c_float, C.c_float, _P, C.c_uint64, _P, _P, C.c_size_t,
                                  C.POINTER(C.c_size_t)]),
    "vt_world_generate": (_S, [_P, C.POINTER(GenDesc_t), _P]),
    "vt_gen_camera": (_S, [C.POINTER(GenDesc_t), C.c_uint64, C.c_int32, C.c_int32, C.POINTER(Camera_t)]),
    "vt_default_palette": (_S, [_P]),
    "vt_gen_sun": (_S, [C.c_uint64, C.POINTER(C.c_float)]),
}

_lib = None


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Loads libvt.so; raises if it is missing (no fallback exists)."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"libvt.so not found at {p}: build it with __graft_entry__.build() "
                           f"(python unnamed-voxel-tracer_gb300/build.py)")
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class VTError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def _check(status: int, ctx=None) -> None:
    if status != VT_OK:
        lib = load()
        msg = lib.vt_last_error_string(ctx).decode() if ctx else lib.vt_status_string(status).decode()
        raise VTError(status, msg)


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


# ------------------------------------------------------------------ context
class Context:
    """One CUDA device; owns the library context (vt_ctx)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = C.c_void_p()
        st = self.lib.vt_ctx_create(device, C.byref(h))
        if st != VT_OK:
            raise VTError(st, self.lib.vt_status_string(st).decode())
        self.handle = h

    def close(self) -> None:
        if self.handle:
            self.lib.vt_ctx_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def check(self, st: int) -> None:
        _check(st, self.handle)

    def sync(self, stream=None) -> None:
        self.check(self.lib.vt_sync(self.handle, stream))

    def wait(self, timeout_us: int, stream=None) -> bool:
        """vt_wait: True once `stream` is done (device status checked), False
        if it is still busy after timeout_us microseconds."""
        st = self.lib.vt_wait(self.handle, stream, int(timeout_us))
        if st == 5:   # VT_ERR_TIMEOUT
            return False
        self.check(st)
        return True

    def set_tuning(self, kernel: int = KERNEL_TILE, warp_tile_w: int = 8, occupancy: int = 1,
                   batch: int = 16, share_bricks: int = 0, l2_persist: int = 0, bounce_refill: int = 0,
                   bounce_walk: int = 0, bounce_sort: int = 0) -> None:
        t = Tuning_t(kernel, warp_tile_w, occupancy, batch, share_bricks, l2_persist, bounce_refill, bounce_walk,
                     bounce_sort)
        self.check(self.lib.vt_set_tuning(self.handle, C.byref(t)))

    def get_tuning(self) -> dict:
        t = Tuning_t()
        self.check(self.lib.vt_get_tuning(self.handle, C.byref(t)))
        return t.as_dict()

    def autotune(self, world: "World", cam, params, reps: int = 5, cache_path: str | None = None):
        """Times every launch configuration on this frame and keeps the fastest."""
        t = Tuning_t()
        ms = C.c_float()
        self.check(self.lib.vt_autotune(self.handle, world.handle, C.byref(cam), C.byref(params), reps,
                                        cache_path.encode() if cache_path else None, C.byref(t), C.byref(ms)))
        return t.as_dict(), float(ms.value)

    def read_bandwidth(self, nbytes: int, passes: int) -> float:
        """GB/s of the library's read probe over a buffer of nbytes, passes times."""
        g = C.c_float()
        self.check(self.lib.vt_probe_read_bandwidth(self.handle, int(nbytes), int(passes), C.byref(g)))
        return g.value

    def device_info(self) -> tuple[str, int]:
        buf = C.create_string_buffer(256)
        sms = C.c_int32()
        self.check(self.lib.vt_device_info(self.handle, buf, 256, C.byref(sms)))
        return buf.value.decode(), sms.value

    # device memory helpers
    def alloc(self, nbytes: int) -> "DeviceBuffer":
        return DeviceBuffer(self, nbytes)

    def stream(self) -> int:
        s = C.c_void_p()
        self.check(self.lib.vt_stream_create(self.handle, C.byref(s)))
        return s.value


class DeviceBuffer:
    def __init__(self, ctx: Context, nbytes: int):
        self.ctx, self.nbytes = ctx, int(nbytes)
        p = C.c_void_p()
        ctx.check(ctx.lib.vt_device_alloc(ctx.handle, self.nbytes, C.byref(p)))
        self.ptr = p.value

    def upload(self, a: np.ndarray, stream=None) -> None:
        a = np.ascontiguousarray(a)
        assert a.nbytes <= self.nbytes
        self.ctx.check(self.ctx.lib.vt_memcpy_h2d(self.ctx.handle, self.ptr, _ptr(a), a.nbytes, stream))
        self.ctx.sync(stream)

    def download(self, out: np.ndarray, stream=None) -> np.ndarray:
        assert out.flags.c_contiguous and out.nbytes <= self.nbytes
        self.ctx.check(self.ctx.lib.vt_memcpy_d2h(self.ctx.handle, _ptr(out), self.ptr, out.nbytes, stream))
        self.ctx.sync(stream)
        return out

    def zero(self, stream=None) -> None:
        self.ctx.check(self.ctx.lib.vt_memset_d(self.ctx.handle, self.ptr, 0, self.nbytes, stream))

    def free(self) -> None:
        if self.ptr:
            self.ctx.lib.vt_device_free(self.ctx.handle, self.ptr)
            self.ptr = None


class PinnedBuffer:
    """Page-locked host memory (vt_host_alloc_pinned) seen as a numpy array."""

    def __init__(self, ctx: Context, count: int, dtype):
        self.ctx, dtype = ctx, np.dtype(dtype)
        p = C.c_void_p()
        ctx.check(ctx.lib.vt_host_alloc_pinned(ctx.handle, max(1, count * dtype.itemsize), C.byref(p)))
        self.ptr = p.value
        raw = (C.c_uint8 * (count * dtype.itemsize)).from_address(self.ptr)
        self.array = np.frombuffer(raw, dtype=dtype, count=count)

    def free(self) -> None:
        if self.ptr:
            self.array = None
            self.ctx.lib.vt_host_free_pinned(self.ctx.handle, self.ptr)
            self.ptr = None


# -------------------------------------------------------------------- world
class World:
    """Mode-P voxel world on the device (VoxelBrickmap, voxel.zig:25-82)."""

    def __init__(self, ctx: Context, dims):
        self.ctx = ctx
        self.dims = tuple(int(d) for d in dims)
        desc = WorldDesc_t((C.c_int32 * 3)(*self.dims))
        h = C.c_void_p()
        ctx.check(ctx.lib.vt_world_create(ctx.handle, C.byref(desc), C.byref(h)))
        self.handle = h

    def close(self) -> None:
        if self.handle:
            self.ctx.lib.vt_world_destroy(self.handle)
            self.handle = None

    def upload_dense(self, mats: np.ndarray, stream=None) -> None:
        """mats: uint8 array indexed [z, y, x] (x fastest), shape (Z, Y, X)."""
        X, Y, Z = self.dims
        mats = np.ascontiguousarray(mats, dtype=np.uint8)
        if mats.shape != (Z, Y, X):
            raise ValueError(f"expected shape {(Z, Y, X)}, got {mats.shape}")
        self.ctx.check(self.ctx.lib.vt_world_upload_dense(self.handle, _ptr(mats), mats.nbytes, stream))

    def upload_chunk(self, cx: int, cy: int, cz: int, chunk: np.ndarray, stream=None) -> None:
        chunk = np.ascontiguousarray(chunk, dtype=np.uint8)
        if chunk.size != 32 ** 3:
            raise ValueError("a chunk is 32^3 bytes")
        self.ctx.check(self.ctx.lib.vt_world_upload_chunk(self.handle, cx, cy, cz, _ptr(chunk), stream))

    def set(self, x: int, y: int, z: int, material: int, stream=None) -> None:
        self.ctx.check(self.ctx.lib.vt_world_set_voxel(self.handle, x, y, z, material, stream))

    def get(self, x: int, y: int, z: int) -> int:
        m = C.c_uint8()
        self.ctx.check(self.ctx.lib.vt_world_get_voxel(self.handle, x, y, z, C.byref(m)))
        return int(m.value)

    def download_dense(self, stream=None) -> np.ndarray:
        """The whole grid as a uint8 array indexed [z, y, x]."""
        X, Y, Z = self.dims
        out = np.empty((Z, Y, X), dtype=np.uint8)
        self.ctx.check(self.ctx.lib.vt_world_download_dense(self.handle, _ptr(out), out.nbytes, stream))
        return out

    def generate(self, desc: "GenDesc_t", stream=None) -> None:
        """Generates the scene `desc` on the device (same bytes as gen_world)."""
        self.ctx.check(self.ctx.lib.vt_world_generate(self.handle, C.byref(desc), stream))

    def clear(self, stream=None) -> None:
        self.ctx.check(self.ctx.lib.vt_world_clear(self.handle, stream))

    def set_entities(self, boxes) -> None:
        """Entity occluders of the shadow pass: (n, 6) boxes {lo xyz, hi xyz}."""
        b = np.ascontiguousarray(boxes if boxes is not None else np.zeros((0, 6)), dtype=np.float32).reshape(-1, 6)
        self.ctx.check(self.ctx.lib.vt_world_set_entities(self.handle, _ptr(b) if b.size else None, b.shape[0]))

    def pick(self, cam: Camera_t, max_steps: int) -> np.ndarray:
        """The centre-of-view pick ray's hit record (vt_pick)."""
        out = np.zeros(1, dtype=HIT_DTYPE)
        self.ctx.check(self.ctx.lib.vt_pick(self.ctx.handle, self.handle, C.byref(cam), int(max_steps), _ptr(out)))
        return out[0]

    def edit(self, cam: Camera_t, max_steps: int, edit_mode: int, d_out=None, stream=None) -> None:
        """Pick and edit on the device (vt_edit); d_out: optional DeviceBuffer."""
        self.ctx.check(self.ctx.lib.vt_edit(self.ctx.handle, self.handle, C.byref(cam), int(max_steps), int(edit_mode),
                                            d_out.ptr if d_out is not None else None, stream))

    def distances(self):
        """(brick distances [8, nchunks*512], chunk distances [8, nchunks]) as
        uint8, one row per direction octant."""
        i = self.info()
        nch = i.chunks[0] * i.chunks[1] * i.chunks[2]
        b, c = np.zeros((8, nch * 512), np.uint8), np.zeros((8, nch), np.uint8)
        self.ctx.check(self.ctx.lib.vt_world_download_distances(self.handle, _ptr(b), b.nbytes, _ptr(c), c.nbytes))
        return b, c

    def set_palette(self, rgba: np.ndarray) -> None:
        rgba = np.ascontiguousarray(rgba, dtype=np.uint32)
        assert rgba.size == 256
        self.ctx.check(self.ctx.lib.vt_world_set_palette(self.handle, _ptr(rgba)))

    def info(self) -> WorldInfo_t:
        info = WorldInfo_t()
        self.ctx.check(self.ctx.lib.vt_world_get_info(self.handle, C.byref(info)))
        return info


# ------------------------------------------------------------------- camera
class Camera:
    """Camera.set_pos / rotate / as_uniform_data (camera.zig:5-44).

    yaw and pitch in radians; a negative pitch looks down.  rotate() applies
    mouse deltas with the reference's 0.001 gain and pitch clamp.
    """

    def __init__(self, pos=(0.0, 0.0, 0.0), yaw=0.0, pitch=0.0, fov=math.pi / 2, width=1280, height=720):
        self.pos = [float(p) for p in pos]
        self.yaw, self.pitch, self.fov = float(yaw), float(pitch), float(fov)
        self.width, self.height = int(width), int(height)

    def set_pos(self, pos) -> None:
        self.pos = [float(p) for p in pos]

    def rotate(self, pitch_delta: float, yaw_delta: float) -> None:
        self.pitch = min(max(self.pitch + pitch_delta * 0.001, -math.pi / 2), math.pi / 2)
        self.yaw = self.yaw + yaw_delta * 0.001

    def as_uniform_data(self) -> Camera_t:
        lib = load()
        cam = Camera_t()
        pos = (C.c_float * 3)(*self.pos)
        _check(lib.vt_camera_look(pos, self.yaw, self.pitch, self.fov, self.width, self.height, C.byref(cam)))
        return cam


def fail_alloc(n: int) -> None:
    """Testing hook: the n-th next allocation of the library fails (0 disarms)."""
    load().vt_debug_fail_alloc(int(n))


def alloc_counts() -> tuple[int, int]:
    """(allocations made, allocations live) by the library, process-wide."""
    made, live = C.c_uint64(), C.c_int64()
    load().vt_debug_alloc_counts(C.byref(made), C.byref(live))
    return made.value, live.value


def default_params(**kw) -> Params_t:
    p = Params_t()
    load().vt_params_default(C.byref(p))
    for k, v in kw.items():
        if k == "sun_dir":
            p.sun_dir = (C.c_float * 3)(*v)
        else:
            setattr(p, k, v)
    return p


def render(ctx: Context, world: World, cam: Camera_t, params: Params_t, d_out: DeviceBuffer, stream=None) -> None:
    """Game.render: one fused launch writing width*height vt_hit records."""
    assert d_out.nbytes >= cam.width * cam.height * 16
    ctx.check(ctx.lib.vt_render(ctx.handle, world.handle, C.byref(cam), C.byref(params), d_out.ptr, stream))


def render_host(ctx: Context, world: World, cam: Camera_t, params: Params_t, out: np.ndarray | None = None):
    if out is None:
        out = np.zeros(cam.width * cam.height, dtype=HIT_DTYPE)
    assert out.dtype == HIT_DTYPE and out.size >= cam.width * cam.height
    ctx.check(ctx.lib.vt_render_host(ctx.handle, world.handle, C.byref(cam), C.byref(params), _ptr(out)))
    return out


REF_PIXEL_DTYPE = np.dtype([("albedo", "<u4"), ("normal", "<u4"), ("illumination", "<u4"), ("color", "<u4"),
                            ("position", "<f4", (4,))])
REF_HIT_DTYPE = np.dtype([("data", "<u4"), ("hit_pos", "<f4", (3,)), ("normal", "<f4", (3,)), ("pad", "<i4")])
assert REF_PIXEL_DTYPE.itemsize == 32 and REF_HIT_DTYPE.itemsize == 32


def vox_decode(data: bytes) -> np.ndarray:
    """MagicaVoxel bytes -> (models, 8, 8, 8) [z, y, x] RGBA8 texels, as the
    reference's model atlas stores them (file y and z swapped)."""
    buf = np.frombuffer(data, dtype=np.uint8)
    count = C.c_int32()
    _check(load().vt_vox_decode(buf.ctypes.data, buf.size, None, 0, C.byref(count)))
    out = np.zeros((count.value, 8, 8, 8), dtype=np.uint32)
    _check(load().vt_vox_decode(buf.ctypes.data, buf.size, out.ctypes.data, count.value, C.byref(count)))
    return out


class Brickmap:
    """The reference's world (VoxelBrickmap(512, 8) + VoxelModelAtlas) on the
    device, traced with the reference's own traceMap ("mode R")."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        h = C.c_void_p()
        ctx.check(ctx.lib.vt_brickmap_create(ctx.handle, C.byref(h)))
        self.handle = h

    def upload(self, chunks: np.ndarray, bricks: np.ndarray) -> None:
        chunks = np.ascontiguousarray(chunks, np.uint32).reshape(-1)
        bricks = np.ascontiguousarray(bricks, np.uint32).reshape(-1)
        assert chunks.size == 64 ** 3 and bricks.size % 512 == 0
        self.ctx.check(self.ctx.lib.vt_brickmap_upload(self.handle, chunks.ctypes.data, bricks.ctypes.data,
                                                       bricks.size // 512))

    def set_model(self, slot: int, texels: np.ndarray) -> None:
        texels = np.ascontiguousarray(texels, np.uint32).reshape(512)
        self.ctx.check(self.ctx.lib.vt_brickmap_set_model(self.handle, slot, texels.ctypes.data))

    def set_atlas(self, atlas: np.ndarray, slots: int) -> None:
        """Uploads the first `slots` models of a 256^3 atlas ([z, y, x] or flat)."""
        a = np.asarray(atlas, np.uint32).reshape(256, 256, 256)
        for s in range(slots):
            ox, oy, oz = (s & 31) * 8, ((s >> 5) & 31) * 8, ((s >> 10) & 31) * 8
            self.set_model(s, a[oz:oz + 8, oy:oy + 8, ox:ox + 8])

    def load_vox(self, data: bytes) -> int:
        buf = np.frombuffer(data, dtype=np.uint8)
        n = C.c_int32()
        self.ctx.check(self.ctx.lib.vt_brickmap_load_vox(self.handle, buf.ctypes.data, buf.size, C.byref(n)))
        return n.value

    def trace_map(self, origins: np.ndarray, dirs: np.ndarray, max_steps: int) -> np.ndarray:
        ctx = self.ctx
        origins = np.ascontiguousarray(origins, np.float32).reshape(-1, 3)
        dirs = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
        n = origins.shape[0]
        do, dd, dh = ctx.alloc(origins.nbytes), ctx.alloc(dirs.nbytes), ctx.alloc(max(n, 1) * 32)
        try:
            do.upload(origins)
            dd.upload(dirs)
            ctx.check(ctx.lib.vt_trace_map(ctx.handle, self.handle, do.ptr, dd.ptr, n, max_steps, dh.ptr, None))
            ctx.sync()
            return dh.download(np.zeros(n, REF_HIT_DTYPE))
        finally:
            do.free(), dd.free(), dh.free()

    def render(self, cam: Camera_t) -> np.ndarray:
        ctx = self.ctx
        n = cam.width * cam.height
        d = ctx.alloc(n * 32)
        try:
            ctx.check(ctx.lib.vt_render_reference(ctx.handle, self.handle, C.byref(cam), d.ptr, None))
            ctx.sync()
            return d.download(np.zeros(n, REF_PIXEL_DTYPE))
        finally:
            d.free()

    def edit(self, cam: Camera_t, edit_mode: int) -> np.ndarray:
        """The editing pass (pick + map_setVoxel); returns the pick's hit."""
        ctx = self.ctx
        d = ctx.alloc(32)
        try:
            ctx.check(ctx.lib.vt_brickmap_edit(ctx.handle, self.handle, C.byref(cam), int(edit_mode), d.ptr, None))
            ctx.sync()
            return d.download(np.zeros(1, REF_HIT_DTYPE))[0]
        finally:
            d.free()

    def download(self, nbricks: int):
        """(chunk table [64^3], first nbricks bricks [nbricks*512]) as uint32."""
        ch, br = np.zeros(64 ** 3, np.uint32), np.zeros(nbricks * 512, np.uint32)
        self.ctx.check(self.ctx.lib.vt_brickmap_download(self.handle, _ptr(ch), _ptr(br), nbricks))
        return ch, br

    def close(self) -> None:
        if self.handle:
            self.ctx.lib.vt_brickmap_destroy(self.handle)
            self.handle = None


class Batch:
    """Many (world, camera, output) jobs rendered by one persistent launch,
    replayed as a CUDA graph (vt_batch_*)."""

    def __init__(self, ctx: Context, jobs, params: Params_t):
        self.ctx = ctx
        arr = (Job_t * len(jobs))()
        for i, (world, cam, d_out) in enumerate(jobs):
            arr[i].world = world.handle.value if hasattr(world.handle, "value") else world.handle
            arr[i].camera = cam
            arr[i].d_out = d_out.ptr
        h = C.c_void_p()
        ctx.check(ctx.lib.vt_batch_create(ctx.handle, arr, len(jobs), C.byref(params), C.byref(h)))
        self.handle = h

    def launch(self, stream=None) -> None:
        self.ctx.check(self.ctx.lib.vt_batch_launch(self.handle, stream))

    def autotune(self, reps: int = 3) -> tuple[int, float]:
        """Times each launch shape and keeps the fastest: (shape, ms)."""
        shape, ms = C.c_int32(), C.c_float()
        self.ctx.check(self.ctx.lib.vt_batch_autotune(self.handle, reps, C.byref(shape), C.byref(ms)))
        return shape.value, ms.value

    def info(self) -> dict:
        px, nj, nu = C.c_uint64(), C.c_int32(), C.c_uint32()
        self.ctx.check(self.ctx.lib.vt_batch_info(self.handle, C.byref(px), C.byref(nj), C.byref(nu)))
        return {"pixels": px.value, "jobs": nj.value, "units": nu.value}

    def close(self) -> None:
        if self.handle:
            self.ctx.lib.vt_batch_destroy(self.handle)
            self.handle = None


class Shading:
    """Differentiable Lambert shading of one world (vt_shade_forward/backward),
    the C-ABI counterpart of a torch.autograd.Function: forward() renders the
    image from the fixed primary hits, backward() the loss and its gradients.
    Parameters live in device buffers owned here; gradients accumulate until
    zero_grad()."""

    def __init__(self, ctx: Context, world: World, palette: np.ndarray, albedo: np.ndarray | None, sun,
                 ambient: float = 0.2, diffuse: float = 0.8, shadow_max_steps: int = 512):
        self.ctx, self.world = ctx, world
        X, Y, Z = world.dims
        self.d_pal = ctx.alloc(256 * 3 * 4)
        self.d_alb = ctx.alloc(X * Y * Z * 4) if albedo is not None else None
        self.d_gpal = ctx.alloc(256 * 3 * 4)
        self.d_galb = ctx.alloc(X * Y * Z * 4) if albedo is not None else None
        self.d_gsun = ctx.alloc(3 * 4)
        self.d_loss = ctx.alloc(4)
        self.inputs = ShadeInputs_t()
        self.set_params(palette, albedo, sun)
        self.inputs.ambient, self.inputs.diffuse = float(ambient), float(diffuse)
        self.inputs.shadow_max_steps = int(shadow_max_steps)
        self.zero_grad()

    def set_params(self, palette, albedo, sun) -> None:
        self.d_pal.upload(np.asarray(palette, np.float32).reshape(256, 3))
        if albedo is not None:
            self.d_alb.upload(np.asarray(albedo, np.float32).reshape(-1))
        self.inputs.d_palette = self.d_pal.ptr
        self.inputs.d_albedo = self.d_alb.ptr if self.d_alb is not None else None
        self.inputs.sun = (C.c_float * 3)(*[float(s) for s in sun])

    def zero_grad(self) -> None:
        self.zero_grad_async()
        self.ctx.sync()

    def zero_grad_async(self, stream=None) -> None:
        for b in (self.d_gpal, self.d_galb, self.d_gsun, self.d_loss):
            if b is not None:
                b.zero(stream)

    def forward(self, cam: Camera_t, d_hits: DeviceBuffer, d_rgb: DeviceBuffer, vis_in=None, vis_out=None,
                stream=None) -> None:
        self.ctx.check(self.ctx.lib.vt_shade_forward(
            self.ctx.handle, self.world.handle, C.byref(cam), d_hits.ptr, C.byref(self.inputs),
            vis_in.ptr if vis_in is not None else None, vis_out.ptr if vis_out is not None else None, d_rgb.ptr,
            stream))

    def backward(self, cam: Camera_t, d_hits: DeviceBuffer, d_target: DeviceBuffer, stream=None) -> None:
        self.ctx.check(self.ctx.lib.vt_shade_backward(
            self.ctx.handle, self.world.handle, C.byref(cam), d_hits.ptr, C.byref(self.inputs), d_target.ptr,
            self.d_loss.ptr, self.d_gpal.ptr, self.d_galb.ptr if self.d_galb is not None else None,
            self.d_gsun.ptr, stream))

    def forward_views(self, cams, d_hits, d_rgbs, stream=None) -> None:
        """forward over many views in one call (concurrent internally)."""
        n = len(cams)
        cam_arr = (Camera_t * n)(*cams)
        hits = (C.c_void_p * n)(*[h.ptr for h in d_hits])
        rgbs = (C.c_void_p * n)(*[r.ptr for r in d_rgbs])
        self.ctx.check(self.ctx.lib.vt_shade_forward_views(self.ctx.handle, self.world.handle, n, cam_arr, hits,
                                                           C.byref(self.inputs), rgbs, stream))

    def backward_views(self, cams, d_hits, d_targets, stream=None) -> None:
        """backward over many views in one call (concurrent internally)."""
        n = len(cams)
        cam_arr = (Camera_t * n)(*cams)
        hits = (C.c_void_p * n)(*[h.ptr for h in d_hits])
        tgts = (C.c_void_p * n)(*[t.ptr for t in d_targets])
        self.ctx.check(self.ctx.lib.vt_shade_backward_views(
            self.ctx.handle, self.world.handle, n, cam_arr, hits, C.byref(self.inputs), tgts, self.d_loss.ptr,
            self.d_gpal.ptr, self.d_galb.ptr if self.d_galb is not None else None, self.d_gsun.ptr, stream))

    def grads(self) -> dict:
        self.ctx.sync()
        out = {"loss": float(self.d_loss.download(np.zeros(1, np.float32))[0]),
               "palette": self.d_gpal.download(np.zeros((256, 3), np.float32)),
               "sun": self.d_gsun.download(np.zeros(3, np.float32))}
        if self.d_galb is not None:
            out["albedo"] = self.d_galb.download(np.zeros(self.world.dims[0] * self.world.dims[1]
                                                          * self.world.dims[2], np.float32))
        return out

    def close(self) -> None:
        for b in (self.d_pal, self.d_alb, self.d_gpal, self.d_galb, self.d_gsun, self.d_loss):
            if b is not None:
                b.free()


STATIC_MAX_PIXELS = 262144


def render_host_static(ctx: Context, world: World, cam: Camera_t, params: Params_t, out: np.ndarray | None = None):
    """render_host without any device allocation (records staged in the
    library's fixed device array; frames of at most STATIC_MAX_PIXELS)."""
    if out is None:
        out = np.zeros(cam.width * cam.height, dtype=HIT_DTYPE)
    assert out.dtype == HIT_DTYPE and out.size >= cam.width * cam.height
    ctx.check(ctx.lib.vt_render_host_static(ctx.handle, world.handle, C.byref(cam), C.byref(params), _ptr(out)))
    return out


def render_stats(ctx: Context, world: World, cam: Camera_t, params: Params_t, stream=None) -> dict:
    st = Stats_t()
    ctx.check(ctx.lib.vt_render_stats(ctx.handle, world.handle, C.byref(cam), C.byref(params), C.byref(st), stream))
    return st.as_dict()


def trace_rays(ctx: Context, world: World, origins: np.ndarray, dirs: np.ndarray, max_steps: int) -> np.ndarray:
    origins = np.ascontiguousarray(origins, dtype=np.float32).reshape(-1, 3)
    dirs = np.ascontiguousarray(dirs, dtype=np.float32).reshape(-1, 3)
    n = origins.shape[0]
    do, dd, dh = ctx.alloc(origins.nbytes), ctx.alloc(dirs.nbytes), ctx.alloc(max(n, 1) * 16)
    try:
        do.upload(origins)
        dd.upload(dirs)
        ctx.check(ctx.lib.vt_trace_rays(ctx.handle, world.handle, do.ptr, dd.ptr, n, max_steps, dh.ptr, None))
        ctx.sync()
        out = np.zeros(n, dtype=HIT_DTYPE)
        if n:
            dh.download(out)
        return out
    finally:
        do.free(), dd.free(), dh.free()


# --------------------------------------------------------------- generators
def gen_desc(dims, scale: float = 1.0, seed: int = 0, trees: int = 0, caves: bool = False) -> GenDesc_t:
    d = GenDesc_t()
    load().vt_gen_desc_init(C.byref(d), int(dims[0]), int(dims[1]), int(dims[2]), float(scale), int(seed))
    d.trees = int(trees)
    d.caves = 1 if caves else 0
    return d


def gen_world(desc: GenDesc_t, threads: int = 0) -> np.ndarray:
    X, Y, Z = desc.dims
    out = np.zeros((Z, Y, X), dtype=np.uint8)
    _check(load().vt_gen_world(C.byref(desc), _ptr(out), out.nbytes, threads))
    return out


def procgen_reference(dim: int = 512, noise: np.ndarray | None = None, seed: int = 0, offset=(0.0, 0.0)):
    """The reference's procgen (procgen.zig:6-70) in its own world format:
    (chunks [(dim/8)^3] u32, bricks [n*512] u32).  noise: (dim, dim) heightfield
    noise indexed [x, z] (FastNoiseLite's role), or None for the seeded fbm."""
    cd = dim // 8
    chunks = np.zeros(cd ** 3, np.uint32)
    nz = None if noise is None else np.ascontiguousarray(noise, np.float32).reshape(dim * dim)
    cap = cd * cd * 4
    while True:
        bricks = np.zeros(cap * 512, np.uint32)
        n = C.c_size_t()
        st = load().vt_procgen_reference(dim, float(offset[0]), float(offset[1]), _ptr(nz) if nz is not None else None,
                                         int(seed), _ptr(chunks), _ptr(bricks), cap, C.byref(n))
        if st == VT_OK:
            return chunks, bricks[:n.value * 512].copy()
        if st != VT_ERR_OOM:
            _check(st)
        cap = max(cap * 2, n.value)


def gen_camera(desc: GenDesc_t, seed: int, width: int, height: int) -> Camera_t:
    cam = Camera_t()
    _check(load().vt_gen_camera(C.byref(desc), int(seed), int(width), int(height), C.byref(cam)))
    return cam


def gen_sun(seed: int):
    out = (C.c_float * 3)()
    _check(load().vt_gen_sun(int(seed), out))
    return [float(v) for v in out]


def default_palette() -> np.ndarray:
    pal = np.zeros(256, dtype=np.uint32)
    _check(load().vt_default_palette(_ptr(pal)))
    return pal
