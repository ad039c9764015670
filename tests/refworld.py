"""Worlds in the reference's own format, for the mode-R oracle checks (the
builders live in the package, unnamed-voxel-tracer_gb300/brickmap.py; the
random models, the .vox writer/reader and the ray sampler are test and
benchmark helpers).

The reference stores a 512^3 voxel map as a 64^3 table of brick indices
(0 = empty, else brick + 1; index x + 64*(y + 64*z), voxel.zig:21-23) and a
pool of 8^3 u32 voxel bricks (voxel x + 8*y + 64*z, voxel.zig:58-61), each
voxel a packed {ty:28, is_solid:1} (voxel.zig:7-19).  ty selects an 8^3 RGBA8
model in a 256^3 atlas at ((ty & 31)*8, (ty>>5 & 31)*8, (ty>>10 & 31)*8)
(voxel.zig:94-112, map.glsl:57-60).
"""
from __future__ import annotations

import numpy as np


from brickmap import build_atlas, build_map  # noqa: E402,F401  (the package's builders)


def random_models(rng: np.random.Generator, n: int, full: bool = False) -> list[np.ndarray]:
    """n models, each an (8, 8, 8) [z, y, x] array of RGBA8 texels (0 = empty)."""
    out = []
    for i in range(n):
        density = 1.0 if full else rng.uniform(0.2, 1.0)
        keep = rng.random((8, 8, 8)) < density
        rgb = rng.integers(1, 256, size=(8, 8, 8, 3), dtype=np.uint32)
        tex = rgb[..., 0] | (rgb[..., 1] << 8) | (rgb[..., 2] << 16) | (np.uint32(255) << 24)
        out.append(np.where(keep, tex, 0).astype(np.uint32))
    return out


def tracemap_f64(occupied, o, d, max_steps: int, snap: float):
    """The reference's traceMap stepping (map.glsl:83-168) restated in float64
    for worlds whose occupied voxels hold full 8^3 models, so that a voxel's
    first sub-voxel already hits.  occupied(x, y, z) -> bool; o, d: the ray as
    traceMap receives it (world units).  snap is the factor of map.glsl:162
    (0.999 in the reference; a value just below 1 makes the snap vanish).
    Returns ((x, y, z), face) of the hit voxel, face = 2 axis + (d_axis > 0 ?
    0 : 1) from the last step's axis (map.glsl:117-125), or None on a miss."""
    d = [x if x != 0 else 0.001 for x in d]                       # :85-90
    bound = 8 * 512
    sgn = [1 if x > 0 else -1 for x in d]
    pos = [(1 + s) >> 1 for s in sgn]
    inv = [1.0 / x for x in d]
    axis = 0
    g = [int(o[k] * 8.0) for k in range(3)]                        # :100 (truncation)
    w = [o[k] * 8.0 - g[k] for k in range(3)]
    step = 0
    for _ in range(max_steps):
        if any(v >= bound or v < 0 for v in g):
            break
        vox = tuple((g[k] + int(w[k])) >> 3 for k in range(3))    # :108, :114
        if occupied(*vox):
            return vox, 2 * axis + (0 if pos[axis] else 1)
        if step != 3:                                               # :138-144
            for k in range(3):
                w[k] += g[k] & 7
                g[k] -= g[k] & 7
            step = 3
        t = [((pos[k] << step) - w[k]) * inv[k] for k in range(3)]  # :157
        axis = (0 if t[0] < t[2] else 2) if t[0] < t[1] else (1 if t[1] < t[2] else 2)
        g[axis] += sgn[axis] << step                                # :160
        tm = t[axis]
        for k in range(3):
            w[k] += d[k] * tm                                       # :161
        w[axis] = ((1 - pos[axis]) << step) * snap                  # :162
    return None


def random_rays(rng: np.random.Generator, lo, hi, n: int):
    o = rng.uniform(lo, hi, size=(n, 3))
    d = rng.normal(size=(n, 3))
    d[rng.random(n) < 0.1, 0] = 0.0
    d[rng.random(n) < 0.1, 1] = 0.0
    k = rng.random(n) < 0.05
    d[k] = np.sign(d[k]) + (d[k] == 0)
    return o.astype(np.float32), d.astype(np.float32)


# ---- MagicaVoxel files (test-only writer and reader, from the published format)
def write_vox(models: list[list[tuple[int, int, int, int]]], palette: np.ndarray) -> bytes:
    """models: per model a list of (x, y, z, colour index 1..255) in file axes;
    palette: 256 RGBA8 (entry i is colour index i + 1)."""
    import struct

    def chunk(tag: bytes, content: bytes, children: bytes = b"") -> bytes:
        return tag + struct.pack("<ii", len(content), len(children)) + content + children

    kids = b""
    for vox in models:
        kids += chunk(b"SIZE", struct.pack("<iii", 8, 8, 8))
        kids += chunk(b"XYZI", struct.pack("<i", len(vox)) + b"".join(bytes(v) for v in vox))
    kids += chunk(b"RGBA", np.asarray(palette, np.uint32).astype("<u4").tobytes())
    return b"VOX " + struct.pack("<i", 150) + chunk(b"MAIN", b"", kids)


def read_vox(data: bytes) -> np.ndarray:
    """(models, 8, 8, 8) [z, y, x] texels with the reference's axis swap:
    file (x, y, z) lands at texture (x, z, y); colour index c -> palette[c-1]."""
    import struct
    assert data[:4] == b"VOX "
    p = 8
    assert data[p:p + 4] == b"MAIN"
    n, m = struct.unpack_from("<ii", data, p + 4)
    p += 12 + n
    end = p + m
    raws, pal = [], None
    while p + 12 <= end:
        tag = data[p:p + 4]
        n, m = struct.unpack_from("<ii", data, p + 4)
        body = data[p + 12:p + 12 + n]
        if tag == b"XYZI":
            cnt = struct.unpack_from("<i", body, 0)[0]
            raws.append(np.frombuffer(body, dtype=np.uint8, count=4 * cnt, offset=4).reshape(-1, 4))
        elif tag == b"RGBA":
            pal = np.frombuffer(body, dtype="<u4", count=256)
        p += 12 + n + m
    out = np.zeros((len(raws), 8, 8, 8), np.uint32)
    for k, r in enumerate(raws):
        for x, y, z, c in r:
            if c and x < 8 and y < 8 and z < 8:
                out[k, y, z, x] = pal[c - 1]     # texture (x, file z, file y), stored [z_tex, y_tex, x]
    return out
