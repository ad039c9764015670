"""Worlds in the reference's own format, for the mode-R oracle checks.

The reference stores a 512^3 voxel map as a 64^3 table of brick indices
(0 = empty, else brick + 1; index x + 64*(y + 64*z), voxel.zig:21-23) and a
pool of 8^3 u32 voxel bricks (voxel x + 8*y + 64*z, voxel.zig:58-61), each
voxel a packed {ty:28, is_solid:1} (voxel.zig:7-19).  ty selects an 8^3 RGBA8
model in a 256^3 atlas at ((ty & 31)*8, (ty>>5 & 31)*8, (ty>>10 & 31)*8)
(voxel.zig:94-112, map.glsl:57-60).
"""
from __future__ import annotations

import numpy as np


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


def build_atlas(models: list[np.ndarray]) -> np.ndarray:
    atlas = np.zeros((256, 256, 256), dtype=np.uint32)  # [z, y, x]
    for s, m in enumerate(models):
        ox, oy, oz = (s & 31) * 8, ((s >> 5) & 31) * 8, ((s >> 10) & 31) * 8
        atlas[oz:oz + 8, oy:oy + 8, ox:ox + 8] = m
    return atlas.reshape(-1)


def build_map(mats: np.ndarray, model_of_material: np.ndarray):
    """Dense uint8 materials [z, y, x] (at most 512 per axis) -> (chunks, data).
    Material m != 0 becomes the solid voxel of model model_of_material[m]."""
    Z, Y, X = mats.shape
    assert max(X, Y, Z) <= 512
    cz, cy, cx = (Z + 7) // 8, (Y + 7) // 8, (X + 7) // 8
    grid = np.zeros((cz * 8, cy * 8, cx * 8), dtype=np.uint8)
    grid[:Z, :Y, :X] = mats
    words = np.where(grid != 0, (model_of_material[grid].astype(np.uint32) & 0xFFFFFFF) | (1 << 28), 0)
    bricks = words.astype(np.uint32).reshape(cz, 8, cy, 8, cx, 8)   # [bz, z, by, y, bx, x]
    occupied = np.zeros((64, 64, 64), dtype=bool)                   # [bz, by, bx]
    occupied[:cz, :cy, :cx] = (bricks != 0).any(axis=(1, 3, 5))
    chunks = np.zeros((64, 64, 64), dtype=np.uint32)
    idx = np.flatnonzero(occupied.reshape(-1))                      # chunk index x + 64*(y + 64*z)
    chunks.reshape(-1)[idx] = np.arange(1, idx.size + 1, dtype=np.uint32)
    bz, by, bx = np.unravel_index(idx, (64, 64, 64))
    data = bricks[bz, :, by, :, bx, :]                              # [k, z, y, x]
    return chunks.reshape(-1), np.ascontiguousarray(data.reshape(-1)).astype(np.uint32)


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
