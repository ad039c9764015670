"""Worlds in the reference's own format, for the mode-R oracle checks (the
builders live in the package, unnamed-voxel-tracer_gb300/brickmap.py; the
.vox writer/reader and the ray sampler are test helpers).

The reference stores a 512^3 voxel map as a 64^3 table of brick indices
(0 = empty, else brick + 1; index x + 64*(y + 64*z), voxel.zig:21-23) and a
pool of 8^3 u32 voxel bricks (voxel x + 8*y + 64*z, voxel.zig:58-61), each
voxel a packed {ty:28, is_solid:1} (voxel.zig:7-19).  ty selects an 8^3 RGBA8
model in a 256^3 atlas at ((ty & 31)*8, (ty>>5 & 31)*8, (ty>>10 & 31)*8)
(voxel.zig:94-112, map.glsl:57-60).
"""
from __future__ import annotations

import numpy as np


from brickmap import build_atlas, build_map, random_models  # noqa: E402,F401  (the package's builders)


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
