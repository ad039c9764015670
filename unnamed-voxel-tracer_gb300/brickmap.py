"""Worlds in the reference's own format ("mode R" of the library).

The reference stores a 512^3 voxel map as a 64^3 table of brick indices
(0 = empty, else brick + 1; index x + 64*(y + 64*z), voxel.zig:21-23) and a
pool of 8^3 u32 voxel bricks (voxel x + 8*y + 64*z, voxel.zig:58-61), each
voxel a packed {ty:28, is_solid:1} (voxel.zig:7-19).  ty selects an 8^3 RGBA8
model in a 256^3 atlas at ((ty & 31)*8, (ty>>5 & 31)*8, (ty>>10 & 31)*8)
(voxel.zig:94-112, map.glsl:57-60).  These helpers build such a world from a
dense material grid, for vt.Brickmap.upload / set_atlas.
"""
from __future__ import annotations

import numpy as np


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
