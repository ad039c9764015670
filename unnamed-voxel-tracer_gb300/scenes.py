"""The seeded synthetic workloads (all inputs generated here; no dataset).

  config 0  128^3 terrain (height 64 + 24 fbm, 4 octaves, period 64, water
            below 56), 640x360 primary rays, max 512 steps
  config 1  512x256x512 terrain + 200 trees, 1920x1080 primary + shadow rays
  config 2  2048x256x2048 terrain + trees + 3-D value-noise caves, 3840x2160
            primary + shadow + one cosine-weighted bounce ray per hit
  config 3  64 cube scenes, edge log-uniform in [32, 512], config-0 terrain
            scaled to the edge, 1-8 cameras each at 320x240 / 640x480 /
            1280x720 / 1920x1080, primary + shadow rays
  config 4  256^3 world from the config-1 generator (50 trees), FP32 palette
            and per-voxel albedo scale in [0.5, 1.5], 16 views at 512x512,
            targets rendered from a hidden palette and sun
"""
from __future__ import annotations

import math

import numpy as np

import vt


def config0(seed: int = 0):
    desc = vt.gen_desc((128, 128, 128), seed=seed)
    cams = [vt.gen_camera(desc, seed, 640, 360)]
    params = vt.default_params(rays=vt.RAYS_PRIMARY, max_steps=512)
    return desc, cams, params


def config1(seed: int = 1, cameras: int = 8, first_camera: int = 0, size=(1920, 1080)):
    desc = vt.gen_desc((512, 256, 512), seed=seed, trees=200)
    cams = [vt.gen_camera(desc, first_camera + s, size[0], size[1]) for s in range(cameras)]
    params = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW, max_steps=512, shadow_max_steps=512,
                               sun_dir=vt.gen_sun(seed))
    return desc, cams, params


def config2(seed: int = 2, cameras: int = 2, size=(3840, 2160)):
    desc = vt.gen_desc((2048, 256, 2048), seed=seed, trees=3200, caves=True)
    cams = [vt.gen_camera(desc, s, size[0], size[1]) for s in range(cameras)]
    params = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW | vt.RAYS_BOUNCE, max_steps=512,
                               shadow_max_steps=512, bounce_max_steps=256, seed=seed, sun_dir=vt.gen_sun(seed))
    return desc, cams, params


RESOLUTIONS = ((320, 240), (640, 480), (1280, 720), (1920, 1080))


def config3(seed: int = 3, scenes: int = 64):
    """[(desc, [cameras])] and the shared params."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(scenes):
        edge = int(round(math.exp(rng.uniform(math.log(32), math.log(512)))))
        desc = vt.gen_desc((edge, edge, edge), scale=edge / 128.0, seed=seed * 1000 + s)
        ncam = int(rng.integers(1, 9))
        cams = []
        for c in range(ncam):
            w, h = RESOLUTIONS[int(rng.integers(0, len(RESOLUTIONS)))]
            cams.append(vt.gen_camera(desc, c, w, h))
        out.append((desc, cams))
    params = vt.default_params(rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW, max_steps=512, shadow_max_steps=512,
                               sun_dir=vt.gen_sun(seed))
    return out, params


def config4(seed: int = 4, views: int = 16, size=(512, 512)):
    """World desc, cameras, (palette, albedo, sun) to optimise from, and the
    hidden (palette, sun) the targets are rendered with."""
    desc = vt.gen_desc((256, 256, 256), seed=seed, trees=50)
    cams = [vt.gen_camera(desc, v, size[0], size[1]) for v in range(views)]
    rng = np.random.default_rng(seed)
    palette = rng.uniform(0.05, 0.95, size=(256, 3)).astype(np.float32)
    albedo = rng.uniform(0.5, 1.5, size=256 * 256 * 256).astype(np.float32)
    hidden_palette = rng.uniform(0.05, 0.95, size=(256, 3)).astype(np.float32)
    sun = np.array(vt.gen_sun(seed + 100), np.float32)
    hidden_sun = np.array(vt.gen_sun(seed + 200), np.float32)
    return desc, cams, (palette, albedo, sun), (hidden_palette, hidden_sun)
