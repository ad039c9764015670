"""The FP64 reference gradient of the shading adjoint against central finite
differences (h = 1e-3) of the FP64 loss, with the hit set and the shadow set
held fixed (CPU only)."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def setup(oracle, vtlib):
    d = vtlib.gen_desc((96, 64, 96), scale=0.5, seed=12, trees=12)
    mats = vtlib.gen_world(d)
    rng = np.random.default_rng(12)
    occ = mats > 0
    mats[occ] = rng.integers(1, 24, occ.sum()).astype(np.uint8)   # many materials in view
    ow = oracle.OracleWorld(mats)
    cam = vtlib.gen_camera(d, 2, 48, 32)
    hits, _ = oracle.render(ow, vtlib.default_palette(), cam, vtlib.default_params(rays=1, shade=0), threads=4)
    pal = rng.uniform(0.1, 0.9, (256, 3))
    alb = rng.uniform(0.5, 1.5, mats.size)
    sun = np.array(vtlib.gen_sun(12), np.float64)
    target = rng.uniform(0, 1, (cam.width * cam.height, 3)).astype(np.float32)
    base = oracle.shade_grad_f64(ow, cam, hits, pal, alb, sun, 0.2, 0.8, 512, target)
    return ow, cam, hits, pal, alb, sun, target, base


def loss_at(oracle, s, pal, alb, sun):
    ow, cam, hits, _, _, _, target, base = s
    return oracle.shade_grad_f64(ow, cam, hits, pal, alb, sun, 0.2, 0.8, 512, target, vis_in=base["vis"])["loss"]


def test_palette_gradient_matches_fd(oracle, setup):
    ow, cam, hits, pal, alb, sun, target, base = setup
    h = 1e-3
    used = np.unique(hits["material"][(hits["flags"] & 1) == 1])
    assert used.size >= 3
    for m in used:
        for k in range(3):
            p1, p2 = pal.copy(), pal.copy()
            p1[m, k] += h
            p2[m, k] -= h
            fd = (loss_at(oracle, setup, p1, alb, sun) - loss_at(oracle, setup, p2, alb, sun)) / (2 * h)
            assert fd == pytest.approx(base["palette"][m, k], rel=1e-6, abs=1e-9)


def test_albedo_gradient_matches_fd(oracle, setup):
    ow, cam, hits, pal, alb, sun, target, base = setup
    h = 1e-3
    voxels = np.unique(hits["voxel"][(hits["flags"] & 1) == 1])[:12]
    for v in voxels:
        a1, a2 = alb.copy(), alb.copy()
        a1[v] += h
        a2[v] -= h
        fd = (loss_at(oracle, setup, pal, a1, sun) - loss_at(oracle, setup, pal, a2, sun)) / (2 * h)
        assert fd == pytest.approx(base["albedo"][v], rel=1e-6, abs=1e-9)


def test_sun_gradient_matches_fd(oracle, setup):
    ow, cam, hits, pal, alb, sun, target, base = setup
    h = 1e-3
    for k in range(3):
        s1, s2 = sun.copy(), sun.copy()
        s1[k] += h
        s2[k] -= h
        fd = (loss_at(oracle, setup, pal, alb, s1) - loss_at(oracle, setup, pal, alb, s2)) / (2 * h)
        assert fd == pytest.approx(base["sun"][k], rel=1e-4, abs=1e-6 * np.abs(base["sun"]).max())


def test_shadow_set_is_nontrivial(setup):
    *_, base = setup
    vis = base["vis"]
    assert vis.sum() > 0 and (vis == 0).sum() > 0
