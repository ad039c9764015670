"""Shading adjoint on the GPU (vt_shade_forward / vt_shade_backward) against
the FP64 CPU gradient over the same hit and shadow sets, and against central
finite differences of the GPU forward image (h = 1e-3, shadow set held fixed).

Tolerance, element by element (grad_close): |g - g64| <= REL |g64| + FLOOR a,
where a is the element's sum of |per-pixel contributions| (from the FP64
oracle).  REL = 1e-4 is the bar itself; FLOOR = 1e-5 (about 170 float32 ulps
of a) only matters where contributions cancel, since a float32 sum of many
terms is accurate relative to the sum of their magnitudes, not to their
(possibly near-zero) total.  Forward colours within 1e-6."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-4
FLOOR = 1e-5


def grad_close(got, ref, abs_sum, what):
    """Every element of a gradient group within REL of the FP64 value, with
    the absolute floor FLOOR * (its sum of |contributions|)."""
    got, ref, a = (np.asarray(x, np.float64).reshape(-1) for x in (got, ref, abs_sum))
    err = np.abs(got - ref)
    tol = REL * np.abs(ref) + FLOOR * a
    bad = np.flatnonzero(err > tol)
    assert bad.size == 0, (f"{what}: {bad.size} of {ref.size} elements off, worst {bad[np.argmax(err[bad] / tol[bad])]}"
                           f": got {got[bad[0]]!r} want {ref[bad[0]]!r} (sum |terms| {a[bad[0]]!r})")
    # the number of elements held to the relative bar alone (err <= REL |g64|)
    return int((err <= REL * np.abs(ref)).sum())


@pytest.fixture(scope="module")
def scene(vt, ctx, oracle):
    d = vt.gen_desc((256, 256, 256), seed=4, trees=50)
    mats = vt.gen_world(d)
    rng = np.random.default_rng(4)
    occ = mats > 0
    mats[occ] = rng.integers(1, 40, occ.sum()).astype(np.uint8)
    w = vt.World(ctx, (256, 256, 256))
    w.upload_dense(mats)
    cams = [vt.gen_camera(d, v, 128, 96) for v in range(2)]
    prim = vt.default_params(rays=vt.RAYS_PRIMARY, shade=vt.SHADE_NONE)
    hits = []
    for cam in cams:
        hb = ctx.alloc(cam.width * cam.height * 16)
        vt.render(ctx, w, cam, prim, hb)
        hits.append(hb)
    ctx.sync()
    pal = rng.uniform(0.05, 0.95, (256, 3)).astype(np.float32)
    alb = rng.uniform(0.5, 1.5, mats.size).astype(np.float32)
    sun = np.array(vt.gen_sun(9), np.float32)
    targets = [rng.uniform(0, 1, (c.width * c.height, 3)).astype(np.float32) for c in cams]
    sh = vt.Shading(ctx, w, pal, alb, sun)
    yield dict(mats=mats, world=w, cams=cams, hits=hits, pal=pal, alb=alb, sun=sun, targets=targets, sh=sh,
               ow=oracle.OracleWorld(mats))
    sh.close()
    for hb in hits:
        hb.free()
    w.close()


def records(vt, hb, cam):
    out = np.zeros(cam.width * cam.height, vt.HIT_DTYPE)
    return hb.download(out)


def test_forward_matches_fp64(vt, ctx, oracle, scene):
    s = scene
    for cam, hb in zip(s["cams"], s["hits"]):
        rgb = ctx.alloc(cam.width * cam.height * 12)
        vis = ctx.alloc(cam.width * cam.height)
        s["sh"].forward(cam, hb, rgb, vis_out=vis)
        ctx.sync()
        got = rgb.download(np.zeros((cam.width * cam.height, 3), np.float32))
        gvis = vis.download(np.zeros(cam.width * cam.height, np.uint8))
        ref = oracle.shade_grad_f64(s["ow"], cam, records(vt, hb, cam), s["pal"], s["alb"], s["sun"], 0.2, 0.8, 512)
        assert np.array_equal(gvis, ref["vis"])
        assert np.abs(got - ref["rgb"]).max() <= 1e-6
        assert gvis.sum() > 100 and (gvis == 0).sum() > 100
        rgb.free()
        vis.free()


def test_backward_matches_fp64_gradient(vt, ctx, oracle, scene):
    s = scene
    sh = s["sh"]
    sh.zero_grad()
    ref_loss, ref_pal, ref_alb, ref_sun = 0.0, np.zeros((256, 3)), np.zeros(s["mats"].size), np.zeros(3)
    abs_pal, abs_alb, abs_sun = np.zeros((256, 3)), np.zeros(s["mats"].size), np.zeros(3)
    for cam, hb, tgt in zip(s["cams"], s["hits"], s["targets"]):
        dt = ctx.alloc(tgt.nbytes)
        dt.upload(tgt)
        sh.backward(cam, hb, dt)
        ctx.sync()
        dt.free()
        r = oracle.shade_grad_f64(s["ow"], cam, records(vt, hb, cam), s["pal"], s["alb"], s["sun"], 0.2, 0.8, 512,
                                  tgt)
        ref_loss += r["loss"]
        ref_pal += r["palette"]
        ref_alb += r["albedo"]
        ref_sun += r["sun"]
        abs_pal += r["abs_palette"]
        abs_alb += r["abs_albedo"]
        abs_sun += r["abs_sun"]
    g = sh.grads()
    assert g["loss"] == pytest.approx(ref_loss, rel=REL)
    grad_close(g["palette"], ref_pal, abs_pal, "palette")
    assert grad_close(g["albedo"], ref_alb, abs_alb, "albedo") > 1000
    grad_close(g["sun"], ref_sun, abs_sun, "sun")
    assert (np.abs(ref_pal).sum(1) > 0).sum() >= 20 and np.count_nonzero(ref_alb) > 1000


def test_backward_matches_finite_differences(vt, ctx, scene):
    """(L(p + h) - L(p - h)) / 2h from GPU forward images, shadow set fixed."""
    s = scene
    cam, hb, tgt = s["cams"][0], s["hits"][0], s["targets"][0]
    n = cam.width * cam.height
    rgb, vis = ctx.alloc(n * 12), ctx.alloc(n)
    sh = s["sh"]
    sh.forward(cam, hb, rgb, vis_out=vis)

    def loss(pal, alb, sun):
        sh.set_params(pal, alb, sun)
        sh.forward(cam, hb, rgb, vis_in=vis)
        ctx.sync()
        c = rgb.download(np.zeros((n, 3), np.float32)).astype(np.float64)
        return float(((c - tgt.astype(np.float64)) ** 2).sum())

    sh.set_params(s["pal"], s["alb"], s["sun"])
    sh.zero_grad()
    dt = ctx.alloc(tgt.nbytes)
    dt.upload(tgt)
    sh.backward(cam, hb, dt)
    g = sh.grads()
    h = 1e-3
    hits = records(vt, hb, cam)
    mats_seen = np.unique(hits["material"][(hits["flags"] & 1) == 1])[:4]
    for m in mats_seen:
        for k in range(3):
            p1, p2 = s["pal"].copy(), s["pal"].copy()
            p1[m, k] += h
            p2[m, k] -= h
            fd = (loss(p1, s["alb"], s["sun"]) - loss(p2, s["alb"], s["sun"])) / (2 * h)
            assert fd == pytest.approx(g["palette"][m, k], rel=2e-3, abs=2e-3 * np.abs(g["palette"]).max())
    for k in range(3):
        s1, s2 = s["sun"].copy(), s["sun"].copy()
        s1[k] += h
        s2[k] -= h
        fd = (loss(s["pal"], s["alb"], s1) - loss(s["pal"], s["alb"], s2)) / (2 * h)
        assert fd == pytest.approx(g["sun"][k], rel=2e-3, abs=2e-3 * np.abs(g["sun"]).max())
    sh.set_params(s["pal"], s["alb"], s["sun"])
    for b in (rgb, vis, dt):
        b.free()


def test_backward_views_equals_per_view_calls(vt, ctx, scene):
    """The multi-view call (views on concurrent streams) accumulates the same
    loss and gradients as one call per view, up to the order of the float
    atomics."""
    s = scene
    sh = s["sh"]
    tgts = []
    for tgt in s["targets"]:
        dt = ctx.alloc(tgt.nbytes)
        dt.upload(tgt)
        tgts.append(dt)
    sh.zero_grad()
    for cam, hb, dt in zip(s["cams"], s["hits"], tgts):
        sh.backward(cam, hb, dt)
    one = sh.grads()
    sh.zero_grad()
    sh.backward_views(s["cams"], s["hits"], tgts)
    many = sh.grads()
    for k in ("palette", "sun"):
        scale = np.abs(one[k]).max()
        assert np.abs(many[k] - one[k]).max() <= 1e-5 * scale, k
    assert abs(many["loss"] - one["loss"]) <= 1e-5 * abs(one["loss"])
    for dt in tgts:
        dt.free()


def test_forward_views_equals_per_view_calls(vt, ctx, scene):
    s = scene
    n = s["cams"][0].width * s["cams"][0].height
    one = [ctx.alloc(n * 12) for _ in s["cams"]]
    many = [ctx.alloc(n * 12) for _ in s["cams"]]
    for cam, hb, rb in zip(s["cams"], s["hits"], one):
        s["sh"].forward(cam, hb, rb)
    s["sh"].forward_views(s["cams"], s["hits"], many)
    ctx.sync()
    for a, b in zip(one, many):
        assert np.array_equal(a.download(np.zeros(n * 3, np.float32)), b.download(np.zeros(n * 3, np.float32)))
    for b in one + many:
        b.free()


def test_views_of_mixed_sizes_beyond_one_launch(vt, ctx, scene):
    """18 views of five sizes (two launches of the multi-view kernel, views
    smaller than its grid): forward images equal the per-view calls, loss and
    gradients agree up to the order of the float atomics."""
    s = scene
    d = vt.gen_desc((256, 256, 256), seed=4, trees=50)
    sizes = [(128, 96), (64, 40), (17, 9), (1, 1), (100, 3)]
    cams = [vt.gen_camera(d, v % 3, *sizes[v % len(sizes)]) for v in range(18)]
    prim = vt.default_params(rays=vt.RAYS_PRIMARY, shade=vt.SHADE_NONE)
    rng = np.random.default_rng(7)
    hits, tgts, one, many = [], [], [], []
    for cam in cams:
        n = cam.width * cam.height
        hb = ctx.alloc(n * 16)
        vt.render(ctx, s["world"], cam, prim, hb)
        hits.append(hb)
        dt = ctx.alloc(n * 12)
        dt.upload(rng.uniform(0, 1, (n, 3)).astype(np.float32))
        tgts.append(dt)
        one.append(ctx.alloc(n * 12))
        many.append(ctx.alloc(n * 12))
    ctx.sync()
    sh = s["sh"]
    for cam, hb, rb in zip(cams, hits, one):
        sh.forward(cam, hb, rb)
    sh.forward_views(cams, hits, many)
    ctx.sync()
    for cam, a, b in zip(cams, one, many):
        n = cam.width * cam.height
        assert np.array_equal(a.download(np.zeros(n * 3, np.float32)), b.download(np.zeros(n * 3, np.float32)))
    sh.zero_grad()
    for cam, hb, dt in zip(cams, hits, tgts):
        sh.backward(cam, hb, dt)
    g1 = sh.grads()
    sh.zero_grad()
    sh.backward_views(cams, hits, tgts)
    g2 = sh.grads()
    for k in ("palette", "sun"):
        scale = np.abs(g1[k]).max()
        assert scale > 0 and np.abs(g2[k] - g1[k]).max() <= 1e-5 * scale, k
    assert abs(g2["loss"] - g1["loss"]) <= 1e-5 * abs(g1["loss"])
    if "albedo" in g1:
        scale = np.abs(g1["albedo"]).max()
        assert np.abs(g2["albedo"] - g1["albedo"]).max() <= 1e-5 * scale
    for b in hits + tgts + one + many:
        b.free()
