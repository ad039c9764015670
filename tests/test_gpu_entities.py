"""Entity occluders in the shadow pass (traceEntities' role,
secondary.comp.glsl:42-46) against the oracle.

Bar: records bit-exact (VT_HIT_ENTITY included), RGBA8 within 1/255; the
adjoint's shadow visibility identical to the FP64 reference's."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def floating_boxes(vt, desc, rng, n):
    """Boxes hovering 3-12 voxels above the terrain, 1-8 voxels wide."""
    X, Y, Z = desc.dims
    out = []
    for _ in range(n):
        x, z = rng.uniform(0, X - 8), rng.uniform(0, Z - 8)
        h = vt.load().vt_gen_height(vt.C.byref(desc), int(x), int(z))
        y = h + rng.uniform(3, 12)
        sx, sy, sz = rng.uniform(1, 8, 3)
        out.append([x, y, z, x + sx, y + sy, z + sz])
    out.append([5.0, -4.0, 5.0, 5.0, 300.0, 5.0])      # a degenerate (zero-width) column
    return np.array(out, np.float32)


@pytest.mark.parametrize("nboxes", [1, 40, 300])
def test_entity_shadows_match_oracle(vt, oracle, ctx, nboxes):
    desc = vt.gen_desc((160, 96, 160), scale=0.6, seed=17, trees=25)
    mats = vt.gen_world(desc)
    rng = np.random.default_rng(nboxes)
    boxes = floating_boxes(vt, desc, rng, nboxes)
    w = vt.World(ctx, (160, 96, 160))
    try:
        w.upload_dense(mats)
        w.set_entities(boxes)
        ow = oracle.OracleWorld(mats, entities=boxes)
        p = vt.default_params(sun_dir=vt.gen_sun(3), rays=vt.RAYS_PRIMARY | vt.RAYS_SHADOW | vt.RAYS_BOUNCE)
        seen = 0
        for cs in range(2):
            cam = vt.gen_camera(desc, cs, 160, 120)
            got = vt.render_host(ctx, w, cam, p)
            ref, _ = oracle.render(ow, vt.default_palette(), cam, p, threads=8)
            for f in ("voxel", "face", "material", "flags"):
                assert np.array_equal(got[f], ref[f]), f
            g = np.ascontiguousarray(got["rgba"]).view(np.uint8).astype(int)
            r = np.ascontiguousarray(ref["rgba"]).view(np.uint8).astype(int)
            assert np.abs(g - r).max() <= 1
            seen += int(((got["flags"] & vt.HIT_ENTITY) != 0).sum())
        if nboxes >= 40:
            assert seen > 0
        # removing the boxes gives the plain frame back
        w.set_entities(None)
        plain = vt.render_host(ctx, w, cam, p)
        assert ((plain["flags"] & vt.HIT_ENTITY) == 0).all()
        ref, _ = oracle.render(oracle.OracleWorld(mats), vt.default_palette(), cam, p, threads=8)
        assert np.array_equal(plain["flags"], ref["flags"])
    finally:
        w.close()


def test_entity_visibility_in_the_adjoint(vt, oracle, ctx):
    desc = vt.gen_desc((128, 96, 128), scale=0.6, seed=23, trees=20)
    mats = vt.gen_world(desc)
    boxes = floating_boxes(vt, desc, np.random.default_rng(23), 120)
    w = vt.World(ctx, (128, 96, 128))
    try:
        w.upload_dense(mats)
        w.set_entities(boxes)
        cam = vt.gen_camera(desc, 4, 96, 64)
        prim = vt.default_params(rays=vt.RAYS_PRIMARY, shade=vt.SHADE_NONE)
        hb = ctx.alloc(cam.width * cam.height * 16)
        vt.render(ctx, w, cam, prim, hb)
        ctx.sync()
        rec = hb.download(np.zeros(cam.width * cam.height, vt.HIT_DTYPE))
        rng = np.random.default_rng(1)
        pal = rng.uniform(0.1, 0.9, (256, 3)).astype(np.float32)
        sun = np.array(vt.gen_sun(5), np.float32)
        sh = vt.Shading(ctx, w, pal, None, sun)
        rgb, vis = ctx.alloc(cam.width * cam.height * 12), ctx.alloc(cam.width * cam.height)
        sh.forward(cam, hb, rgb, vis_out=vis)
        ctx.sync()
        gvis = vis.download(np.zeros(cam.width * cam.height, np.uint8))
        ref = oracle.shade_grad_f64(oracle.OracleWorld(mats, entities=boxes), cam, rec, pal, None, sun, 0.2, 0.8, 512)
        plain = oracle.shade_grad_f64(oracle.OracleWorld(mats), cam, rec, pal, None, sun, 0.2, 0.8, 512)
        assert np.array_equal(gvis, ref["vis"])
        assert (plain["vis"] != ref["vis"]).sum() > 0
        sh.close()
        for b in (hb, rgb, vis):
            b.free()
    finally:
        w.close()
