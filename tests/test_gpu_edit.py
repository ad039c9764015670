"""Pick and edit on the device against the oracle, and the incremental
empty-space distance updates against a full rebuild.

Bar: pick hit records bit-exact; the world after every edit byte-identical
to the oracle's simulation; distances after any sequence of edits equal to
those of a fresh upload of the same bytes (brick and chunk level); the
mode-R editing pass bit-exact against the oracle's restatement (pinned to
the reference by test_oracle_edit)."""
import hashlib
import sys
from pathlib import Path

import numpy as np
import pytest

sys.path.insert(0, str(Path(__file__).resolve().parent / "golden"))
import make_golden as G  # noqa: E402

pytestmark = pytest.mark.gpu


def fresh_distances(vt, ctx, mats):
    Z, Y, X = mats.shape
    w = vt.World(ctx, (X, Y, Z))
    try:
        w.upload_dense(mats)
        return w.distances()
    finally:
        w.close()


def assert_same_distances(vt, ctx, world, mats):
    b, c = world.distances()
    fb, fc = fresh_distances(vt, ctx, mats)
    assert np.array_equal(c, fc)
    bad = np.flatnonzero(b != fb)
    assert bad.size == 0, (bad[:8], b[bad[:8]], fb[bad[:8]])


@pytest.fixture(scope="module")
def host_fields():
    """Distance fields computed on the host by an independent method (a
    summed-area table per octant, tests/host/trace_host.cpp)."""
    import ctypes as C
    import subprocess
    import test_host_trace as T
    if not T.OUT.exists() or any(d.stat().st_mtime > T.OUT.stat().st_mtime for d in T.DEPS):
        T.OUT.parent.mkdir(exist_ok=True)
        subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-I", T.cuda_include(),
                        str(T.SRC), "-o", str(T.OUT)], check=True)
    lib = C.CDLL(str(T.OUT))
    lib.ht_distances.argtypes = [C.POINTER(C.c_int32), C.c_void_p, C.c_void_p, C.c_void_p]

    def fields(mats):
        Z, Y, X = mats.shape
        nch = ((X + 31) // 32) * ((Y + 31) // 32) * ((Z + 31) // 32)
        b, c = np.zeros((8, nch * 512), np.uint8), np.zeros((8, nch), np.uint8)
        m = np.ascontiguousarray(mats)
        lib.ht_distances((C.c_int32 * 3)(X, Y, Z), m.ctypes.data, b.ctypes.data, c.ctypes.data)
        return b, c
    return fields


@pytest.mark.parametrize("dims,seed", [((70, 45, 90), 1), ((160, 96, 128), 2), ((33, 200, 40), 3)])
def test_distances_equal_independent_computation(vt, ctx, host_fields, dims, seed):
    desc = vt.gen_desc(dims, scale=0.5, seed=seed, trees=30, caves=True)
    mats = vt.gen_world(desc)
    rng = np.random.default_rng(seed)
    mats[rng.random(mats.shape) < 0.0005] = 9          # scattered floating voxels
    w = vt.World(ctx, dims)
    try:
        w.upload_dense(mats)
        b, c = w.distances()
        hb, hc = host_fields(mats)
        assert np.array_equal(c, hc)
        for o in range(8):
            bad = np.flatnonzero(b[o] != hb[o])
            assert bad.size == 0, (o, bad[:8], b[o][bad[:8]], hb[o][bad[:8]])
        assert (b > 1).mean() > 0.3 and (b == 0).any()
    finally:
        w.close()


def _shaped_world(dims, seed):
    """A slab, an overhang, pillars and floating voxels: flat and tall empty
    boxes, open space beyond the distance cap, ragged edges."""
    X, Y, Z = dims
    rng = np.random.default_rng(seed)
    mats = np.zeros((Z, Y, X), np.uint8)
    mats[:, : max(1, Y // 6), :] = 2                                  # ground slab
    mats[Z // 4: Z // 2, Y // 2: Y // 2 + 2, X // 5: 4 * X // 5] = 3   # overhang
    for _ in range(12):                                                # pillars
        x, z = rng.integers(0, X), rng.integers(0, Z)
        mats[z, : rng.integers(1, Y), x] = 4
    mats[rng.random(mats.shape) < 0.0003] = 9                          # floating voxels
    return mats


@pytest.mark.parametrize("dims,seed", [((97, 41, 133), 21), ((300, 150, 40), 22), ((64, 7, 64), 23)])
def test_distances_shaped_worlds(vt, ctx, host_fields, dims, seed):
    """Brick and chunk fields against the independent host computation on
    worlds whose empty boxes favour every box shape, with long reaches to the
    cap and a world thinner than a brick's four layers would suggest."""
    mats = _shaped_world(dims, seed)
    w = vt.World(ctx, dims)
    try:
        w.upload_dense(mats)
        b, c = w.distances()
        hb, hc = host_fields(mats)
        assert np.array_equal(c, hc)
        for o in range(8):
            bad = np.flatnonzero(b[o] != hb[o])
            assert bad.size == 0, (o, bad[:8], b[o][bad[:8]], hb[o][bad[:8]])
        down = b[[0, 1, 4, 5]]
        assert ((down >> 6) > 0).any() and ((down >> 6) == 0).any() and ((b & 63) == 63).any()
    finally:
        w.close()


def test_pick_matches_oracle(vt, oracle, ctx):
    desc = vt.gen_desc((160, 96, 128), scale=0.6, seed=4, trees=40, caves=True)
    mats = vt.gen_world(desc)
    ow = oracle.OracleWorld(mats)
    w = vt.World(ctx, (160, 96, 128))
    try:
        w.upload_dense(mats)
        hits = 0
        for s in range(24):
            cam = vt.gen_camera(desc, s, 64, 48)
            for steps in (40, 1000):
                h = w.pick(cam, steps)
                tr, _ = oracle.pick_p(ow, cam, steps)
                if tr.hit:
                    hits += 1
                    assert h["voxel"] == tr.voxel and h["face"] == tr.face and h["material"] == tr.material
                    assert np.float32(tr.t).view(np.uint32) == h["t"].view(np.uint32)
                else:
                    assert h["face"] == 0xFF and h["voxel"] == 0xFFFFFFFF
        assert hits > 10
    finally:
        w.close()


def test_edit_sequence_matches_oracle_and_distances_stay_exact(vt, oracle, ctx):
    desc = vt.gen_desc((128, 96, 160), scale=0.6, seed=12, trees=30)
    mats = vt.gen_world(desc)
    rng = np.random.default_rng(12)
    w = vt.World(ctx, (128, 96, 160))
    hit_buf = ctx.alloc(16)
    try:
        w.upload_dense(mats)
        w.pick(vt.gen_camera(desc, 0, 8, 8), 10)         # builds the distances once
        changed = 0
        for i in range(60):
            cam = vt.gen_camera(desc, 1000 + i % 20, 8, 8)   # cameras repeat: digging into the same spot
            mode = int(rng.choice([0, 0, 0, 1, 6, 200]))
            tr, tgt = oracle.pick_p(oracle.OracleWorld(mats), cam, 600, edit_mode=mode)
            w.edit(cam, 600, mode, d_out=hit_buf)
            got = hit_buf.download(np.zeros(1, vt.HIT_DTYPE))[0]
            assert got["voxel"] == (tr.voxel if tr.hit else 0xFFFFFFFF)
            if tgt[3]:
                x, y, z = tgt[:3]
                changed += mats[z, y, x] != mode
                mats[z, y, x] = mode
            if i % 15 == 14:
                assert np.array_equal(w.download_dense(), mats)
                assert_same_distances(vt, ctx, w, mats)
        assert changed > 20
    finally:
        hit_buf.free()
        w.close()


def test_host_edits_update_distances_incrementally(vt, ctx):
    rng = np.random.default_rng(9)
    X, Y, Z = 200, 72, 136
    mats = np.zeros((Z, Y, X), np.uint8)
    mats[:20] = 3                                     # a floor
    w = vt.World(ctx, (X, Y, Z))
    try:
        w.upload_dense(mats)
        w.distances()
        for rnd in range(4):
            # scattered single voxels, a cleared chunk, a filled chunk
            for _ in range(40):
                x, y, z = rng.integers(0, X), rng.integers(0, Y), rng.integers(0, Z)
                m = int(rng.choice([0, 7]))
                w.set(int(x), int(y), int(z), m)
                mats[z, y, x] = m
            cx, cy, cz = rng.integers(0, X // 32), rng.integers(0, Y // 32), rng.integers(0, Z // 32)
            chunk = (rng.random((32, 32, 32)) < (0.0 if rnd % 2 else 0.3)).astype(np.uint8) * 5
            w.upload_chunk(int(cx), int(cy), int(cz), chunk)
            sl = (slice(cz * 32, cz * 32 + 32), slice(cy * 32, cy * 32 + 32), slice(cx * 32, cx * 32 + 32))
            mats[sl] = chunk[:mats[sl].shape[0], :mats[sl].shape[1], :mats[sl].shape[2]]
            assert_same_distances(vt, ctx, w, mats)
        # clearing the whole floor voxel by voxel in one column range empties chunks
        for x in range(0, 32):
            for z in range(0, 8):
                for y in range(0, 20):
                    w.set(x, y, z, 0)
        mats[0:8, 0:20, 0:32] = 0
        assert_same_distances(vt, ctx, w, mats)
    finally:
        w.close()


def test_corner_and_edge_edits_update_distances(vt, ctx):
    """Single-voxel edits at the world's corners and edges, on chunk and brick
    boundaries, in a world whose sides are not multiples of a brick: the
    update boxes are clipped on every side and the result still equals a
    fresh rebuild."""
    X, Y, Z = 61, 45, 77
    mats = _shaped_world((X, Y, Z), 31)
    w = vt.World(ctx, (X, Y, Z))
    try:
        w.upload_dense(mats)
        w.distances()
        cells = [(x, y, z) for x in (0, X - 1) for y in (0, Y - 1) for z in (0, Z - 1)]
        cells += [(31, 0, 0), (32, Y - 1, Z - 1), (0, 31, 40), (X - 1, 32, 3), (17, 44, 63), (60, 4, 64)]
        for i, (x, y, z) in enumerate(cells):
            m = 0 if mats[z, y, x] else 6
            w.set(x, y, z, m)
            mats[z, y, x] = m
            if i % 3 == 2:
                assert_same_distances(vt, ctx, w, mats)
        assert_same_distances(vt, ctx, w, mats)
    finally:
        w.close()


def test_edited_world_renders_like_fresh_upload(vt, oracle, ctx):
    desc = vt.gen_desc((96, 80, 112), scale=0.5, seed=31, trees=20)
    mats = vt.gen_world(desc)
    w = vt.World(ctx, (96, 80, 112))
    try:
        w.upload_dense(mats)
        cam = vt.gen_camera(desc, 2, 128, 96)
        p = vt.default_params()
        vt.render_host(ctx, w, cam, p)
        for i in range(30):
            w.edit(vt.gen_camera(desc, 500 + i % 6, 8, 8), 500, 0 if i % 3 else 9)
        got = vt.render_host(ctx, w, cam, p)
        now = w.download_dense()
        ref, _ = oracle.render(oracle.OracleWorld(now), vt.default_palette(), cam, p, threads=8)
        for f in ("voxel", "face", "material", "flags"):
            assert np.array_equal(got[f], ref[f]), f
        assert not np.array_equal(now, mats)
    finally:
        w.close()


def test_brickmap_edit_matches_oracle(vt, oracle, ctx):
    _, _, chunks, data, atlas = G.golden_world()
    bm = vt.Brickmap(ctx)
    rw = oracle.OracleRefWorld(chunks, data.copy(), atlas)
    try:
        bm.upload(chunks, data)
        bm.set_atlas(atlas, 8)
        g = np.load(Path(__file__).resolve().parent / "golden" / "ref_edit.npz")
        for i, (cam, mode) in enumerate(G.edit_sequence()):
            h = bm.edit(cam, mode)
            o = oracle.edit_r(rw, cam, mode)
            assert h["data"] == o.data == g["data"][i], i
            assert np.array_equal(h["hit_pos"].view(np.uint32), np.array(o.hit_pos, np.float32).view(np.uint32))
            assert np.array_equal(h["normal"], np.array(o.normal, np.float32))
        _, pool = bm.download(data.size // 512)
        assert np.array_equal(pool, rw.data)
        assert hashlib.sha256(pool.tobytes()).hexdigest() == g["pool_sha256"][-1]
    finally:
        bm.close()
