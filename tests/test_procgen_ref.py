"""The reference's own world generator (src/procgen.zig:6-70) in its own
world format, vt_procgen_reference, against a restatement in plain Python of
the same source (util.LCG, VoxelBrickmap.set/get with bricks allocated on
first touch, the column loop and place_tree).  Both are written from the Zig
source; the Zig itself cannot be built here (no Zig toolchain), so this pins
the C++ to an independent reading rather than to the reference's binary."""
import numpy as np
import pytest


class Lcg:
    def __init__(self):
        self.seed = 0x46AE4F

    def rand(self):
        self.seed = (self.seed * 1103515245 + 12345) & 0xFFFFFFFF
        return self.seed


class Brickmap:
    def __init__(self, dim):
        self.dim, self.cd = dim, dim // 8
        self.chunks = np.zeros(self.cd ** 3, np.uint32)
        self.bricks = []

    def _ci(self, x, y, z):
        return x // 8 + self.cd * (y // 8 + (z // 8) * self.cd)

    def set(self, x, y, z, ty, solid):
        # at dim 512 the reference's own guard (x, z < 500) keeps every write
        # inside the map; at smaller dims a tree at the far edge would write
        # past it (unchecked in the reference): those writes are dropped
        if not (0 <= x < self.dim and 0 <= y < self.dim and 0 <= z < self.dim):
            return
        ci = self._ci(x, y, z)
        if self.chunks[ci] == 0:
            self.bricks.append(np.zeros(512, np.uint32))
            self.chunks[ci] = len(self.bricks)
        self.bricks[self.chunks[ci] - 1][x % 8 + ((y % 8) + (z % 8) * 8) * 8] = (ty & 0xFFFFFFF) | (int(solid) << 28)

    def get(self, x, y, z):
        ci = self._ci(x, y, z)
        return 0 if self.chunks[ci] == 0 else int(self.bricks[self.chunks[ci] - 1][x % 8 + ((y % 8) + (z % 8) * 8) * 8])


def procgen_py(dim, noise):
    w, lcg = Brickmap(dim), Lcg()
    for x in range(dim):
        for z in range(dim):
            for y in range(16):
                w.set(x, y, z, 13, True)
    for x in range(dim):
        for z in range(dim):
            vh = int(max(np.float32(np.float32(noise[x, z]) * np.float32(dim)) * np.float32(0.1), np.float32(0)))
            for h in range(vh):
                w.set(x, h, z, 21 + lcg.rand() % 3, True)
                if h <= 15:
                    w.set(x, h, z, 25 + lcg.rand() % 3, True)
                elif h == vh - 1 and h > 15:
                    w.set(x, h, z, lcg.rand() % 6, True)
            if vh > 16:
                if w.get(x, vh, z) != 0:
                    continue
                if lcg.rand() % 5 == 0:
                    w.set(x, vh, z, 7 + lcg.rand() % 5, False)
                if lcg.rand() % 71 == 0:
                    w.set(x, vh, z, 7 + 5, True)
                if lcg.rand() % 420 == 0 and x < 500 and z < 500 and x > 5 and z > 5:
                    trunk = lcg.rand() % 4 + 4
                    w.set(x + 1, vh, z + 1, 15, True)
                    for o in range(trunk):
                        w.set(x + 1, vh + o, z + 1, 14 + lcg.rand() % 3, True)
                    for a in range(3):
                        for b in range(3):
                            for c in range(3):
                                w.set(x + a, vh + trunk + b, z + c, 18 + lcg.rand() % 2, True)
            lcg.rand()
    return w.chunks, (np.concatenate(w.bricks) if w.bricks else np.zeros(0, np.uint32))


@pytest.mark.parametrize("dim,seed", [(64, 1), (96, 2), (200, 3)])
def test_procgen_matches_python_restatement(vtlib, dim, seed):
    rng = np.random.default_rng(seed)
    # smooth-ish noise with enough tall columns (> 16) for grass, flowers and trees
    base = rng.uniform(-0.2, 1.0, (dim // 8 + 2, dim // 8 + 2))
    xs = np.arange(dim) / 8.0
    noise = np.array([[np.interp(z / 8.0, np.arange(base.shape[1]), base[int(x), :]) for z in range(dim)]
                      for x in xs], np.float32)
    noise += rng.normal(0, 0.05, noise.shape).astype(np.float32)
    chunks, bricks = vtlib.procgen_reference(dim, noise)
    want_chunks, want_bricks = procgen_py(dim, noise)
    assert np.array_equal(chunks, want_chunks)
    assert np.array_equal(bricks, want_bricks)
    vals = bricks >> 28
    assert (bricks & 0xFFFFFFF == 13).any() and (bricks != 0).sum() >= dim * dim * 16
    tys = set(np.unique(bricks[bricks != 0] & 0xFFFFFFF).tolist())
    if dim >= 200:   # columns above the floor (vh > 16): grass tufts, flowers, trees
        assert {14, 15, 18}.issubset(tys) and (tys & {7, 8, 9, 10, 11}), tys
    assert vals.max() <= 1


def test_procgen_default_noise_and_capacity(vtlib):
    chunks, bricks = vtlib.procgen_reference(128, None, seed=5)
    assert chunks.max() == bricks.size // 512 and bricks.size % 512 == 0
    # the default noise is seeded: same seed, same world; another seed, another
    c2, b2 = vtlib.procgen_reference(128, None, seed=5)
    c3, b3 = vtlib.procgen_reference(128, None, seed=6)
    assert np.array_equal(bricks, b2) and not np.array_equal(bricks, b3)


def test_procgen_rejects_bad_dims(vtlib):
    import ctypes as C
    n = C.c_size_t()
    ch = np.zeros(8, np.uint32)
    assert vtlib.load().vt_procgen_reference(12, 0.0, 0.0, None, 0, ch.ctypes.data, None, 0, C.byref(n)) == 1
