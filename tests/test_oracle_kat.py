"""Known-answer rays for the mode-P oracle (CPU only).

Each case is worked out by hand from the traversal rules the oracle restates:
plane crossing times t = (k - o) / d, events ordered by t with ties to the
higher axis (map.glsl:158), zero direction components replaced by 0.001
(map.glsl:85-90), faces 2*axis + (d > 0 ? 0 : 1) (map.glsl:119-127) and the
max-step loop (map.glsl:106).
"""
import numpy as np
import pytest


def one_voxel_world(oracle, dims=(32, 32, 32), cells=((10, 5, 7),), mat=3):
    X, Y, Z = dims
    m = np.zeros((Z, Y, X), dtype=np.uint8)
    for (x, y, z) in cells:
        m[z, y, x] = mat
    return oracle.OracleWorld(m)


def test_axis_aligned_positive(oracle):
    w = one_voxel_world(oracle)
    tr = oracle.trace_one(w, (0.5, 5.5, 7.5), (1.0, 0.0, 0.0), 512)
    assert tr.hit == 1
    assert tuple(tr.cell) == (10, 5, 7)
    assert tr.face == 0                      # entered moving +x: the -x face
    assert tr.t == pytest.approx(9.5, abs=0)  # plane x=10 at (10 - 0.5) / 1
    assert tr.steps == 10
    assert tr.material == 3


def test_axis_aligned_negative(oracle):
    w = one_voxel_world(oracle)
    tr = oracle.trace_one(w, (20.5, 5.5, 7.5), (-1.0, 0.0, 0.0), 512)
    assert tr.hit == 1 and tuple(tr.cell) == (10, 5, 7)
    assert tr.face == 1
    assert tr.t == 9.5                        # plane x=11 at (11 - 20.5) / -1
    assert tr.steps == 10                     # planes 20, 19, ..., 11


def test_max_step_cutoff_exact(oracle):
    w = one_voxel_world(oracle)
    # the hit cell is reached after 10 crossings: tested iff 10 < max_steps
    assert oracle.trace_one(w, (0.5, 5.5, 7.5), (1.0, 0.0, 0.0), 11).hit == 1
    miss = oracle.trace_one(w, (0.5, 5.5, 7.5), (1.0, 0.0, 0.0), 10)
    assert miss.hit == 0 and miss.face == -1 and miss.t == -1.0


def test_two_axis_tie_goes_to_higher_axis(oracle):
    # from (0.5, 0.5, 0.5) along (1, 1, 0): x and y planes cross at t = 0.5;
    # the y crossing comes first, so the ray visits (0,1,0) before (1,1,0)
    w = one_voxel_world(oracle, cells=((0, 1, 0),))
    tr = oracle.trace_one(w, (0.5, 0.5, 0.5), (1.0, 1.0, 0.0), 64)
    assert tr.hit == 1 and tuple(tr.cell) == (0, 1, 0) and tr.face == 2 and tr.t == 0.5 and tr.steps == 1
    # (1,0,0) is never visited
    w = one_voxel_world(oracle, cells=((1, 0, 0),))
    assert oracle.trace_one(w, (0.5, 0.5, 0.5), (1.0, 1.0, 0.0), 64).hit == 0
    w = one_voxel_world(oracle, cells=((1, 1, 0),))
    tr = oracle.trace_one(w, (0.5, 0.5, 0.5), (1.0, 1.0, 0.0), 64)
    assert tr.hit == 1 and tr.face == 0 and tr.t == 0.5 and tr.steps == 2


def test_three_axis_tie_order_z_y_x(oracle):
    # all three planes at t = 0.5: z, then y, then x
    for cell, face, steps in (((0, 0, 1), 4, 1), ((0, 1, 1), 2, 2), ((1, 1, 1), 0, 3)):
        w = one_voxel_world(oracle, cells=(cell,))
        tr = oracle.trace_one(w, (0.5, 0.5, 0.5), (1.0, 1.0, 1.0), 64)
        assert tr.hit == 1 and tuple(tr.cell) == cell and tr.face == face and tr.t == 0.5 and tr.steps == steps
    for cell in ((1, 0, 0), (0, 1, 0), (1, 0, 1)):
        w = one_voxel_world(oracle, cells=(cell,))
        assert oracle.trace_one(w, (0.5, 0.5, 0.5), (1.0, 1.0, 1.0), 4).hit == 0


def test_zero_direction_is_fixed_to_0001(oracle):
    # (0, 0, 0) becomes (0.001, 0.001, 0.001): the same three-way tie
    w = one_voxel_world(oracle, cells=((0, 1, 1),))
    tr = oracle.trace_one(w, (0.5, 0.5, 0.5), (0.0, 0.0, 0.0), 64)
    assert tr.hit == 1 and tr.face == 2 and tr.steps == 2
    inv = np.float32(1.0) / np.float32(0.001)
    assert tr.t == np.float32(0.5) * inv   # fma(1, inv, -(0.5 * inv)), exact


def test_start_inside_solid(oracle):
    w = one_voxel_world(oracle)
    tr = oracle.trace_one(w, (10.25, 5.5, 7.5), (-1.0, 0.2, 0.3), 16)
    assert tr.hit == 1 and tr.steps == 0 and tr.t == 0.0
    assert tr.face == 1   # initial axis 0 (map.glsl:98), moving -x


def test_entry_from_outside(oracle):
    w = one_voxel_world(oracle, cells=((0, 5, 7),))
    tr = oracle.trace_one(w, (-3.5, 5.5, 7.5), (1.0, 0.0, 0.0), 16)
    assert tr.hit == 1 and tuple(tr.cell) == (0, 5, 7) and tr.face == 0 and tr.t == 3.5 and tr.steps == 0
    # negative origin on another axis, entering through the y face
    w = one_voxel_world(oracle, cells=((4, 0, 4),))
    tr = oracle.trace_one(w, (4.5, -2.0, 4.5), (0.0, 1.0, 0.0), 16)
    assert tr.hit == 1 and tr.face == 2 and tr.t == 2.0


def test_box_missed_or_behind(oracle):
    w = one_voxel_world(oracle)
    assert oracle.trace_one(w, (-5.0, 50.0, 5.0), (0.0, 1.0, 0.0), 512).hit == 0    # moving away above
    assert oracle.trace_one(w, (40.0, 5.5, 7.5), (1.0, 0.0, 0.0), 512).hit == 0     # box behind
    assert oracle.trace_one(w, (-1.0, -1.0, 40.0), (1.0, 1.0, 0.0), 512).hit == 0   # passes beside


def test_exit_through_far_side(oracle):
    w = one_voxel_world(oracle, cells=())
    tr = oracle.trace_one(w, (0.5, 0.5, 0.5), (1.0, 0.25, 0.125), 10000)
    assert tr.hit == 0 and tr.steps > 31


def test_counters_unit_world(oracle):
    # one chunk, one occupied brick at (8..11, 4..7, 4..7): a +x ray through
    # y=5, z=7 consults bricks x=0..2 of that row (3 words) and one coarse word
    w = one_voxel_world(oracle)
    tr = oracle.trace_one(w, (0.5, 5.5, 7.5), (1.0, 0.0, 0.0), 512)
    assert tr.mask_words == 3 and tr.coarse_words == 1


def test_sincos_accuracy(oracle):
    lib = oracle.load()
    xs = np.linspace(0.0, 6.28, 2001, dtype=np.float32)
    s = np.array([lib.vto_sinf(float(x)) for x in xs])
    c = np.array([lib.vto_cosf(float(x)) for x in xs])
    assert np.max(np.abs(s - np.sin(xs.astype(np.float64)))) < 3e-7
    assert np.max(np.abs(c - np.cos(xs.astype(np.float64)))) < 3e-7
