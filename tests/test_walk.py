"""The walk engine's plan (engine 5) executed on the CPU by a
statement-for-statement model of its kernel, against the oracle: every
index is checked, and the product matches the reference algorithm in all
three arithmetics (exact integers, FP64, FP32)."""
import ctypes

import numpy as np
import pytest

import oracle
from tests.test_plan import open_plan


def walk_lib():
    from tests.test_plan import emu_lib
    L = emu_lib()
    L.emu_matvec5.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] * 2
    L.emu_walk_stats.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    L.emu_walk_shape.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    L.emu_walk_validate.argtypes = [ctypes.c_void_p]
    L.emu_walk_validate.restype = ctypes.c_int64
    L.emu_walk_corrupt.argtypes = [ctypes.c_void_p, ctypes.c_int]
    return L


MODES = {1: 1e-12, 64: 1e-12, 32: 2e-6}     # mode -> tolerance relative to max|y| (1: exact integers)


@pytest.mark.parametrize("name", ["he4_n2_2b", "he4_n2_3b", "he4_n4_2b", "li6_n2_3b"])
@pytest.mark.parametrize("mode", sorted(MODES))
def test_walk_model_matches_port(problem, name, mode):
    d, Z, N, *_ = problem(name)
    _, h, err = open_plan(d, Z, N)
    assert h, err
    L = walk_lib()
    D = L.emu_dimension(h)
    p = oracle.Port(d)
    rng = np.random.default_rng(mode)
    x, y0 = rng.standard_normal(D), rng.standard_normal(D)
    want = p.matvec(x, y0.copy())
    got = y0.copy()
    assert L.emu_matvec5(h, x.ctypes.data, got.ctypes.data, 1, mode) == 0    # 0: every index in bounds
    assert np.abs(got - want).max() <= MODES[mode] * np.abs(want).max()
    L.emu_close(h)
    p.close()


def test_walk_plan_shape(problem):
    """Every multiply-add of the product is in the plan once: the padded
    count is at least the real one, lane chunks are 8, 4 or 2 wide, and the
    walk element array holds the transposed copies after the plan's elements."""
    d, Z, N, *_ = problem("he4_n4_2b")
    _, h, err = open_plan(d, Z, N)
    L = walk_lib()
    st = np.zeros(8)
    L.emu_walk_stats(h, st.ctypes.data)
    shape = np.zeros(13)
    L.emu_walk_shape(h, shape.ctypes.data)
    tasks, padded, slots, real = st[0], st[3], st[5], st[7]
    assert tasks > 0 and tasks == shape[0] + shape[4] + shape[8]
    assert real <= padded <= slots            # padding and idle lanes only add
    assert padded <= 1.6 * real               # chunk widths keep the padding small
    assert st[6] >= st[2] > 0                 # walk elements, row groups
    L.emu_close(h)


@pytest.mark.parametrize("name", ["he4_n4_2b", "li6_n2_3b"])
def test_walk_lane_sets_are_shared(problem, name):
    """A walk view's lane records are stored once: every stored lane word
    belongs to exactly one set that tasks read, and sets are read by the
    instructions of several matrix-element blocks."""
    d, Z, N, *_ = problem(name)
    _, h, err = open_plan(d, Z, N)
    assert h, err
    L = walk_lib()
    L.emu_walk_lane_sharing.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    out = np.zeros(3)
    L.emu_walk_lane_sharing(h, out.ctypes.data)
    stored, referenced, shared = out
    assert stored > 0 and referenced == stored
    assert shared > 0
    L.emu_close(h)


@pytest.mark.parametrize("name", ["he4_n2_2b", "he4_n2_3b", "he4_n4_2b", "li6_n2_3b", "he4_n6_3b"])
def test_walk_plan_is_sound(problem, name):
    """Every index the walk kernel reads stays inside its array, the entries'
    sign multipliers and padding are well formed, every group ends, and the
    kernel's read-ahead past the last row lands on the plan's zero spare words."""
    d, Z, N, *_ = problem(name)
    _, h, err = open_plan(d, Z, N)
    assert h, err
    L = walk_lib()
    assert L.emu_walk_validate(h) == 0
    L.emu_close(h)


@pytest.mark.parametrize("kind", [0, 1, 2])
def test_walk_plan_validator_finds_planted_defects(problem, kind):
    """The validator is not vacuous: a nonzero spare row word, an invalid
    multiplier code and a row slot beyond its piece's, each planted in the CPU
    model's copy of the plan, are reported."""
    d, Z, N, *_ = problem("he4_n4_2b")
    _, h, err = open_plan(d, Z, N)
    assert h, err
    L = walk_lib()
    assert L.emu_walk_validate(h) == 0
    assert L.emu_walk_corrupt(h, kind) == 0
    assert L.emu_walk_validate(h) > 0
    L.emu_close(h)
