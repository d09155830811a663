"""The device plan (CSR views, terms, tiles, chunks) executed on the CPU by a
statement-for-statement model of the kernels, against the oracle; and the
host-side validation that keeps every device access in bounds."""
import ctypes
import os
import shutil

import numpy as np
import pytest

import oracle

EMU = os.path.join(os.path.dirname(__file__), "_build", "libplan_emu.so")


def emu_lib():
    L = ctypes.CDLL(EMU)
    L.emu_open.restype = ctypes.c_void_p
    L.emu_open.argtypes = [ctypes.c_char_p] * 4 + [ctypes.c_int] * 3 + [ctypes.c_char_p, ctypes.c_int]
    L.emu_matvec.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int]
    L.emu_dimension.restype = ctypes.c_long
    L.emu_dimension.argtypes = [ctypes.c_void_p]
    L.emu_units.argtypes = [ctypes.c_void_p]
    L.emu_close.argtypes = [ctypes.c_void_p]
    return L


def open_plan(d, Z, N, units=1216):
    L = emu_lib()
    err = ctypes.create_string_buffer(2048)
    e = lambda s: s.encode()
    h = L.emu_open(e(f"{d}/comb.txt"), e(f"{d}/evaluation_order.txt"), e(f"{d}/index_lists"),
                   e(f"{d}/matrix_elements"), Z, N, units, err, 2048)
    return L, h, err.value.decode()


@pytest.mark.parametrize("name", ["he4_n2_2b", "he4_n2_3b", "he4_n4_2b", "li6_n2_3b"])
@pytest.mark.parametrize("units", [1, 64, 1216])
def test_plan_matches_port(problem, name, units):
    d, Z, N, *_ = problem(name)
    L, h, err = open_plan(d, Z, N, units)
    assert h, err
    D = L.emu_dimension(h)
    p = oracle.Port(d)
    rng = np.random.default_rng(units)
    x, y0 = rng.standard_normal(D), rng.standard_normal(D)
    a = y0.copy()
    L.emu_matvec(h, x.ctypes.data, a.ctypes.data, 1)
    b = p.matvec(x, y0.copy())
    assert np.abs(a - b).max() <= 1e-12 * np.abs(b).max()
    c = np.full(D, np.nan)
    L.emu_matvec(h, x.ctypes.data, c.ctypes.data, 0)
    assert np.abs(c - (b - y0)).max() <= 1e-12 * np.abs(b).max()
    L.emu_close(h)
    p.close()


def corrupt_copy(src, dst):
    shutil.copytree(src, dst)
    return dst


def first_list(d):
    return sorted(os.listdir(f"{d}/index_lists"), key=lambda s: int(s.split("_")[-1]))[0]


def test_rejects_out_of_range_index(problem, tmp_path):
    d, Z, N, *_ = problem("he4_n2_2b")
    c = corrupt_copy(d, str(tmp_path / "c"))
    f = f"{c}/index_lists/{first_list(c)}"
    a = np.fromfile(f, dtype=np.int32)
    a[1] = 1 << 20
    a.tofile(f)
    L, h, err = open_plan(c, Z, N)
    assert not h and "outside" in err


def test_rejects_out_of_range_matrix_index(problem, tmp_path):
    d, Z, N, *_ = problem("he4_n2_2b")
    c = corrupt_copy(d, str(tmp_path / "c"))
    f = f"{c}/index_lists/{first_list(c)}"
    a = np.fromfile(f, dtype=np.uint32)
    a[2] = 0x80000000 | 0x7ffffff0
    a.tofile(f)
    L, h, err = open_plan(c, Z, N)
    assert not h and "matrix index" in err


def test_rejects_truncated_list(problem, tmp_path):
    d, Z, N, *_ = problem("he4_n2_2b")
    c = corrupt_copy(d, str(tmp_path / "c"))
    f = f"{c}/index_lists/{first_list(c)}"
    open(f, "ab").write(b"\x01\x02")
    L, h, err = open_plan(c, Z, N)
    assert not h and "whole index triples" in err


def test_rejects_short_matrix_file(problem, tmp_path):
    d, Z, N, *_ = problem("he4_n2_2b")
    c = corrupt_copy(d, str(tmp_path / "c"))
    name = sorted(os.listdir(f"{c}/matrix_elements"))[0]
    f = f"{c}/matrix_elements/{name}"
    raw = open(f, "rb").read()
    open(f, "wb").write(raw[:-8])
    L, h, err = open_plan(c, Z, N)
    assert not h and "matrix" in err


def test_missing_matrix_file_reports_path(problem, tmp_path):
    d, Z, N, *_ = problem("he4_n2_2b")
    c = corrupt_copy(d, str(tmp_path / "c"))
    name = sorted(os.listdir(f"{c}/matrix_elements"))[-1]
    os.remove(f"{c}/matrix_elements/{name}")
    L, h, err = open_plan(c, Z, N)
    assert not h and "Could not open block file" in err and name in err


def test_missing_file_reports_path(problem, tmp_path):
    d, Z, N, *_ = problem("he4_n2_2b")
    c = corrupt_copy(d, str(tmp_path / "c"))
    os.remove(f"{c}/index_lists/{first_list(c)}")
    L, h, err = open_plan(c, Z, N)
    assert not h and "Could not open" in err


@pytest.mark.parametrize("name", ["he4_n2_2b", "he4_n2_3b", "he4_n4_2b", "li6_n2_3b"])
@pytest.mark.parametrize("units", [1, 97, 608])
def test_block_tile_plan_model_matches_port(problem, name, units):
    """CPU model of the fixed-point block-tile kernels: every index checked,
    FP64 within 1e-12 and FP32 within 2e-6 of the oracle."""
    d, Z, N, *_ = problem(name)
    L, h, err = open_plan(d, Z, N, units)
    assert h, err
    L.emu_matvec3.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] * 2
    D = L.emu_dimension(h)
    x = np.random.default_rng(units).standard_normal(D)
    want = oracle.Port(d).matvec(x)
    for f32, tol in ((0, 1e-12), (1, 2e-6)):
        y = np.zeros(D)
        assert L.emu_matvec3(h, x.ctypes.data, y.ctypes.data, 0, f32) == 0
        assert np.abs(y - want).max() <= tol * np.abs(want).max()
    L.emu_close(h)


@pytest.mark.parametrize("name", ["he4_n2_2b", "he4_n2_3b", "he4_n4_2b", "li6_n2_3b"])
def test_panel_plan_model_matches_port(problem, name):
    """CPU model of the panel kernel (compacted coefficients, runs rounded
    once, transposes per product): every index checked, FP64 within 1e-12
    and FP32 within 2e-6 of the oracle."""
    d, Z, N, *_ = problem(name)
    L, h, err = open_plan(d, Z, N)
    assert h, err
    L.emu_matvec4.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] * 2
    D = L.emu_dimension(h)
    x = np.random.default_rng(7).standard_normal(D)
    want = oracle.Port(d).matvec(x)
    for f32, tol in ((0, 1e-12), (1, 2e-6)):
        y = np.zeros(D)
        assert L.emu_matvec4(h, x.ctypes.data, y.ctypes.data, 0, f32) == 0
        assert np.abs(y - want).max() <= tol * np.abs(want).max()
    L.emu_close(h)


@pytest.mark.parametrize("name", ["he4_n4_2b", "he4_n2_3b", "li6_n2_3b"])
def test_panel_list_order_spreads_atomics(problem, name):
    """Each list's panel order is a permutation of its entries, and it keeps
    equal destinations (and sources) apart: the product's shared-memory
    atomics take fewer bank wavefronts than with the lists in by-out order."""
    d, Z, N, *_ = problem(name)
    L, h, err = open_plan(d, Z, N)
    assert h, err
    L.emu_panel_wavefronts.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    got, ref = np.zeros(4), np.zeros(4)
    assert L.emu_panel_wavefronts(h, 0, got.ctypes.data) == 0
    assert L.emu_panel_wavefronts(h, 1, ref.ctypes.data) == 0
    assert got[0] == ref[0] and got[2] == ref[2] and got[0] > 0
    print(name, "wavefronts per atomic: forward %.2f -> %.2f, transpose %.2f -> %.2f"
          % (ref[1] / ref[0], got[1] / got[0], ref[3] / max(ref[2], 1), got[3] / max(got[2], 1)))
    assert got[1] + got[3] < 0.8 * (ref[1] + ref[3])
    L.emu_close(h)


@pytest.mark.parametrize("name", ["he4_n4_2b", "li6_n2_3b", "he4_n6_3b"])
def test_plans_do_not_depend_on_the_host_thread_count(problem, name, monkeypatch):
    """The host builds its plans on all cores; with one thread (JN_HOST_THREADS=1)
    every array a product reads (engines 2, 3 and 5, the walk element arrays,
    the bounds) is the same, byte for byte."""
    d, Z, N, *_ = problem(name)
    digests = []
    for threads in ("1", "3", None):
        if threads:
            monkeypatch.setenv("JN_HOST_THREADS", threads)
        else:
            monkeypatch.delenv("JN_HOST_THREADS", raising=False)
        L, h, err = open_plan(d, Z, N)
        assert h, err
        L.emu_plan_digest.restype = ctypes.c_uint64
        L.emu_plan_digest.argtypes = [ctypes.c_void_p]
        digests.append(L.emu_plan_digest(h))
        L.emu_close(h)
    assert digests[0] != 0 and digests[0] == digests[1] == digests[2]


def test_plans_built_concurrently_match(problem):
    """Plans opened from several threads at once (each build uses all host
    cores) equal the plans built one after another: the builds share no state."""
    import threading
    names = ["he4_n4_2b", "li6_n2_3b", "he4_n2_3b", "he4_n4_2b"]
    probs = [problem(n) for n in names]

    def digest(d, Z, N):
        L, h, err = open_plan(d, Z, N)
        assert h, err
        L.emu_plan_digest.restype = ctypes.c_uint64
        L.emu_plan_digest.argtypes = [ctypes.c_void_p]
        v = L.emu_plan_digest(h)
        L.emu_close(h)
        return v

    want = [digest(d, Z, N) for d, Z, N, *_ in probs]
    got = [None] * len(probs)

    def run(i):
        d, Z, N, *_ = probs[i]
        got[i] = digest(d, Z, N)

    ts = [threading.Thread(target=run, args=(i,)) for i in range(len(probs))]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert got == want and all(want)


def test_empty_lists_match_port(problem, tmp_path):
    """Index lists with no entries (0-byte files; the reference reads size / 12
    triples) contribute nothing: every engine's model still matches the oracle
    and the walk plan stays sound."""
    d0, Z, N, *_ = problem("he4_n2_3b")
    d = corrupt_copy(d0, str(tmp_path / "c"))
    names = sorted(os.listdir(f"{d}/index_lists"), key=lambda s: int(s.split("_")[-1]))
    for n in names[:3] + names[-2:]:
        open(f"{d}/index_lists/{n}", "wb").close()
    L, h, err = open_plan(d, Z, N)
    assert h, err
    D = L.emu_dimension(h)
    x = np.random.default_rng(3).standard_normal(D)
    want = oracle.Port(d).matvec(x)
    scale = np.abs(want).max()
    y = np.zeros(D)
    L.emu_matvec(h, x.ctypes.data, y.ctypes.data, 0)
    assert np.abs(y - want).max() <= 1e-12 * scale
    for fn, modes in (("emu_matvec3", ((0, 1e-12), (1, 2e-6))), ("emu_matvec4", ((0, 1e-12), (1, 2e-6))),
                      ("emu_matvec5", ((1, 1e-12), (64, 1e-12), (32, 2e-6)))):
        f = getattr(L, fn)
        f.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] * 2
        for mode, tol in modes:
            y = np.zeros(D)
            assert f(h, x.ctypes.data, y.ctypes.data, 0, mode) == 0, (fn, mode)
            assert np.abs(y - want).max() <= tol * scale, (fn, mode)
    L.emu_walk_validate.restype = ctypes.c_int64
    L.emu_walk_validate.argtypes = [ctypes.c_void_p]
    assert L.emu_walk_validate(h) == 0
    L.emu_close(h)


@pytest.mark.parametrize("name", ["he4_n2_3b", "li6_n2_3b"])
def test_power_of_two_scaling_is_exact_in_the_models(problem, name):
    """Inside the fixed-point range, x scaled by 2^60 (or 2^-40) gives y scaled
    by the same power of two, bit for bit, in every engine's model and
    arithmetic: the unit exponent moves with max|x| and nothing else rounds
    differently."""
    d, Z, N, *_ = problem(name)
    L, h, err = open_plan(d, Z, N)
    assert h, err
    D = L.emu_dimension(h)
    x = np.random.default_rng(11).standard_normal(D)
    for fn, modes in (("emu_matvec3", (0, 1)), ("emu_matvec4", (0, 1)), ("emu_matvec5", (1, 64, 32))):
        f = getattr(L, fn)
        f.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] * 2
        for mode in modes:
            a = np.zeros(D)
            assert f(h, x.ctypes.data, a.ctypes.data, 0, mode) == 0
            for k in (60, -40):
                xs = x * 2.0 ** k
                b = np.zeros(D)
                assert f(h, xs.ctypes.data, b.ctypes.data, 0, mode) == 0
                assert np.array_equal(b, a * 2.0 ** k), (fn, mode, k)
    L.emu_close(h)


def test_wide_neutron_basis_opens_without_block_tiles(tmp_path):
    """4 neutrons at Nmax 8 (D = 30 626) have a sub-basis of 23 868 states,
    wider than a block-tile row.  The plan still opens: the block tiles are
    marked unavailable, and the walk engine's model matches the oracle."""
    import jupiterncsm_gb300 as jn
    d = str(tmp_path / "n4")
    jn.generate(d, Z=0, N=4, nmax=8, nbody=2, basis_files=False)
    L, h, err = open_plan(d, 0, 4)
    assert h, err
    L.emu_btiles_off.argtypes = [ctypes.c_void_p]
    assert L.emu_btiles_off(h) == 1
    D = L.emu_dimension(h)
    x = np.random.default_rng(2).standard_normal(D)
    port = oracle.Port(d)
    want = port.matvec(x)
    port.close()
    scale = np.abs(want).max()
    L.emu_matvec5.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] * 2
    for mode, tol in ((1, 1e-12), (64, 1e-12), (32, 2e-6)):
        y = np.zeros(D)
        assert L.emu_matvec5(h, x.ctypes.data, y.ctypes.data, 0, mode) == 0
        assert np.abs(y - want).max() <= tol * scale, mode
    L.emu_walk_validate.restype = ctypes.c_int64
    L.emu_walk_validate.argtypes = [ctypes.c_void_p]
    assert L.emu_walk_validate(h) == 0
    L.emu_close(h)
    assert jn.inspect(d, 0, 4)["dimension"] == D


def test_duplicate_list_entries_match_port(problem, tmp_path):
    """Index lists that hold some triples more than once (the reference adds
    each copy): every engine's model still matches the oracle, and the walk
    plan stays sound."""
    d0, Z, N, *_ = problem("he4_n4_2b")
    d = corrupt_copy(d0, str(tmp_path / "dup"))
    names = sorted(os.listdir(f"{d}/index_lists"), key=lambda s: int(s.split("_")[-1]))
    rng = np.random.default_rng(0)
    for n in names[::7]:
        f = f"{d}/index_lists/{n}"
        a = np.fromfile(f, dtype=np.int32).reshape(-1, 3)
        if len(a):
            pick = a[rng.integers(0, len(a), size=max(1, len(a) // 3))]
            np.concatenate([a, pick, a[:1]]).astype(np.int32).tofile(f)
    L, h, err = open_plan(d, Z, N)
    assert h, err
    D = L.emu_dimension(h)
    x = np.random.default_rng(1).standard_normal(D)
    port = oracle.Port(d)
    want = port.matvec(x)
    port.close()
    scale = np.abs(want).max()
    y = np.zeros(D)
    L.emu_matvec(h, x.ctypes.data, y.ctypes.data, 0)
    assert np.abs(y - want).max() <= 1e-12 * scale
    for fn, modes in (("emu_matvec3", ((0, 1e-12), (1, 2e-6))), ("emu_matvec4", ((0, 1e-12), (1, 2e-6))),
                      ("emu_matvec5", ((1, 1e-12), (64, 1e-12), (32, 2e-6)))):
        f = getattr(L, fn)
        f.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] * 2
        for mode, tol in modes:
            y = np.zeros(D)
            assert f(h, x.ctypes.data, y.ctypes.data, 0, mode) == 0, (fn, mode)
            assert np.abs(y - want).max() <= tol * scale, (fn, mode)
    L.emu_walk_validate.restype = ctypes.c_int64
    L.emu_walk_validate.argtypes = [ctypes.c_void_p]
    assert L.emu_walk_validate(h) == 0
    L.emu_close(h)
