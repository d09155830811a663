"""The walk engine (engine 5, the product for large bases) through the C ABI:
bit for bit against its CPU model, against the oracle, and at the size it
serves, 6Li Nmax 6 with two- plus three-body forces (D = 186 894)."""
import ctypes
import os

import numpy as np
import pytest

import jupiterncsm_gb300 as jn
import oracle

pytestmark = pytest.mark.gpu
TOL = {1: 1e-12, 64: 1e-12, 32: 2e-6}      # mode -> tolerance relative to max|y| (1: exact integers)


def set_mode(H, mode):
    H.set_precision(32 if mode == 32 else 64)
    H.set_walk_arithmetic(mode == 64)


def emu5(d, Z, N, x, mode):
    L = ctypes.CDLL(os.path.join(os.path.dirname(__file__), "_build", "libplan_emu.so"))
    L.emu_open.restype = ctypes.c_void_p
    L.emu_open.argtypes = [ctypes.c_char_p] * 4 + [ctypes.c_int] * 3 + [ctypes.c_char_p, ctypes.c_int]
    L.emu_matvec5.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] * 2
    L.emu_close.argtypes = [ctypes.c_void_p]
    err = ctypes.create_string_buffer(1024)
    e = lambda s: s.encode()
    h = L.emu_open(e(f"{d}/comb.txt"), e(f"{d}/evaluation_order.txt"), e(f"{d}/index_lists"),
                   e(f"{d}/matrix_elements"), Z, N, 100, err, 1024)
    assert h, err.value
    y = np.zeros(len(x))
    assert L.emu_matvec5(h, x.ctypes.data, y.ctypes.data, 0, mode) == 0
    L.emu_close(h)
    return y


@pytest.mark.parametrize("name", ["he4_n4_2b", "li6_n2_3b", "he4_n6_3b"])
@pytest.mark.parametrize("mode", [1, 64, 32])
def test_walk_engine_is_exact_model(problem, name, mode):
    """The walk kernel gives bit for bit what its CPU model gives, in every arithmetic."""
    d, Z, N, *_ = problem(name)
    H = jn.Hamiltonian.from_dir(d, Z, N)
    H.set_engine(5)
    set_mode(H, mode)
    x = np.random.default_rng(31).standard_normal(H.dimension)
    got = H.matvec(x)
    assert np.array_equal(got.view(np.uint64), emu5(d, Z, N, x, mode).view(np.uint64))
    assert np.array_equal(got.view(np.uint64), H.matvec(x).view(np.uint64))
    ref = oracle.Port(d).matvec(x)
    assert np.abs(got - ref).max() <= TOL[mode] * np.abs(ref).max()
    H.close()


def test_walk_engine_accumulates_and_follows_new_elements(problem):
    """y += H x on device buffers, and a product after new matrix elements
    (the walk element arrays are rebuilt from them)."""
    import torch
    d, Z, N, *_ = problem("li6_n2_3b")
    H = jn.Hamiltonian.from_dir(d, Z, N)
    H.set_engine(5)
    rng = np.random.default_rng(32)
    x, y0 = rng.standard_normal(H.dimension), rng.standard_normal(H.dimension)
    xd, yd = torch.from_numpy(x).cuda(), torch.from_numpy(y0).cuda()
    H.matvec_device(xd.data_ptr(), yd.data_ptr(), True)
    H.synchronize()
    p = oracle.Port(d)
    want = p.matvec(x, y0.copy())
    assert np.abs(yd.cpu().numpy() - want).max() <= 1e-12 * np.abs(want).max()
    me = 0.5 * H.read_matrix_elements(os.path.join(d, "matrix_elements"))
    H.set_matrix_elements(me)
    got = H.matvec(x)
    want_half = p.matvec(x)     # H is linear in the matrix elements
    assert np.abs(got - 0.5 * want_half).max() <= 1e-12 * np.abs(want_half).max()
    H.close()


@pytest.fixture(scope="module")
def large(problem):
    """6Li Nmax 6, 2M = 2, two- plus three-body forces, one x and the oracle's y = H x."""
    d, Z, N, *_ = problem("li6_n6_3b")
    p = oracle.Port(d)
    x = np.random.default_rng(41).standard_normal(p.dimension)
    want = np.zeros(p.dimension)
    p.matvec_omp(x, want, os.cpu_count() or 1)
    p.close()
    return d, Z, N, x, want


def test_large_basis_is_the_walk_engine(large):
    d, Z, N, x, want = large
    H = jn.Hamiltonian.from_dir(d, Z, N)
    assert H.dimension == 186894
    assert H.active_engine() == 5
    H.close()


@pytest.mark.parametrize("mode", [1, 64, 32])
def test_large_basis_walk_products(large, mode):
    """At the size the walk engine serves: against the oracle in every
    arithmetic, and the exact-integer path bit for bit against the CPU model."""
    d, Z, N, x, want = large
    H = jn.Hamiltonian.from_dir(d, Z, N)
    set_mode(H, mode)
    got = H.matvec(x)
    assert np.abs(got - want).max() <= TOL[mode] * np.abs(want).max()
    if mode == 1:
        assert np.array_equal(got.view(np.uint64), emu5(d, Z, N, x, 1).view(np.uint64))
        assert np.array_equal(got.view(np.uint64), H.matvec(x).view(np.uint64))
    H.close()


def test_large_basis_block_tile_engine(large):
    """The block-tile engine (the batched solver's product) at the same size, FP64."""
    d, Z, N, x, want = large
    H = jn.Hamiltonian.from_dir(d, Z, N)
    H.set_engine(3)
    H.set_precision(64)
    got = H.matvec(x)
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    H.close()


def test_wide_neutron_basis_runs_on_the_walk_engine(tmp_path):
    """4 neutrons at Nmax 8 (D = 30 626; a sub-basis of 23 868 states, wider
    than a block-tile row): the context opens, the walk engine's products at
    both precisions match the oracle, and what needs the block tiles (engine
    3, the batched solver) is refused with the reason."""
    d = str(tmp_path / "n4")
    jn.generate(d, Z=0, N=4, nmax=8, nbody=2, basis_files=False)
    port = oracle.Port(d)
    x = np.random.default_rng(4).standard_normal(port.dimension)
    want = port.matvec(x)
    port.close()
    scale = np.abs(want).max()
    H = jn.Hamiltonian.from_dir(d, 0, 4)
    try:
        assert H.active_engine() == 5
        for bits, tol in ((64, 1e-12), (32, 2e-6)):
            H.set_precision(bits)
            assert np.abs(H.matvec(x) - want).max() <= tol * scale, bits
        with pytest.raises(jn.JnError, match="block-tile"):
            H.set_engine(3)
        me = H.read_matrix_elements(os.path.join(d, "matrix_elements"))
        with pytest.raises(jn.JnError, match="block-tile"):
            H.lanczos_batch([me], num_eigenvalues=2, max_iterations=20)
    finally:
        H.close()
