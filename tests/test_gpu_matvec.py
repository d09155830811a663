"""GPU matrix-vector product through the C ABI against the oracle."""
import json
import os

import numpy as np
import pytest

import jupiterncsm_gb300 as jn
import oracle

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TOL = 1e-12   # relative to max|y|: FP64 path, only the summation order differs


@pytest.mark.parametrize("name", ["he4_n2_2b", "he4_n2_3b", "li6_n2_3b"])
def test_golden_reference_products(tmp_path, name):
    meta = json.load(open(os.path.join(GOLDEN, f"{name}.json")))
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    d = str(tmp_path / name)
    jn.generate(d, basis_files=False, **meta["config"])
    H = jn.Hamiltonian.from_dir(d, meta["config"]["Z"], meta["config"]["N"])
    y = H.matvec(g["x"])
    assert np.abs(y - g["y"]).max() <= TOL * np.abs(g["y"]).max()
    H.close()


@pytest.mark.parametrize("name", ["he4_n2_2b", "he4_n2_3b", "he4_n4_2b", "li6_n2_3b", "he4_n6_3b"])
def test_matches_port_and_accumulates(problem, name):
    d, Z, N, *_ = problem(name)
    H = jn.Hamiltonian.from_dir(d, Z, N)
    p = oracle.Port(d)
    rng = np.random.default_rng(11)
    x, y0 = rng.standard_normal(H.dimension), rng.standard_normal(H.dimension)
    want = p.matvec(x, y0.copy())
    got = H.matvec(x, y0.copy())
    assert np.abs(got - want).max() <= TOL * np.abs(want).max()
    H.close()
    p.close()


def test_bit_identical_repeats(problem):
    d, Z, N, *_ = problem("he4_n6_3b")
    H = jn.Hamiltonian.from_dir(d, Z, N)
    x = np.random.default_rng(3).standard_normal(H.dimension)
    a = H.matvec(x)
    b = H.matvec(x)
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
    H.close()


def test_unit_vector_products_rebuild_dense_h(problem):
    from oracle import dense_h
    d, Z, N, nmax, nbody = problem("he4_n2_3b")
    H = jn.Hamiltonian.from_dir(d, Z, N)
    D = H.dimension
    M = np.column_stack([H.matvec(np.eye(D)[j]) for j in range(D)])
    Hd = dense_h.build_dense_h(d, Z, N, nmax, nbody=nbody)
    assert np.abs(M - Hd).max() <= TOL * np.abs(Hd).max()
    H.close()


def test_file_level_drop_in(problem, tmp_path):
    d, Z, N, *_ = problem("he4_n4_2b")
    blocks = oracle.read_blocks(d)
    D = sum(a * b for _, a, b in blocks)
    rng = np.random.default_rng(4)
    x, y0 = rng.standard_normal(D), rng.standard_normal(D)
    oracle.write_vector_dir(str(tmp_path / "in"), blocks, x)
    oracle.write_vector_dir(str(tmp_path / "out"), blocks, y0)
    H = jn.Hamiltonian.from_dir(d, Z, N)
    H.matvec_files(str(tmp_path / "out"), str(tmp_path / "in"))
    got = oracle.read_vector_dir(str(tmp_path / "out"), blocks)
    want = oracle.Port(d).matvec(x, y0.copy())
    assert np.abs(got - want).max() <= TOL * np.abs(want).max()
    H.close()


def test_open_errors_are_status_codes(problem, tmp_path):
    d, Z, N, *_ = problem("he4_n2_2b")
    with pytest.raises(jn.JnError) as e:
        jn.Hamiltonian(comb=f"{d}/nope.txt", order=f"{d}/evaluation_order.txt", lists=f"{d}/index_lists",
                       mes=f"{d}/matrix_elements", Z=Z, N=N)
    assert e.value.status == 2


def test_runfile_open(problem):
    d, Z, N, *_ = problem("he4_n2_3b")
    H = jn.Hamiltonian(f"{d}/bacchus.conf")
    x = np.random.default_rng(2).standard_normal(H.dimension)
    want = oracle.Port(d).matvec(x)
    assert np.abs(H.matvec(x) - want).max() <= TOL * np.abs(want).max()
    H.close()


def emu3(d, Z, N, x, f32):
    import ctypes
    L = ctypes.CDLL(os.path.join(os.path.dirname(__file__), "_build", "libplan_emu.so"))
    L.emu_open.restype = ctypes.c_void_p
    L.emu_open.argtypes = [ctypes.c_char_p] * 4 + [ctypes.c_int] * 3 + [ctypes.c_char_p, ctypes.c_int]
    L.emu_matvec3.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] * 2
    L.emu_close.argtypes = [ctypes.c_void_p]
    err = ctypes.create_string_buffer(1024)
    e = lambda s: s.encode()
    import subprocess
    out = subprocess.run(["nvidia-smi", "--query-gpu=multiprocessor_count", "--format=csv,noheader"],
                         capture_output=True, text=True)
    sms = int(out.stdout.split()[0]) if out.returncode == 0 and out.stdout.strip() else 152
    h = L.emu_open(e(f"{d}/comb.txt"), e(f"{d}/evaluation_order.txt"), e(f"{d}/index_lists"),
                   e(f"{d}/matrix_elements"), Z, N, sms * 48, err, 1024)
    y = np.zeros(len(x))
    assert L.emu_matvec3(h, x.ctypes.data, y.ctypes.data, 0, int(f32)) == 0
    L.emu_close(h)
    return y


@pytest.mark.parametrize("name", ["he4_n4_2b", "li6_n2_3b", "he4_n6_3b"])
@pytest.mark.parametrize("bits", [64, 32])
def test_block_tile_engine_is_exact_model(problem, name, bits):
    """The fixed-point engine gives bit for bit what its CPU model gives."""
    d, Z, N, *_ = problem(name)
    H = jn.Hamiltonian.from_dir(d, Z, N)
    H.set_engine(3)
    H.set_precision(bits)
    x = np.random.default_rng(21).standard_normal(H.dimension)
    got = H.matvec(x)
    want = emu3(d, Z, N, x, bits == 32)
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
    ref = oracle.Port(d).matvec(x)
    tol = 1e-12 if bits == 64 else 2e-6
    assert np.abs(got - ref).max() <= tol * np.abs(ref).max()
    H.close()


def emu4(d, Z, N, x, f32):
    import ctypes
    L = ctypes.CDLL(os.path.join(os.path.dirname(__file__), "_build", "libplan_emu.so"))
    L.emu_open.restype = ctypes.c_void_p
    L.emu_open.argtypes = [ctypes.c_char_p] * 4 + [ctypes.c_int] * 3 + [ctypes.c_char_p, ctypes.c_int]
    L.emu_matvec4.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] * 2
    L.emu_close.argtypes = [ctypes.c_void_p]
    err = ctypes.create_string_buffer(1024)
    e = lambda s: s.encode()
    h = L.emu_open(e(f"{d}/comb.txt"), e(f"{d}/evaluation_order.txt"), e(f"{d}/index_lists"),
                   e(f"{d}/matrix_elements"), Z, N, 1216, err, 1024)
    y = np.zeros(len(x))
    assert L.emu_matvec4(h, x.ctypes.data, y.ctypes.data, 0, int(f32)) == 0
    L.emu_close(h)
    return y


@pytest.mark.parametrize("name", ["he4_n4_2b", "li6_n2_3b", "he4_n6_3b"])
@pytest.mark.parametrize("bits", [64, 32])
def test_panel_engine_is_exact_model(problem, name, bits):
    """The panel engine (the 32-bit default at these sizes) gives bit for bit what its CPU model gives."""
    d, Z, N, *_ = problem(name)
    H = jn.Hamiltonian.from_dir(d, Z, N)
    H.set_engine(4)
    H.set_precision(bits)
    x = np.random.default_rng(23).standard_normal(H.dimension)
    got = H.matvec(x)
    want = emu4(d, Z, N, x, bits == 32)
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
    ref = oracle.Port(d).matvec(x)
    tol = 1e-12 if bits == 64 else 2e-6
    assert np.abs(got - ref).max() <= tol * np.abs(ref).max()
    H.close()


@pytest.mark.gpu
def test_panel_engine_rounds_ties_to_even(problem):
    """x whose 32-bit fixed-point values fall exactly halfway between integers
    (max|x| = 1 gives the scale 2^29, x = (k + 1/2) 2^-29), plus subnormals,
    signed zeros and values that round to zero: the device conversion rounds
    half to even as the CPU model's llrint does, bit for bit."""
    d, Z, N, *_ = problem("he4_n4_2b")
    H = jn.Hamiltonian.from_dir(d, Z, N)
    H.set_engine(4)
    H.set_precision(32)
    rng = np.random.default_rng(29)
    k = rng.integers(-(1 << 28), 1 << 28, H.dimension)
    x = (k + 0.5) * 2.0 ** -29
    x[::7] = k[::7] * 2.0 ** -29                     # exact integers at the scale
    x[1::11] = rng.standard_normal(len(x[1::11])) * 1e-12   # round to zero or to +-1
    x[2::13] = 5e-324                                # subnormal
    x[3::17] = -0.0
    x[0] = 1.0
    got = H.matvec(x)
    want = emu4(d, Z, N, x, True)
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
    H.close()


def test_empty_lists_on_every_engine(problem, tmp_path):
    """Index lists with no entries (0-byte files) contribute nothing: every
    engine at both precisions matches the oracle on the same files."""
    import shutil
    d0, Z, N, *_ = problem("he4_n2_3b")
    d = str(tmp_path / "empty")
    shutil.copytree(d0, d)
    names = sorted(os.listdir(f"{d}/index_lists"), key=lambda s: int(s.split("_")[-1]))
    for n in names[:3] + names[-2:]:
        open(f"{d}/index_lists/{n}", "wb").close()
    port = oracle.Port(d)
    x = np.random.default_rng(5).standard_normal(port.dimension)
    want = port.matvec(x)
    port.close()
    scale = np.abs(want).max()
    H = jn.Hamiltonian.from_dir(d, Z, N)
    try:
        for engine in (3, 4, 5):
            H.set_engine(engine)
            for bits, tol in ((64, 1e-12), (32, 2e-6)):
                H.set_precision(bits)
                got = H.matvec(x)
                assert np.abs(got - want).max() <= tol * scale, (engine, bits)
    finally:
        H.close()


def test_out_of_range_x_is_refused_and_scaling_is_exact(problem):
    """The fixed-point products refuse an x outside their range instead of
    returning a wrong result (engine 2 at precision 64, plain FP64 sums,
    takes it and matches the oracle); x = 0 gives exact zeros; and inside the
    range, scaling x by 2^60 scales y by 2^60 bit for bit."""
    d, Z, N, *_ = problem("he4_n2_3b")
    port = oracle.Port(d)
    H = jn.Hamiltonian.from_dir(d, Z, N)
    D = H.dimension
    huge, tiny = np.full(D, 1e300), np.full(D, 5e-324)
    x = np.random.default_rng(9).standard_normal(D)
    try:
        for engine in (3, 4, 5):
            H.set_engine(engine)
            for bits in (64, 32):
                H.set_precision(bits)
                assert np.array_equal(H.matvec(np.zeros(D)), np.zeros(D)), (engine, bits)
                for bad in (huge, tiny):
                    with pytest.raises(jn.JnError):
                        H.matvec(bad)
                a, b = H.matvec(x), H.matvec(x * 2.0 ** 60)
                assert np.array_equal(b, a * 2.0 ** 60), (engine, bits)
        H.set_engine(2)
        H.set_precision(64)
        want = port.matvec(huge)
        assert np.abs(H.matvec(huge) - want).max() <= 1e-12 * np.abs(want).max()
    finally:
        H.close()
        port.close()


def test_engines_agree(problem):
    d, Z, N, *_ = problem("he4_n6_3b")
    H = jn.Hamiltonian.from_dir(d, Z, N)
    x = np.random.default_rng(22).standard_normal(H.dimension)
    ys = []
    for engine in (2, 3, 4):
        H.set_engine(engine)
        ys.append(H.matvec(x))
    for y in ys[1:]:
        assert np.abs(y - ys[0]).max() <= 1e-12 * np.abs(ys[0]).max()
    H.close()


def test_panel_engine_after_new_matrix_elements(problem):
    """Replacing the matrix elements rebuilds the panel coefficients."""
    d, Z, N, *_ = problem("he4_n4_2b")
    H = jn.Hamiltonian.from_dir(d, Z, N)
    H.set_engine(4)
    x = np.random.default_rng(24).standard_normal(H.dimension)
    a = H.matvec(x)
    me = H.read_matrix_elements(os.path.join(d, "matrix_elements"))
    H.set_matrix_elements(2.5 * me)
    b = H.matvec(x)
    assert np.abs(b - 2.5 * a).max() <= 1e-12 * np.abs(b).max()
    H.close()


@pytest.mark.parametrize("bits", [32, 64])
def test_panel_schedules_do_not_change_a_bit(problem, bits):
    """Every panel schedule (rows per lane, CTAs per SM) gives the same bits, and
    the autotuner installs one of them without changing the product."""
    d, Z, N, *_ = problem("he4_n6_3b")
    H = jn.Hamiltonian.from_dir(d, Z, N)
    H.set_engine(4)                 # at both precisions
    other = 64 if bits == 32 else 32
    x = np.random.default_rng(25).standard_normal(H.dimension)
    H.set_precision(other)
    want_other = H.matvec(x)
    H.set_precision(bits)
    want = H.matvec(x)
    for rows, per in ((8, 1), (64, 2), (128, 3)):
        H.set_panel_schedule(rows, per)
        assert np.array_equal(H.matvec(x).view(np.uint64), want.view(np.uint64))
    t = H.autotune(trials=3)
    assert t["engine"] == 4 and t["candidates"] >= 5 and t["ms"] > 0
    assert np.array_equal(H.matvec(x).view(np.uint64), want.view(np.uint64))
    # the other precision was tuned too: switching installs its schedule, and back
    H.set_precision(other)
    assert np.array_equal(H.matvec(x).view(np.uint64), want_other.view(np.uint64))
    H.set_precision(bits)
    assert np.array_equal(H.matvec(x).view(np.uint64), want.view(np.uint64))
    with pytest.raises(jn.JnError):
        H.set_panel_schedule(0, 1)
    with pytest.raises(jn.JnError):
        H.set_panel_schedule(32, 99)
    # the context still works after a rejected schedule
    assert np.array_equal(H.matvec(x).view(np.uint64), want.view(np.uint64))
    H.close()


def test_autotune_may_choose_the_engine(problem):
    d, Z, N, *_ = problem("he4_n4_2b")
    H = jn.Hamiltonian.from_dir(d, Z, N)
    x = np.random.default_rng(26).standard_normal(H.dimension)
    t = H.autotune(trials=3, tune_engine=True)
    assert t["engine"] in (3, 4, 5) and H.active_engine() == t["engine"]
    ref = oracle.Port(d).matvec(x)
    assert np.abs(H.matvec(x) - ref).max() <= 1e-12 * np.abs(ref).max()
    H.close()


def test_mars_order_gives_the_same_product_bits(problem, tmp_path):
    """The evaluation order jn_mars writes gives the panel engine's product bit for bit."""
    d, Z, N, *_ = problem("he4_n6_3b")
    order = str(tmp_path / "order.txt")
    jn.mars(f"{d}/comb.txt", Z, N, order)
    a = jn.Hamiltonian.from_dir(d, Z, N)
    b = jn.Hamiltonian(comb=f"{d}/comb.txt", order=order, lists=f"{d}/index_lists", mes=f"{d}/matrix_elements",
                       Z=Z, N=N)
    a.set_engine(4)
    b.set_engine(4)
    x = np.random.default_rng(27).standard_normal(a.dimension)
    for bits in (32, 64):
        a.set_precision(bits)
        b.set_precision(bits)
        assert np.array_equal(a.matvec(x).view(np.uint64), b.matvec(x).view(np.uint64))
    a.close()
    b.close()


def test_subspace_matrices_and_ceres_files(problem, tmp_path):
    """Norm and projected-operator matrices of training vectors (the Ceres
    analogue) against the dense oracle, in memory and through .npy files."""
    d, Z, N, *_ = problem("he4_n4_2b")
    H = jn.Hamiltonian.from_dir(d, Z, N)
    Hd = np.array([oracle.Port(d).matvec(e) for e in np.eye(H.dimension)]).T
    rng = np.random.default_rng(28)
    V = rng.standard_normal((5, H.dimension))
    Nm, Om = H.subspace_matrices(list(V))
    assert np.abs(Nm - V @ V.T).max() <= 1e-12 * np.abs(V @ V.T).max()
    want = V @ Hd @ V.T
    assert np.abs(Om - want).max() <= 1e-12 * np.abs(want).max()
    assert np.array_equal(Om, Om.T) and np.array_equal(Nm, Nm.T)
    dirs = []
    for i, v in enumerate(V):
        vd = tmp_path / f"v{i}"
        vd.mkdir()
        for bid, off, n in H.blocks():
            v[off:off + n].tofile(str(vd / f"vec_{bid}"))
        dirs.append(str(vd))
    H.ceres_files(dirs, str(tmp_path / "norm.npy"), str(tmp_path / "op.npy"))
    assert np.array_equal(np.load(str(tmp_path / "norm.npy")), Nm)
    assert np.array_equal(np.load(str(tmp_path / "op.npy")), Om)
    H.close()
