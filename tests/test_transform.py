"""The J -> M two-body transform (Mercury): host plan, CPU model, GPU kernel.

The reference's own transform (oracle/_ref/ref_mercury, compiled from the
reference sources where they exist) pins the CPU model of the kernel here,
and golden fixtures written from it (tests/golden/transform_*.npz) pin the
GPU kernel on machines without the reference tree.  Tolerances: the product
and the reference compute the same sums in the same order and differ only
in the last bits of the Clebsch-Gordan coefficients (each within 2.3e-16 of
the exact value), so matrix elements agree to 1e-12 MeV absolute; the GPU
kernel and its CPU model agree bit for bit.
"""
import ctypes
import glob
import hashlib
import json
import os
import subprocess

import numpy as np
import pytest

import jupiterncsm_gb300 as jn
import oracle
from oracle import jt_transform as jt

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
ME_TOL = 1e-12      # MeV, absolute, product vs reference


class Emu:
    """CPU model of jn_jt_to_m_kernel over the product's plan (tests/native/transform_emulator.c)."""
    lib = None

    def __init__(self, d, Z, N, e1, e2, antoine=None, kinetic=True):
        if Emu.lib is None:
            L = ctypes.CDLL(os.path.join(ROOT, "tests", "_build", "libtransform_emu.so"))
            L.temu_open.restype = ctypes.c_void_p
            L.temu_open.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_char_p, ctypes.c_int]
            L.temu_block.restype = ctypes.c_int64
            L.temu_block.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
            L.temu_ids.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
            L.temu_stats.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
            L.temu_header.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
            L.temu_close.argtypes = [ctypes.c_void_p]
            L.temu_error.restype = ctypes.c_char_p
            Emu.lib = L
        antoine = antoine or os.path.join(d, "antoine_2nf.bin")
        self.h = Emu.lib.temu_open(os.path.join(d, "comb.txt").encode(), os.path.join(d, "anicr").encode(), Z, N, e1,
                                   e2, antoine.encode(), int(kinetic))
        if not self.h:
            raise RuntimeError(Emu.lib.temu_error().decode())

    def ids(self):
        n = Emu.lib.temu_ids(self.h, None, 0)
        a = np.zeros(n, dtype=np.int32)
        Emu.lib.temu_ids(self.h, a.ctypes.data, n)
        return [int(x) for x in a]

    def block(self, bid):
        n = Emu.lib.temu_block(self.h, bid, None)
        out = np.zeros(max(n, 0))
        Emu.lib.temu_block(self.h, bid, out.ctypes.data)
        return out

    def header(self, bid):
        h = np.zeros(2, dtype=np.uint64)
        assert Emu.lib.temu_header(self.h, bid, h.ctypes.data) == 0
        return h

    def stats(self):
        v = np.zeros(6, dtype=np.int64)
        Emu.lib.temu_stats(self.h, v.ctypes.data)
        return dict(zip(["elements", "pair_states", "configurations", "two_body", "one_body", "jt_states"], v.tolist()))

    def close(self):
        Emu.lib.temu_close(self.h)


def write_blocks(emu, out):
    os.makedirs(out, exist_ok=True)
    for bid in emu.ids():
        x = emu.block(bid)
        open(os.path.join(out, f"{bid}_matrix_elements"), "wb").write(emu.header(bid).tobytes() + x.tobytes())


def reference_blocks(d, Z, N, e1, e2, tmp):
    out = os.path.join(tmp, "ref_me")
    oracle.reference_transform(os.path.join(d, "comb.txt"), os.path.join(d, "anicr"), out, Z, N, e1, e2,
                               os.path.join(d, "antoine_2nf.bin"))
    return {int(os.path.basename(f).split("_")[0]): oracle.read_me_file(f) for f in glob.glob(out + "/*_matrix_elements")}


# ---------------------------------------------------------------- host pieces

def test_clebsch_gordan_matches_exact_values():
    worst, n = 0.0, 0
    for j1 in range(1, 16, 2):
        for j2 in range(1, 16, 2):
            for j3 in range(abs(j1 - j2), j1 + j2 + 1, 2):
                for m1 in range(-j1, j1 + 1, 2):
                    m2 = j3 - m1 if abs(j3 - m1) <= j2 else None
                    for mm2 in ([m2] if m2 is not None else []) + [-j2, j2]:
                        if abs(m1 + mm2) > j3:
                            continue
                        a = jt.cg_exact(j1, j2, j3, m1, mm2, m1 + mm2)
                        b = jn.clebsch_gordan(j1, j2, j3, m1, mm2, m1 + mm2)
                        worst = max(worst, abs(a - b))
                        n += 1
    assert n > 5000
    assert worst <= 4.5e-16
    # known values and selection rules
    assert jn.clebsch_gordan(1, 1, 0, 1, -1, 0) == pytest.approx(np.sqrt(0.5), abs=1e-16)
    assert jn.clebsch_gordan(1, 1, 0, -1, 1, 0) == pytest.approx(-np.sqrt(0.5), abs=1e-16)
    assert jn.clebsch_gordan(2, 2, 4, 2, 2, 4) == pytest.approx(1.0, abs=3e-16)
    assert jn.clebsch_gordan(3, 1, 2, 1, 1, 4) == 0.0          # m1 + m2 != m3
    assert jn.clebsch_gordan(1, 1, 6, 1, 1, 2) == 0.0          # triangle


@pytest.mark.parametrize("e1,e2", [(0, 0), (2, 2), (3, 4), (5, 6), (7, 8)])
def test_coupled_basis_matches_restatement(e1, e2, tmp_path):
    """Configuration count of the product's JT basis equals the Python restatement's,
    as seen through the Antoine file the generator writes with it."""
    path = str(tmp_path / "v.bin")
    jn.write_antoine(path, e1, e2, 4, seed=3)
    states, nconf = jt.jt_basis(e1, e2)
    title, ncol, hw, nrow, data = jt.read_antoine(path)
    assert ncol == 6 and nrow == nconf and hw == pytest.approx(20.0)
    # the kinetic column holds A (e_a + e_b) / (2 (A - 1)) on diagonal configurations only
    sh = jt.antoine_shells(e1)
    row = 0
    for i, s in enumerate(states):
        k = i
        while k < len(states) and states[k][2:] == s[2:]:
            want = 4 * (sh[s[0]][0] + sh[s[1]][0]) / 6.0 if k == i else 0.0
            assert data[row, 0] == pytest.approx(want, rel=1e-6, abs=0)
            row += 1
            k += 1
    assert row == nrow
    assert np.all(data[:, 1:3] == 0)
    assert 0.8 < np.std(data[:, 3:6]) < 1.2


def test_antoine_file_is_deterministic(tmp_path):
    a, b = str(tmp_path / "a"), str(tmp_path / "b")
    jn.write_antoine(a, 3, 4, 6, seed=11)
    jn.write_antoine(b, 3, 4, 6, seed=11)
    assert open(a, "rb").read() == open(b, "rb").read()


def test_golden_inputs_regenerate_identically(jproblem):
    for name in ("he4_n2", "li6_n2"):
        d, Z, N, e1, e2 = jproblem(name)
        meta = json.load(open(os.path.join(GOLDEN, f"transform_{name}.json")))
        assert (e1, e2) == (meta["emax_single"], meta["emax_pair"])
        assert hashlib.sha256(open(os.path.join(d, "antoine_2nf.bin"), "rb").read()).hexdigest() == meta["antoine_sha256"]
        assert hashlib.sha256(open(os.path.join(d, "comb.txt"), "rb").read()).hexdigest() == meta["comb_sha256"]


@pytest.mark.parametrize("name", ["he4_n2", "li6_n2"])
def test_model_matches_golden(jproblem, name):
    d, Z, N, e1, e2 = jproblem(name)
    g = np.load(os.path.join(GOLDEN, f"transform_{name}.npz"))
    emu = Emu(d, Z, N, e1, e2)
    try:
        assert sorted(emu.ids()) == sorted(int(k[1:]) for k in g.files)
        worst = max(np.abs(emu.block(int(k[1:])) - g[k]).max(initial=0.0) for k in g.files)
        assert worst <= ME_TOL
    finally:
        emu.close()


@pytest.mark.skipif(not oracle.reference_transform_available(), reason="reference tree absent")
@pytest.mark.parametrize("name", ["he4_n2", "li6_n2", "he4_n4", "li6_n4"])
def test_model_matches_reference(jproblem, name, tmp_path):
    d, Z, N, e1, e2 = jproblem(name)
    ref = reference_blocks(d, Z, N, e1, e2, str(tmp_path))
    emu = Emu(d, Z, N, e1, e2)
    try:
        assert sorted(ref) == sorted(emu.ids())
        worst = 0.0
        for bid, (nd_n, nd_p, x) in ref.items():
            y = emu.block(bid)
            assert len(y) == len(x)
            worst = max(worst, np.abs(y - x).max(initial=0.0))
        assert worst <= ME_TOL
    finally:
        emu.close()


@pytest.mark.skipif(not oracle.reference_transform_available(), reason="reference tree absent")
def test_model_matches_reference_without_kinetic_term(jproblem, tmp_path):
    d, Z, N, e1, e2 = jproblem("he4_n2")
    out = str(tmp_path / "ref")
    oracle.reference_transform(os.path.join(d, "comb.txt"), os.path.join(d, "anicr"), out, Z, N, e1, e2,
                               os.path.join(d, "antoine_2nf.bin"), include_kinetic=False)
    emu = Emu(d, Z, N, e1, e2, kinetic=False)
    try:
        for f in glob.glob(out + "/*_matrix_elements"):
            x = oracle.read_me_file(f)[2]
            assert np.abs(emu.block(int(os.path.basename(f).split("_")[0])) - x).max(initial=0.0) <= ME_TOL
    finally:
        emu.close()


def test_transformed_interaction_is_rotationally_invariant(tmp_path):
    """Physics check independent of the reference: with the transformed
    interaction, every level of the 2M = 2 basis is a level of the 2M = 0
    basis (the many-body Hamiltonian commutes with J^2)."""
    spectra = {}
    for M2 in (0, 2):
        d = str(tmp_path / f"m{M2}")
        s = jn.generate(d, Z=2, N=2, nmax=2, M2=M2, nbody=2, antoine=True)
        emu = Emu(d, 2, 2, s["emax_single"], s["emax_pair"])
        write_blocks(emu, os.path.join(d, "matrix_elements"))
        emu.close()
        P = oracle.Port(d)
        D = P.dimension
        H = np.zeros((D, D))
        for i in range(D):
            e = np.zeros(D)
            e[i] = 1.0
            H[:, i] = P.matvec(e)
        assert np.abs(H - H.T).max() < 1e-12
        spectra[M2] = np.linalg.eigvalsh(H)
    gap = max(np.abs(spectra[0] - e).min() for e in spectra[2])
    assert gap < 1e-10
    # and the 2M = 0 basis has levels (J = 0) that 2M = 2 lacks
    assert len(spectra[0]) > len(spectra[2])


def test_kinetic_column_gives_oscillator_diagonal(tmp_path):
    """With a zero interaction the transformed blocks are hw (e_a + e_b)/(A-1) on the
    diagonal of every energy-conserving single-species block: the J -> M
    coefficients are unitary (the reference's own unitarity tests,
    src/Neptune/jt_transformation/jt_transformation.c:349-441)."""
    d = str(tmp_path / "p")
    s = jn.generate(d, Z=2, N=2, nmax=2, nbody=2, antoine=True)
    title, ncol, hw, nrow, data = jt.read_antoine(os.path.join(d, "antoine_2nf.bin"))
    zero = data.copy()
    zero[:, 3:] = 0.0
    path = os.path.join(d, "kinetic_only.bin")
    with open(path, "wb") as f:
        for rec in (title, np.array([ncol], np.int32).tobytes() + np.array([hw], np.float32).tobytes()
                    + np.array([nrow], np.int32).tobytes(), zero.astype(np.float32).tobytes()):
            f.write(np.int32(len(rec)).tobytes() + rec + np.int32(len(rec)).tobytes())
    emu = Emu(d, 2, 2, s["emax_single"], s["emax_pair"], antoine=path)
    try:
        for line in open(os.path.join(d, "comb.txt")):
            w = line.split()
            if "ARRAY:" not in line or len(w) != 9 or w[0] not in ("pp", "nn"):
                continue
            dE, dM, depth, n = int(w[1]), int(w[2]), int(w[3]), int(w[4])
            x = emu.block(int(w[8].rstrip("=")))
            pairs = np.fromfile(os.path.join(d, "anicr", f"{w[0]}_inds_index_lists", f"basis_energy_{depth}"),
                                dtype=np.int16).reshape(-1, 2)
            if dE != 0:
                assert np.abs(x).max(initial=0.0) < 1e-12
                continue
            # single-species diagonal blocks list, per annihilated pair, the created pairs of equal M:
            # the element is hw E / (A-1) when created == annihilated and 0 otherwise
            want = 20.0 * depth / 3.0
            diag = [v for v in x if abs(v) > 1e-9]
            assert len(diag) == len(pairs)
            assert np.allclose(diag, want, rtol=1e-6)
    finally:
        emu.close()


def test_open_reports_bad_inputs_before_touching_a_device(jproblem, tmp_path):
    d, Z, N, e1, e2 = jproblem("he4_n2")
    comb, lists, v = os.path.join(d, "comb.txt"), os.path.join(d, "anicr"), os.path.join(d, "antoine_2nf.bin")
    st, msg = jn.transform_status(comb, lists, Z, N, e1, e2 + 1, v)
    assert st == jn.JN_ERR_FORMAT and "configurations" in msg
    st, msg = jn.transform_status(comb, str(tmp_path / "missing"), Z, N, e1, e2, v)
    assert st == jn.JN_ERR_IO and "basis_energy" in msg
    bad = str(tmp_path / "short.bin")
    open(bad, "wb").write(open(v, "rb").read()[:-9])
    st, msg = jn.transform_status(comb, lists, Z, N, e1, e2, bad)
    assert st == jn.JN_ERR_FORMAT
    st, msg = jn.transform_status(comb, lists, 1, 0, e1, e2, v)
    assert st == jn.JN_ERR_FORMAT and "two particles" in msg


def test_mercury_cli_without_a_device(jproblem, tmp_path):
    """--no-2nf writes the one- and two-body blocks as zeros on the host (the
    reference's generate_2nf_zero_matrix_blocks); a three-body path that is not
    a J-scheme directory (the HDF5 format) is reported, and no usage error."""
    d, Z, N, e1, e2 = jproblem("he4_n2")
    out = str(tmp_path / "me")
    r = subprocess.run([jn.MERCURY_CLI, os.path.join(d, "comb.txt"), os.path.join(d, "anicr"), out, "--num-protons",
                        str(Z), "--num-neutrons", str(N), "--single-particle-energy", str(e1), "--no-2nf",
                        "--finished-blocks-file", str(tmp_path / "fin"), "three_body.h5"],
                       capture_output=True, text=True, cwd=str(tmp_path))
    assert r.returncode == 1 and "HDF5" in r.stderr
    files = os.listdir(out)
    assert files
    for f in files:
        nd_n, nd_p, x = oracle.read_me_file(os.path.join(out, f))
        assert len(x) == (nd_n * nd_p if nd_n and nd_p else nd_n + nd_p) and not x.any()
    r = subprocess.run([jn.MERCURY_CLI], capture_output=True, text=True)
    assert r.returncode == 0 and "Usage" in r.stdout


# ---------------------------------------------------------------- GPU

@pytest.mark.gpu
@pytest.mark.parametrize("name", ["he4_n2", "li6_n2", "he4_n4", "li6_n4"])
def test_gpu_transform_is_bit_identical_to_model(jproblem, name):
    d, Z, N, e1, e2 = jproblem(name)
    T = jn.Transform.from_dir(d, Z, N, e1, e2)
    emu = Emu(d, Z, N, e1, e2)
    try:
        T.run()
        for bid in emu.ids():
            assert np.array_equal(T.block(bid), emu.block(bid)), f"block {bid}"
        st = T.stats()
        assert st["num_elements"] == emu.stats()["elements"]
    finally:
        emu.close()
        T.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["he4_n2", "li6_n2"])
def test_gpu_transform_matches_reference_golden(jproblem, name, tmp_path):
    d, Z, N, e1, e2 = jproblem(name)
    g = np.load(os.path.join(GOLDEN, f"transform_{name}.npz"))
    meta = json.load(open(os.path.join(GOLDEN, f"transform_{name}.json")))
    out = str(tmp_path / "me")
    jn.transform_2nf(os.path.join(d, "comb.txt"), os.path.join(d, "anicr"), out, Z, N, e1, e2,
                     os.path.join(d, "antoine_2nf.bin"))
    files = glob.glob(out + "/*_matrix_elements")
    assert len(files) == len(g.files)
    for f in files:
        bid = os.path.basename(f).split("_")[0]
        nd_n, nd_p, x = oracle.read_me_file(f)
        assert [nd_n, nd_p] == meta["headers"][bid]
        assert np.abs(x - g["b" + bid]).max(initial=0.0) <= ME_TOL


@pytest.mark.gpu
def test_gpu_transform_feeds_the_matvec(jproblem, tmp_path):
    """Mercury -> Bacchus on one GPU: the transformed blocks written by the GPU
    are read by jn_open and the GPU product equals the oracle's product on
    the same files; the 2M=0 spectrum contains the 2M=2 one."""
    d, Z, N, e1, e2 = jproblem("he4_n4")
    jn.transform_2nf(os.path.join(d, "comb.txt"), os.path.join(d, "anicr"), os.path.join(d, "matrix_elements"), Z, N,
                     e1, e2, os.path.join(d, "antoine_2nf.bin"))
    H = jn.Hamiltonian.from_dir(d, Z, N)
    try:
        x = np.random.default_rng(5).standard_normal(H.dimension)
        y = H.matvec(x)
        want = oracle.Port(d).matvec(x)
        assert np.abs(y - want).max() <= 1e-12 * np.abs(want).max()
    finally:
        H.close()


@pytest.mark.gpu
def test_gpu_mercury_cli_writes_the_same_files(jproblem, tmp_path):
    d, Z, N, e1, e2 = jproblem("li6_n2")
    a, b = str(tmp_path / "cli"), str(tmp_path / "api")
    os.makedirs(a)
    r = subprocess.run([jn.MERCURY_CLI, os.path.join(d, "comb.txt"), os.path.join(d, "anicr"), a, "--num-protons",
                        str(Z), "--num-neutrons", str(N), "--single-particle-energy", str(e1),
                        "--two-particle-energy", str(e2), os.path.join(d, "antoine_2nf.bin")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    jn.transform_2nf(os.path.join(d, "comb.txt"), os.path.join(d, "anicr"), b, Z, N, e1, e2,
                     os.path.join(d, "antoine_2nf.bin"))
    fa, fb = sorted(os.listdir(a)), sorted(os.listdir(b))
    assert fa == fb and len(fa) > 0
    for f in fa:
        assert open(os.path.join(a, f), "rb").read() == open(os.path.join(b, f), "rb").read()
