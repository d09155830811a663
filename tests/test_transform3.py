"""The J -> M three-body transform (Mercury, three-body part): J-scheme reader,
host plan, CPU model, GPU kernel.

The reference's own three-body transform with its ASCII J-scheme reader
(oracle/_ref/ref_mercury3, compiled from the reference sources where they
exist) pins the CPU model of the kernel here, and golden fixtures written
from it (tests/golden/transform3_*.npz) pin the GPU kernel on machines
without the reference tree.  Tolerances: the product and the reference
compute the same sums in the same order and differ only in the last bits of
the Clebsch-Gordan coefficients, so matrix elements agree to 1e-12 MeV
absolute (observed: below 2e-16); the GPU kernel and its CPU model agree bit
for bit.
"""
import ctypes
import glob
import hashlib
import json
import os
import shutil

import numpy as np
import pytest

import jupiterncsm_gb300 as jn
import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
ME_TOL = 1e-12      # MeV, absolute, product vs reference
CASES = ["transform3_he4_n2", "transform3_li6_n0"]


class Emu3:
    """CPU model of jn_jjj_to_m_kernel over the product's plan (tests/native/transform3_emulator.c)."""
    lib = None

    def __init__(self, d, Z, N, e, jdir=None):
        if Emu3.lib is None:
            L = ctypes.CDLL(os.path.join(ROOT, "tests", "_build", "libtransform3_emu.so"))
            L.t3emu_open.restype = ctypes.c_void_p
            L.t3emu_open.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_char_p]
            L.t3emu_block.restype = ctypes.c_int64
            L.t3emu_block.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
            L.t3emu_ids.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
            L.t3emu_stats.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
            L.t3emu_close.argtypes = [ctypes.c_void_p]
            L.t3emu_error.restype = ctypes.c_char_p
            L.t3emu_check_shared.restype = ctypes.c_int64
            L.t3emu_check_shared.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
            Emu3.lib = L
        jdir = jdir or os.path.join(d, "jjj")
        self.h = Emu3.lib.t3emu_open(os.path.join(d, "comb.txt").encode(), os.path.join(d, "anicr").encode(), Z, N, e,
                                     jdir.encode())
        if not self.h:
            raise RuntimeError(Emu3.lib.t3emu_error().decode())

    def ids(self):
        n = Emu3.lib.t3emu_ids(self.h, None, 0)
        a = np.zeros(n, dtype=np.int32)
        Emu3.lib.t3emu_ids(self.h, a.ctypes.data, n)
        return [int(x) for x in a]

    def block(self, bid):
        n = Emu3.lib.t3emu_block(self.h, bid, None)
        out = np.zeros(max(n, 0))
        Emu3.lib.t3emu_block(self.h, bid, out.ctypes.data)
        return out

    def stats(self):
        v = np.zeros(8, dtype=np.int64)
        Emu3.lib.t3emu_stats(self.h, v.ctypes.data)
        return dict(zip(["elements", "states", "terms", "coupled", "file_states", "file_elements", "v_entries",
                         "energy_blocks"], v.tolist()))

    def check_shared(self):
        """(elements that differ, {pairs, segments, inner sums}) of the shared-inner-sum arithmetic."""
        v = np.zeros(3, dtype=np.int64)
        bad = Emu3.lib.t3emu_check_shared(self.h, v.ctypes.data)
        return int(bad), dict(zip(["pairs", "segments", "inner_sums"], v.tolist()))

    def close(self):
        Emu3.lib.t3emu_close(self.h)


def make_case(d, Z, N, nmax, M2):
    s = jn.generate(d, Z=Z, N=N, nmax=nmax, M2=M2, nbody=3, antoine=True)
    e3 = jn.three_body_energy(os.path.join(d, "comb.txt"))
    jn.write_jjj(os.path.join(d, "jjj"), s["emax_single"], e3)
    return s["emax_single"], e3


def reference_blocks(d, Z, N, e, tmp, jdir=None):
    out = os.path.join(tmp, "ref_me3")
    oracle.reference_transform3(os.path.join(d, "comb.txt"), os.path.join(d, "anicr"), out, Z, N, e,
                                jdir or os.path.join(d, "jjj"))
    return {int(os.path.basename(f).split("_")[0]): oracle.read_me_file(f) for f in glob.glob(out + "/*_matrix_elements")}


def sha(path):
    return hashlib.sha256(open(path, "rb").read()).hexdigest()


@pytest.fixture(scope="module")
def j3problem(tmp_path_factory):
    """The golden cases' inputs, regenerated: name -> (dir, metadata)."""
    out = {}
    for name in CASES:
        meta = json.load(open(os.path.join(GOLDEN, name + ".json")))
        c = meta["case"]
        d = str(tmp_path_factory.mktemp(name))
        make_case(d, c["Z"], c["N"], c["nmax"], c["M2"])
        out[name] = (d, meta)
    return out


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


# ---------------------------------------------------------------- inputs

def test_golden_inputs_regenerate_identically(j3problem):
    for name, (d, meta) in j3problem.items():
        assert sha(os.path.join(d, "comb.txt")) == meta["comb_sha256"]
        assert sha(os.path.join(d, "jjj", "jjj.cnf")) == meta["cnf_sha256"]
        assert sha(os.path.join(d, "jjj", "jjj.mat")) == meta["mat_sha256"]
        assert jn.three_body_energy(os.path.join(d, "comb.txt")) == meta["emax_triple"]


def test_jjj_file_is_symmetric_and_complete_per_channel(j3problem):
    d, meta = j3problem["transform3_he4_n2"]
    rows = [r.split() for r in open(os.path.join(d, "jjj", "jjj.mat")) if not r.startswith("---")]
    vals = {(int(b), int(k)): float(e) for b, k, e in rows}
    assert len(vals) == len(rows)                       # every ordered pair once
    assert all(vals[(k, b)] == v for (b, k), v in vals.items())
    assert 0.05 < np.std(list(vals.values())) < 0.2    # N(0, 0.1^2)
    # the .cnf: shells in the file's own order, then jjj-coupled states with the reader's heading
    text = open(os.path.join(d, "jjj", "jjj.cnf")).read()
    assert text.startswith("---single-particle-states---\n")
    assert "---three-particle-states---\n---i---a---b---c---Jab-Jabc---\n" in text


# ---------------------------------------------------------------- CPU model

@pytest.mark.parametrize("name", CASES)
def test_model_matches_golden(j3problem, name):
    d, meta = j3problem[name]
    c = meta["case"]
    g = golden(name)
    emu = Emu3(d, c["Z"], c["N"], meta["emax_single"])
    try:
        assert sorted(emu.ids()) == sorted(int(k[1:]) for k in g.files)
        worst = 0.0
        for k in g.files:
            x = emu.block(int(k[1:]))
            assert len(x) == len(g[k])
            worst = max(worst, np.abs(x - g[k]).max(initial=0.0))
        assert worst <= ME_TOL
        st = emu.stats()
        assert st["elements"] == meta["num_elements"]
    finally:
        emu.close()


@pytest.mark.parametrize("Z,N,nmax,M2", [(2, 2, 4, 0), (3, 4, 2, 1), (1, 2, 2, 1)])
def test_shared_inner_sums_are_bit_identical(Z, N, nmax, M2, tmp_path):
    """The GPU's two launches (inner sums V s_ket once per (energy block, ket)
    pair and slot, then each element from them) give every element bit for bit
    as summing each inner sum on the spot: He4 Nmax 4, Li7 Nmax 2, H3 Nmax 2."""
    d = str(tmp_path / "p")
    e, _ = make_case(d, Z, N, nmax, M2)
    emu = Emu3(d, Z, N, e)
    try:
        bad, st = emu.check_shared()
        assert bad == 0
        assert st["pairs"] > 0 and st["segments"] >= st["pairs"] and st["inner_sums"] > 0
    finally:
        emu.close()


@pytest.mark.skipif(not oracle.reference_transform3_available(), reason="needs the reference tree (oracle/_ref)")
@pytest.mark.parametrize("Z,N,nmax,M2", [(2, 2, 4, 0), (3, 4, 2, 1), (1, 2, 2, 1)])
def test_model_matches_reference(Z, N, nmax, M2, tmp_path):
    """He4 Nmax 4 (pp n / p nn blocks), Li7 Nmax 2 (ppp, nnn and mixed,
    Z != N), H3 Nmax 2: every three-body block against the reference."""
    d = str(tmp_path / "p")
    e, _ = make_case(d, Z, N, nmax, M2)
    ref = reference_blocks(d, Z, N, e, str(tmp_path))
    emu = Emu3(d, Z, N, e)
    try:
        assert sorted(ref) == sorted(emu.ids())
        worst, n = 0.0, 0
        for bid, (nd_n, nd_p, x) in ref.items():
            y = emu.block(bid)
            assert len(y) == len(x)
            worst = max(worst, np.abs(x - y).max(initial=0.0))
            n += len(x)
        assert n > 1000 and worst <= ME_TOL
    finally:
        emu.close()


@pytest.mark.skipif(not oracle.reference_transform3_available(), reason="needs the reference tree (oracle/_ref)")
def test_reader_overwrites_and_mirrors_as_the_reference(j3problem, tmp_path):
    """Rows repeated with new values (the last one wins), rows whose states the
    file orders against the manager's shells (phase -1), blank and comment
    rows: the model and the reference read the same matrix."""
    d, meta = j3problem["transform3_he4_n2"]
    c = meta["case"]
    jdir = str(tmp_path / "jjj")
    shutil.copytree(os.path.join(d, "jjj"), jdir)
    rows = [r.split() for r in open(os.path.join(jdir, "jjj.mat")) if not r.startswith("---")]
    rng = np.random.default_rng(5)
    with open(os.path.join(jdir, "jjj.mat"), "a") as f:
        f.write("--- overrides\n")
        for i in rng.choice(len(rows), 200, replace=False):
            b, k, _ = rows[i]
            f.write(f"{b} {k} {rng.normal():.17g}\n")     # asymmetric: bra <-> ket no longer mirror
        f.write("\n# a comment row the reader skips\n")
    ref = reference_blocks(d, c["Z"], c["N"], meta["emax_single"], str(tmp_path), jdir)
    emu = Emu3(d, c["Z"], c["N"], meta["emax_single"], jdir)
    base = golden("transform3_he4_n2")
    try:
        changed = 0
        for bid, (_, _, x) in ref.items():
            y = emu.block(bid)
            assert np.abs(x - y).max(initial=0.0) <= ME_TOL
            changed += int(np.abs(x - base[f"b{bid}"]).max(initial=0.0) > 1e-9)
        assert changed > 0
    finally:
        emu.close()


def test_bad_inputs_are_reported_before_touching_a_device(j3problem, tmp_path):
    d, meta = j3problem["transform3_he4_n2"]
    c, e = meta["case"], meta["emax_single"]
    comb, lists = os.path.join(d, "comb.txt"), os.path.join(d, "anicr")

    def status(jdir, emax=e):
        return jn.transform3_status(comb, lists, c["Z"], c["N"], emax, jdir)

    st, msg = status(str(tmp_path / "absent"))
    assert st == jn.JN_ERR_IO and "J-scheme directory" in msg
    # a state index past the file's states
    bad = tmp_path / "bad_index"
    shutil.copytree(os.path.join(d, "jjj"), bad)
    with open(bad / "jjj.mat", "a") as f:
        f.write("999999 0 1.0\n")
    st, msg = status(str(bad))
    assert st == jn.JN_ERR_FORMAT and "names state" in msg
    # a row with two numbers
    bad = tmp_path / "short_row"
    shutil.copytree(os.path.join(d, "jjj"), bad)
    with open(bad / "jjj.mat", "a") as f:
        f.write("3 4\n")
    st, msg = status(str(bad))
    assert st == jn.JN_ERR_FORMAT and "incomplete row" in msg
    # JT-coupled three-particle states: not a jjj file
    bad = tmp_path / "jt"
    shutil.copytree(os.path.join(d, "jjj"), bad)
    txt = open(bad / "jjj.cnf").read().replace("---i---a---b---c---Jab-Jabc---", "---i---a---b---c---Jab-Jabc-Tab-Tabc---")
    open(bad / "jjj.cnf", "w").write(txt)
    st, msg = status(str(bad))
    assert st == jn.JN_ERR_FORMAT and "not jjj-coupled" in msg
    # two .cnf files
    bad = tmp_path / "two"
    shutil.copytree(os.path.join(d, "jjj"), bad)
    shutil.copy(bad / "jjj.cnf", bad / "other.cnf")
    st, msg = status(str(bad))
    assert st == jn.JN_ERR_FORMAT and "one .cnf and one .mat" in msg
    # shells above the manager's single-particle energy limit
    st, msg = status(os.path.join(d, "jjj"), emax=e - 1)
    assert st == jn.JN_ERR_FORMAT and "beyond the single-particle energy limit" in msg


# ---------------------------------------------------------------- GPU kernel

@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_kernel_matches_model_and_golden(j3problem, name):
    d, meta = j3problem[name]
    c = meta["case"]
    g = golden(name)
    T = jn.Transform3.from_dir(d, c["Z"], c["N"], meta["emax_single"])
    emu = Emu3(d, c["Z"], c["N"], meta["emax_single"])
    try:
        T.run()
        for k in g.files:
            x = T.block(int(k[1:]))
            y = emu.block(int(k[1:]))
            assert np.array_equal(x, y)                            # bit for bit with the CPU model
            assert np.abs(x - g[k]).max(initial=0.0) <= ME_TOL     # the reference's values
        st = T.stats()
        assert st["num_elements"] == meta["num_elements"] and st["num_three_body_blocks"] == meta["num_blocks"]
        assert st["algorithmic_bytes"] > 8 * st["num_elements"]
    finally:
        T.close()
        emu.close()


@pytest.mark.gpu
def test_kernel_matches_model_on_a_larger_problem(tmp_path):
    """He4 Nmax 4: about 7e5 three-body elements, bit for bit with the CPU model."""
    d = str(tmp_path / "he4n4")
    e, _ = make_case(d, 2, 2, 4, 0)
    T = jn.Transform3.from_dir(d, 2, 2, e)
    emu = Emu3(d, 2, 2, e)
    try:
        T.run()
        n = 0
        for bid in emu.ids():
            x, y = T.block(bid), emu.block(bid)
            assert np.array_equal(x, y)
            n += len(x)
        assert n > 500_000
        assert T.profile() > 0
    finally:
        T.close()
        emu.close()


@pytest.mark.gpu
def test_written_blocks_feed_the_product(j3problem, tmp_path):
    """jn_transform_2nf + jn_transform_3nf write every one-, two- and three-body
    block in the reference's format; the GPU product on them matches the
    oracle's restatement of the reference kernels on the same files."""
    d, meta = j3problem["transform3_he4_n2"]
    c = meta["case"]
    g = golden("transform3_he4_n2")
    p = str(tmp_path / "p")
    shutil.copytree(d, p)
    mes = os.path.join(p, "matrix_elements")
    shutil.rmtree(mes)
    s = jn.generate(str(tmp_path / "again"), Z=c["Z"], N=c["N"], nmax=c["nmax"], M2=c["M2"], nbody=3, antoine=True)
    jn.transform_2nf(os.path.join(p, "comb.txt"), os.path.join(p, "anicr"), mes, c["Z"], c["N"], s["emax_single"],
                     s["emax_pair"], os.path.join(p, "antoine_2nf.bin"))
    jn.transform_3nf(os.path.join(p, "comb.txt"), os.path.join(p, "anicr"), mes, c["Z"], c["N"], meta["emax_single"],
                     os.path.join(p, "jjj"))
    for bid, hdr in meta["headers"].items():
        nd_n, nd_p, x = oracle.read_me_file(os.path.join(mes, f"{bid}_matrix_elements"))
        assert [nd_n, nd_p] == hdr
        assert np.abs(x - g[f"b{bid}"]).max(initial=0.0) <= ME_TOL
    H = jn.Hamiltonian.from_dir(p, c["Z"], c["N"])
    try:
        x = np.random.default_rng(3).standard_normal(H.dimension)
        y = H.matvec(x)
        want = oracle.Port(p).matvec(x)
        assert np.abs(y - want).max() / np.abs(want).max() <= 1e-12
    finally:
        H.close()


@pytest.mark.gpu
def test_mercury_program_writes_all_blocks_and_resumes(j3problem, tmp_path):
    """jn_mercury with the reference's command line: one-body zeros, the
    two-body transform, the three-body transform; a second run with the same
    finished-blocks file skips every energy block; --no-2nf writes the
    one- and two-body blocks as zeros and takes the only path as three-body."""
    import subprocess
    d, meta = j3problem["transform3_he4_n2"]
    c = meta["case"]
    g = golden("transform3_he4_n2")
    exe = os.path.join(ROOT, "jupiterncsm_gb300", "lib", "jn_mercury")
    s = json.load(open(os.path.join(GOLDEN, "transform_he4_n2.json")))
    out = str(tmp_path / "me")
    fin = str(tmp_path / "finished")
    args = [exe, os.path.join(d, "comb.txt"), os.path.join(d, "anicr"), out, "--num-protons", str(c["Z"]),
            "--num-neutrons", str(c["N"]), "--single-particle-energy", str(meta["emax_single"]),
            "--two-particle-energy", str(s["emax_pair"]), "--finished-blocks-file", fin, "--LEC-CE", "0.5"]
    r = subprocess.run(args + [os.path.join(d, "antoine_2nf.bin"), os.path.join(d, "jjj")], capture_output=True,
                       text=True, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    for k in g.files:
        _, _, x = oracle.read_me_file(os.path.join(out, f"{k[1:]}_matrix_elements"))
        assert np.abs(x - g[k]).max(initial=0.0) <= ME_TOL
    nfin = os.path.getsize(fin) // 8
    assert nfin > 0 and sorted(np.fromfile(fin, dtype=np.uint64).tolist()) == list(range(nfin))
    # resume: every energy block is finished, so nothing three-body is written again
    victim = os.path.join(out, f"{g.files[0][1:]}_matrix_elements")
    os.remove(victim)
    r = subprocess.run(args + [os.path.join(d, "antoine_2nf.bin"), os.path.join(d, "jjj")], capture_output=True,
                       text=True, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    assert not os.path.exists(victim)
    assert os.path.getsize(fin) // 8 == nfin
    # --no-2nf: the only interaction path is the three-body one
    out2 = str(tmp_path / "me2")
    args2 = [out2 if a == out else fin + "2" if a == fin else a for a in args]
    r = subprocess.run(args2 + ["--no-2nf", os.path.join(d, "jjj")], capture_output=True, text=True,
                       cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr
    for k in g.files:
        _, _, x = oracle.read_me_file(os.path.join(out2, f"{k[1:]}_matrix_elements"))
        assert np.abs(x - g[k]).max(initial=0.0) <= ME_TOL
    two = [f for f in os.listdir(out2) if f"b{f.split('_')[0]}" not in g.files]
    assert two and all(not oracle.read_me_file(os.path.join(out2, f))[2].any() for f in two)
