"""The oracle itself: the plain-C port pinned against the compiled reference
and against the golden fixtures written from the reference."""
import hashlib
import json
import os

import numpy as np
import pytest

import jupiterncsm_gb300 as jn
import oracle
from tests.conftest import reference_tree_present

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CASES = ["he4_n2_2b", "he4_n2_3b", "li6_n2_3b"]


@pytest.mark.parametrize("name", CASES)
def test_golden_files_and_port(tmp_path, name):
    """The generator reproduces the fixture's files and the port reproduces the
    reference's y = H x stored in the fixture."""
    meta = json.load(open(os.path.join(GOLDEN, f"{name}.json")))
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    d = str(tmp_path / name)
    jn.generate(d, basis_files=False, **meta["config"])
    h = hashlib.sha256()
    names = sorted(os.listdir(f"{d}/index_lists"))
    for f in names:
        h.update(f.encode())
        h.update(open(f"{d}/index_lists/{f}", "rb").read())
    assert h.hexdigest() == meta["files"]["index_lists"]
    assert len(names) == meta["files"]["index_lists_count"]
    p = oracle.Port(d)
    assert p.dimension == meta["dimension"]
    y = p.matvec(g["x"])
    assert np.abs(y - g["y"]).max() <= 1e-12 * np.abs(g["y"]).max()
    p.close()


@pytest.mark.skipif(not reference_tree_present(), reason="reference tree absent")
@pytest.mark.parametrize("name", ["he4_n2_3b", "he4_n4_2b", "li6_n2_3b", "he4_n6_3b", "li6_n6_3b"])
def test_port_pinned_to_reference(problem, name):
    """The port against the compiled reference kernels, up to the largest
    single-GPU problem (6Li Nmax 6, two- plus three-body, D = 186 894)."""
    d, Z, N, *_ = problem(name)
    threads = os.cpu_count() or 4
    ref = oracle.Reference(d, Z, N, threads=threads)
    p = oracle.Port(d)
    rng = np.random.default_rng(5)
    for _ in range(1 if name == "li6_n6_3b" else 3):
        x = rng.standard_normal(p.dimension)
        y0 = rng.standard_normal(p.dimension)
        a = ref.matvec(x, y0.copy())
        b = p.matvec(x, y0.copy())
        c = y0.copy()
        p.matvec_omp(x, c, threads)
        scale = np.abs(a).max()
        assert np.abs(a - b).max() <= 1e-12 * scale
        assert np.abs(a - c).max() <= 1e-12 * scale
    ref.close()
    p.close()


@pytest.mark.skipif(not reference_tree_present(), reason="reference tree absent")
def test_reference_file_level_scheduler_matches_port(problem, tmp_path):
    """run_matrix_vector_multiplication as shipped (files in, files out)."""
    d, Z, N, *_ = problem("he4_n2_3b")
    blocks = oracle.read_blocks(d)
    D = sum(a * b for _, a, b in blocks)
    rng = np.random.default_rng(9)
    x, y0 = rng.standard_normal(D), rng.standard_normal(D)
    oracle.write_vector_dir(str(tmp_path / "in"), blocks, x)
    oracle.write_vector_dir(str(tmp_path / "out"), blocks, y0)
    ref = oracle.Reference(d, Z, N, threads=2)
    ref.matvec_files(str(tmp_path / "out"), str(tmp_path / "in"), threads=2)
    got = oracle.read_vector_dir(str(tmp_path / "out"), blocks)
    want = oracle.Port(d).matvec(x, y0.copy())
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()


def test_golden_eigenvalues_from_port(tmp_path):
    meta = json.load(open(os.path.join(GOLDEN, "he4_n2_3b.json")))
    g = np.load(os.path.join(GOLDEN, "he4_n2_3b.npz"))
    d = str(tmp_path / "p")
    jn.generate(d, basis_files=False, **meta["config"])
    p = oracle.Port(d)
    D = p.dimension
    H = np.column_stack([p.matvec(np.eye(D)[j]) for j in range(D)])
    w = np.linalg.eigvalsh(0.5 * (H + H.T))[:10]
    assert np.abs(w - g["eig"]).max() < 1e-10


@pytest.mark.skipif(not reference_tree_present(), reason="reference tree absent")
@pytest.mark.parametrize("name", ["bacchus_he4_n4_2b", "bacchus_he4_n4_2b_vec", "bacchus_he4_n2_3b",
                                  "bacchus_li6_n2_3b_vec"])
def test_reference_bacchus_fixtures_and_dense_eigh(tmp_path, name):
    """The reference's Bacchus, run again, reproduces its fixture, and its
    lowest eigenpair is the dense matrix's (within its convergence tolerance)."""
    if not oracle.reference_bacchus_available():
        oracle.build()
    meta = json.load(open(os.path.join(GOLDEN, f"{name}.json")))
    d = str(tmp_path / "p")
    jn.generate(d, basis_files=False, **meta["config"])
    r = oracle.reference_bacchus(d, meta["config"]["Z"], meta["config"]["N"], **meta["lanczos"])
    assert r["num_eigenvalues"] == meta["num_eigenvalues"]
    assert np.abs(r["eigenvalues"] - meta["eigenvalues"]).max() <= 1e-10 * np.abs(r["eigenvalues"]).max()
    p = oracle.Port(d)
    D = p.dimension
    Hd = np.column_stack([p.matvec(np.eye(D)[j]) for j in range(D)])
    w, V = np.linalg.eigh(0.5 * (Hd + Hd.T))
    assert abs(r["eigenvalues"][0] - w[0]) < 1e-6
    assert abs(V[:, 0] @ r["eigenvectors"][0]) > 1 - 1e-8
