"""Generator: determinism, bit-exact index lists against the Python
restatement, and the Hamiltonian it encodes against the dense oracle."""
import filecmp
import hashlib
import os

import numpy as np
import pytest

import jupiterncsm_gb300 as jn
import oracle
from oracle import dense_h, index_lists


def tree_digest(d):
    h = hashlib.sha256()
    for sub in ("comb.txt", "evaluation_order.txt"):
        h.update(open(os.path.join(d, sub), "rb").read())
    for sub in ("index_lists", "matrix_elements"):
        for f in sorted(os.listdir(os.path.join(d, sub))):
            h.update(f.encode())
            h.update(open(os.path.join(d, sub, f), "rb").read())
    return h.hexdigest()


def test_two_runs_are_bit_identical(tmp_path):
    a, b = str(tmp_path / "a"), str(tmp_path / "b")
    jn.generate(a, nmax=4, nbody=3)
    jn.generate(b, nmax=4, nbody=3)
    assert tree_digest(a) == tree_digest(b)


def test_files_do_not_depend_on_the_host_thread_count(tmp_path, monkeypatch):
    """The matrix-element blocks are written by all host cores; one thread
    (JN_HOST_THREADS=1) writes the same files."""
    a, b = str(tmp_path / "a"), str(tmp_path / "b")
    monkeypatch.setenv("JN_HOST_THREADS", "1")
    jn.generate(a, nmax=4, nbody=3)
    monkeypatch.delenv("JN_HOST_THREADS")
    jn.generate(b, nmax=4, nbody=3)
    assert tree_digest(a) == tree_digest(b)


@pytest.mark.parametrize("name", ["he4_n2_2b", "he4_n2_3b", "li6_n2_3b"])
def test_index_lists_bit_exact_against_restatement(problem, name):
    d, Z, N, nmax, nbody = problem(name)
    B = index_lists.Builder(Z, N, nmax)
    specs = index_lists.conn_lists(f"{d}/comb.txt")
    assert specs
    for s in specs:
        want = B.build(s)
        got = open(f"{d}/index_lists/index_list_{s['id']}", "rb").read()
        assert got == want, f"index list {s['id']} ({s}) differs"
        assert len(got) == 12 * s["length"]


def test_index_lists_he4_nmax4_bit_exact(problem):
    d, Z, N, nmax, nbody = problem("he4_n4_2b")
    B = index_lists.Builder(Z, N, nmax)
    for s in index_lists.conn_lists(f"{d}/comb.txt"):
        assert open(f"{d}/index_lists/index_list_{s['id']}", "rb").read() == B.build(s)


def test_matrix_element_headers(problem):
    d, *_ = problem("he4_n2_3b")
    for f in os.listdir(f"{d}/matrix_elements"):
        raw = open(f"{d}/matrix_elements/{f}", "rb").read()
        nd_n, nd_p = np.frombuffer(raw[:16], dtype=np.uint64)
        n = nd_p if nd_n == 0 else nd_n if nd_p == 0 else nd_n * nd_p
        assert len(raw) == 16 + 8 * int(n)


def test_pair_normal_matches_restatement():
    G = jn.gen_lib()
    for (s, t, a, b) in [(1, 2, 3, 4), (20261203, 5, 17, 9), (7, 9, 123456789, 42)]:
        assert G.jn_gen_pair_normal(s, t, a, b) == dense_h.pair_normal(s, t, a, b)
        assert G.jn_gen_pair_normal(s, t, a, b) == G.jn_gen_pair_normal(s, t, b, a)


def dense_from_port(d):
    p = oracle.Port(d)
    D = p.dimension
    H = np.zeros((D, D))
    for j in range(D):
        e = np.zeros(D)
        e[j] = 1.0
        H[:, j] = p.matvec(e)
    p.close()
    return H


@pytest.mark.parametrize("name", ["he4_n2_2b", "he4_n2_3b", "li6_n2_3b"])
def test_encoded_hamiltonian_equals_dense_oracle(problem, name):
    d, Z, N, nmax, nbody = problem(name)
    H = dense_from_port(d)
    Hd = dense_h.build_dense_h(d, Z, N, nmax, nbody=nbody)
    assert np.abs(H - H.T).max() < 1e-12
    assert np.abs(H - Hd).max() <= 1e-12 * np.abs(Hd).max()


def test_me_only_mode_rewrites_only_matrix_elements(tmp_path):
    d = str(tmp_path / "p")
    jn.generate(d, nmax=2)
    before = open(f"{d}/comb.txt").read()
    jn.generate(d, nmax=2, seed=99, hbar_omega=0.0, me_only_subdir="me_op1")
    assert open(f"{d}/comb.txt").read() == before
    assert sorted(os.listdir(f"{d}/me_op1")) == sorted(os.listdir(f"{d}/matrix_elements"))
