"""Batched Lanczos over several bases in one solve (jn_lanczos_batch_bases):
instances H(c) = H0 + c H1 on three bases, every step one graph with one
product launch for all of them, checked against dense FP64 eigenvalues of
the oracle's matrices.

Tolerance: 1e-6 MeV on the ten lowest eigenvalues, the target of the
benchmark's solves.
"""
import os

import numpy as np
import pytest

import jupiterncsm_gb300 as jn
import oracle

pytestmark = pytest.mark.gpu
EIG_TOL = 1e-6
# name -> (Z, N, Nmax, nbody, 2M)
BASES = {"he4_n2_2b": (2, 2, 2, 2, 0), "he4_n4_2b": (2, 2, 4, 2, 0), "li6_n2_3b": (3, 3, 2, 3, 2)}
CS = {"he4_n2_2b": (0.0, -0.7), "he4_n4_2b": (0.4, -0.2, 0.9), "li6_n2_3b": (0.3, -0.5)}


def dense(d):
    P = oracle.Port(d)
    D = P.dimension
    H = np.zeros((D, D))
    for i in range(D):
        e = np.zeros(D)
        e[i] = 1.0
        H[:, i] = P.matvec(e)
    P.close()
    return H


@pytest.fixture(scope="module")
def families(tmp_path_factory):
    """Per basis: H0 (interaction + oscillator term) and H1 (another seeded
    interaction, no oscillator term) on the same lists, with their dense
    matrices from the oracle."""
    root = tmp_path_factory.mktemp("bases")
    out = {}
    for name, (Z, N, nmax, nbody, M2) in BASES.items():
        d0, d1 = str(root / f"{name}_h0"), str(root / f"{name}_h1")
        jn.generate(d0, Z=Z, N=N, nmax=nmax, nbody=nbody, M2=M2, basis_files=False)
        jn.generate(d1, Z=Z, N=N, nmax=nmax, nbody=nbody, M2=M2, seed=777, hbar_omega=0.0, basis_files=False)
        out[name] = (d0, d1, Z, N, dense(d0), dense(d1))
    return out


def open_all(families):
    hs, mes = {}, {}
    for name, (d0, d1, Z, N, _, _) in families.items():
        H = jn.Hamiltonian.from_dir(d0, Z, N)
        me0 = H.read_matrix_elements(os.path.join(d0, "matrix_elements"))
        me1 = H.read_matrix_elements(os.path.join(d1, "matrix_elements"))
        hs[name] = H
        mes[name] = [me0 + c * me1 for c in CS[name]]
    return hs, mes


@pytest.mark.parametrize("engine,precision", [(4, 32), (5, 32), (5, 64)])
def test_bases_match_dense_eigenvalues(families, engine, precision):
    """Panel-engine contexts at precision 32 share one panel launch per step;
    otherwise (a context on the walk engine, or precision 64) one walk launch."""
    hs, mes = open_all(families)
    try:
        names = list(BASES)
        if engine == 5:
            hs[names[0]].set_engine(5)
        res = jn.lanczos_batch_bases([(hs[n], mes[n]) for n in names], precision=precision, num_eigenvalues=10,
                                     tolerance=1e-6, max_iterations=300)
        assert [len(r) for r in res] == [len(CS[n]) for n in names]
        for n, rs in zip(names, res):
            H0, H1 = families[n][4], families[n][5]
            for c, r in zip(CS[n], rs):
                want = np.linalg.eigvalsh(H0 + c * H1)[:10]
                assert r["converged"], (n, c, r["iterations"])
                assert len(r["eigenvalues"]) == 10
                assert np.abs(r["eigenvalues"] - want).max() <= EIG_TOL, (n, c, r["eigenvalues"] - want)
                assert r["iterations"] <= hs[n].dimension
    finally:
        for H in hs.values():
            H.close()


def test_bases_graph_replay_is_bit_identical(families):
    hs, mes = open_all(families)
    try:
        bases = [(hs[n], mes[n]) for n in BASES]
        a = jn.lanczos_batch_bases(bases, use_graph=True)
        b = jn.lanczos_batch_bases(bases, use_graph=False)
        for ra, rb in zip(a, b):
            for x, y in zip(ra, rb):
                assert x["iterations"] == y["iterations"]
                assert np.array_equal(x["eigenvalues"], y["eigenvalues"])
    finally:
        for H in hs.values():
            H.close()


def test_bases_return_eigenvectors(families):
    """Per basis, vectors of that basis's dimension: orthonormal, with the refined
    eigenvalues as their Rayleigh quotients."""
    hs, mes = open_all(families)
    try:
        names = list(BASES)
        res, vecs = jn.lanczos_batch_bases([(hs[n], mes[n]) for n in names], eigenvectors=3, num_eigenvalues=3,
                                           tolerance=1e-8)
        for n, rs, vs in zip(names, res, vecs):
            H0, H1 = families[n][4], families[n][5]
            for c, r, X in zip(CS[n], rs, vs):
                assert X.shape == (3, hs[n].dimension)
                Hc = H0 + c * H1
                assert np.abs(X @ X.T - np.eye(3)).max() < 1e-8
                assert np.abs(np.diag(X @ Hc @ X.T) - r["eigenvalues"]).max() < 1e-7
    finally:
        for H in hs.values():
            H.close()


def test_bases_reject_mismatched_options(families):
    hs, mes = open_all(families)
    try:
        n0, n1 = list(BASES)[:2]
        opts = (jn.BatchOptions * 2)()
        keep = []
        for o, n in zip(opts, (n0, n1)):
            arrs = [np.ascontiguousarray(m) for m in mes[n]]
            ptrs = (jn.ctypes.c_void_p * len(arrs))(*[a.ctypes.data for a in arrs])
            keep += [arrs, ptrs]
            o.num_instances, o.matrix_elements = len(arrs), jn.ctypes.cast(ptrs, jn.ctypes.c_void_p)
            o.max_iterations, o.num_eigenvalues, o.tolerance, o.precision = 100, 5, 1e-6, 32
            o.check_every, o.use_graph, o.refine_extra = 10, 1, 4
        opts[1].tolerance = 1e-7
        res = [(jn.BatchResult * len(mes[n]))() for n in (n0, n1)]
        ctxs = (jn.ctypes.c_void_p * 2)(hs[n0]._h, hs[n1]._h)
        rp = (jn.ctypes.c_void_p * 2)(*[jn.ctypes.addressof(r) for r in res])
        assert jn.gpu_lib().jn_lanczos_batch_bases(ctxs, 2, opts, rp) != 0
        assert b"differ" in jn.gpu_lib().jn_last_error()
        with pytest.raises(jn.JnError):
            jn.lanczos_batch_bases([(hs[n0], mes[n0])], precision=16)
    finally:
        for H in hs.values():
            H.close()
