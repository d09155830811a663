"""GPU Lanczos (FP64) against dense diagonalisation of the oracle's matrix,
and the FP32-matrix-element product against the FP64 oracle."""
import numpy as np
import pytest

import jupiterncsm_gb300 as jn
import oracle

pytestmark = pytest.mark.gpu


def dense_from_port(d):
    p = oracle.Port(d)
    D = p.dimension
    H = np.column_stack([p.matvec(np.eye(D)[j]) for j in range(D)])
    p.close()
    return 0.5 * (H + H.T)


@pytest.mark.parametrize("name", ["he4_n2_3b", "he4_n4_2b", "li6_n2_3b"])
def test_full_reorth_lanczos_ten_lowest(problem, name):
    d, Z, N, *_ = problem(name)
    w = np.linalg.eigvalsh(dense_from_port(d))[:10]
    H = jn.Hamiltonian.from_dir(d, Z, N)
    r = H.lanczos(max_iterations=min(300, H.dimension), num_eigenvalues=10, tolerance=1e-8)
    assert r["converged"]
    # eigenvalue error stated against the FP64 oracle (dense eigh of the same H): 1e-6 MeV
    assert np.abs(r["eigenvalues"] - w).max() < 1e-6, (r["eigenvalues"], w)
    assert np.abs(r["ritz_values"] - w).max() < 1e-6
    assert r["residual_norms"].max() < 1e-3
    x0 = H.eigenvector(0)
    assert abs(np.linalg.norm(x0) - 1) < 1e-8
    H.close()


def test_reference_mode_converges_to_ground_state(problem):
    d, Z, N, *_ = problem("he4_n4_2b")
    w = np.linalg.eigvalsh(dense_from_port(d))
    H = jn.Hamiltonian.from_dir(d, Z, N)
    r = H.lanczos(max_iterations=200, num_eigenvalues=1, tolerance=1e-10, mode=jn.LANCZOS_REFERENCE)
    # the reference's convergence test is on the lowest Ritz value only
    assert abs(r["eigenvalues"][0] - w[0]) < 1e-6
    rv = H.ritz_values()
    assert len(rv) == r["iterations"] and np.all(np.diff(rv) >= 0)
    H.close()


def test_lanczos_alpha_beta_bit_identical(problem):
    d, Z, N, *_ = problem("he4_n4_2b")
    H = jn.Hamiltonian.from_dir(d, Z, N)
    a = H.lanczos(max_iterations=60, num_eigenvalues=5, tolerance=1e-300, allow_unconverged=True)
    ra = H.ritz_values()
    b = H.lanczos(max_iterations=60, num_eigenvalues=5, tolerance=1e-300, allow_unconverged=True)
    rb = H.ritz_values()
    assert np.array_equal(ra.view(np.uint64), rb.view(np.uint64))
    H.close()


@pytest.mark.parametrize("name", ["he4_n4_2b", "he4_n6_3b"])
def test_fp32_product_within_single_precision(problem, name):
    d, Z, N, *_ = problem(name)
    H = jn.Hamiltonian.from_dir(d, Z, N)
    x = np.random.default_rng(8).standard_normal(H.dimension)
    want = oracle.Port(d).matvec(x)
    H.set_precision(32)
    got = H.matvec(x)
    # FP32 matrix elements and x: about 1e-7 relative per product term
    assert np.abs(got - want).max() <= 2e-6 * np.abs(want).max()
    H.set_precision(64)
    got64 = H.matvec(x)
    assert np.abs(got64 - want).max() <= 1e-12 * np.abs(want).max()
    H.close()


def test_save_eigenvectors_layout(problem, tmp_path):
    d, Z, N, *_ = problem("he4_n2_2b")
    H = jn.Hamiltonian.from_dir(d, Z, N)
    H.lanczos(max_iterations=59, num_eigenvalues=2, tolerance=1e-8)
    H.save_eigenvectors(str(tmp_path / "ev"), 2)
    blocks = oracle.read_blocks(d)
    v = oracle.read_vector_dir(str(tmp_path / "ev" / "eigenvector_1"), [(i + 1, a, b) for i, (_, a, b) in enumerate(blocks)])
    assert np.allclose(v, H.eigenvector(0))
    H.close()
