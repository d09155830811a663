"""4He Nmax 6 with two- plus three-body forces (D = 7 916): each of the 10
lowest eigenvalues from the plain FP64 solver and from the mixed-precision
solvers (FP32 products, FP64 recurrence and refinement), against the dense
eigenvalues of the oracle's matrix (the port's products of every unit
vector).  Every state must agree within 1e-6 MeV."""
import os

import numpy as np
import pytest

import jupiterncsm_gb300 as jn
import oracle

pytestmark = pytest.mark.gpu
TOL_MEV = 1e-6


@pytest.fixture(scope="module")
def dense(problem):
    d, Z, N, *_ = problem("he4_n6_3b")
    p = oracle.Port(d)
    D = p.dimension
    threads = os.cpu_count() or 1
    H = np.zeros((D, D))
    e = np.zeros(D)
    for j in range(D):
        e[j] = 1.0
        col = np.zeros(D)
        p.matvec_omp(e, col, threads)
        H[:, j] = col
        e[j] = 0.0
    p.close()
    from scipy.linalg import eigh
    w = eigh(0.5 * (H + H.T), eigvals_only=True, subset_by_index=[0, 9])
    return d, Z, N, w


def test_per_state_errors_plain_and_mixed(dense):
    d, Z, N, w = dense
    H = jn.Hamiltonian.from_dir(d, Z, N)
    me = H.read_matrix_elements(os.path.join(d, "matrix_elements"))
    rows = {}
    H.set_precision(64)
    rows["plain_fp64"] = H.lanczos(max_iterations=400, num_eigenvalues=10, tolerance=TOL_MEV)["eigenvalues"]
    H.set_precision(32)
    rows["mixed_single"] = H.lanczos(max_iterations=400, num_eigenvalues=10, tolerance=TOL_MEV)["eigenvalues"]
    rows["mixed_batched"] = H.lanczos_batch([me], max_iterations=400, num_eigenvalues=10, tolerance=TOL_MEV,
                                            precision=32)[0]["eigenvalues"]
    H.close()
    print("\nstate  dense eigh (MeV)        " + "  ".join(f"{k:>14}" for k in rows))
    for i in range(10):
        print(f"{i:5d}  {w[i]: .15f}  " + "  ".join(f"{abs(rows[k][i] - w[i]):14.3e}" for k in rows))
    for k, v in rows.items():
        err = np.abs(np.asarray(v[:10]) - w)
        assert err.max() <= TOL_MEV, (k, err)
