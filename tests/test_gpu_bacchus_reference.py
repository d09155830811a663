"""The reference-algorithm Lanczos (JN_LANCZOS_REFERENCE) against the
reference's own Bacchus: fixtures written by the compiled reference
eigensolver (tests/golden/make_golden_bacchus.py) hold the final eigensystem
block (its length is the Lanczos dimension reached) and the lowest
eigenvector, under both convergence criteria of the run file."""
import glob
import json
import os

import numpy as np
import pytest

import jupiterncsm_gb300 as jn

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CASES = sorted(os.path.basename(f)[:-5] for f in glob.glob(os.path.join(GOLDEN, "bacchus_*.json")))


@pytest.mark.parametrize("name", CASES)
def test_reference_mode_matches_reference_bacchus(tmp_path, name):
    meta = json.load(open(os.path.join(GOLDEN, f"{name}.json")))
    want = np.array(meta["eigenvalues"])
    want_vec = np.load(os.path.join(GOLDEN, f"{name}.npz"))["eigenvector"]
    d = str(tmp_path / "p")
    jn.generate(d, basis_files=False, **meta["config"])
    run = meta["lanczos"]
    H = jn.Hamiltonian.from_dir(d, meta["config"]["Z"], meta["config"]["N"])
    r = H.lanczos(max_iterations=run["max_iterations"], num_eigenvalues=1, tolerance=run["tolerance"],
                  mode=jn.LANCZOS_REFERENCE, converge_eigenvectors=run.get("converge_eigenvectors", False))
    got = H.ritz_values()
    vec = H.eigenvector(0)
    H.close()
    # the same Lanczos dimension and the same eigensystem block
    assert r["iterations"] == meta["num_eigenvalues"] == len(got)
    assert np.abs(got - want).max() <= 1e-10 * max(1.0, np.abs(want).max())
    # the same ground-state vector, with the reference's sign (the tridiagonal eigenvector's first
    # component is not negative, diagonalization.c:55-58), as its eigenvector files hold it
    assert np.abs(vec - want_vec).max() <= 1e-8
