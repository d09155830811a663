"""The jn_bacchus command line: a drop-in for bacchus.x reading the same run
file and printing the same eigensystem block."""
import os
import re
import subprocess

import numpy as np
import pytest

import jupiterncsm_gb300 as jn
import oracle

pytestmark = pytest.mark.gpu


def parse_eigensystem(text):
    m = re.search(r"eigensystem:\n\{\n\tnum_eigenvalues = (\d+);\n\teigenvalues = \( (.*) \);\n\}", text)
    assert m, text[-2000:]
    vals = [float(v.strip()) for v in m.group(2).split(",")]
    assert len(vals) == int(m.group(1))
    return np.array(vals)


@pytest.mark.parametrize("full", [False, True])
def test_cli_matches_dense_ground_state(problem, tmp_path, full):
    d, Z, N, *_ = problem("he4_n4_2b")
    conf = tmp_path / "run.conf"
    text = open(f"{d}/bacchus.conf").read()
    text = text.replace(f"{d}/eigen_vectors", str(tmp_path / "ev"))
    if full:
        text += 'gpu:\n{\n\treorthogonalize = "full";\n\tnum_eigenvalues = 10;\n};\n'
    conf.write_text(text)
    out = subprocess.run([jn.BACCHUS_CLI, "--settings-file", str(conf)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    ev = parse_eigensystem(out.stdout)
    p = oracle.Port(d)
    D = p.dimension
    H = np.column_stack([p.matvec(np.eye(D)[j]) for j in range(D)])
    w = np.linalg.eigvalsh(0.5 * (H + H.T))
    assert abs(ev[0] - w[0]) < 1e-6
    if full:
        assert np.abs(ev[:10] - w[:10]).max() < 1e-6
    assert os.path.exists(tmp_path / "ev" / "eigenvector_1" / "vec_1")


def test_cli_rejects_bad_settings_name(tmp_path):
    out = subprocess.run([jn.BACCHUS_CLI, "--settings-file", str(tmp_path / "x.txt")], capture_output=True, text=True)
    assert out.returncode != 0 and "must end in .conf" in out.stderr
