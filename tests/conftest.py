import os
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


def _ensure_built():
    import jupiterncsm_gb300 as jn
    import oracle
    if not (os.path.exists(jn.GPU_LIB) and os.path.exists(jn.GEN_LIB)):
        jn.build()
    if not os.path.exists(oracle.PORT_LIB):
        subprocess.run(["make", "-s", "-C", oracle.HERE, "port"], check=True)
    if oracle.reference_tree_present() and not (os.path.exists(oracle.REF_LIB) and os.path.exists(oracle.REF_MERCURY)):
        subprocess.run(["make", "-s", "-C", oracle.HERE, "ref", f"REFERENCE={oracle.REFERENCE}"], check=True)
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "tests", "native")], check=True)


_ensure_built()

# name -> (Z, N, Nmax, nbody, 2M)
PROBLEMS = {
    "he4_n2_2b": (2, 2, 2, 2, 0),
    "he4_n2_3b": (2, 2, 2, 3, 0),
    "he4_n4_2b": (2, 2, 4, 2, 0),
    "li6_n2_3b": (3, 3, 2, 3, 2),
    "he4_n6_3b": (2, 2, 6, 3, 0),
    # 6Li Nmax 6, 2M = 2, two- plus three-body: D = 186 894, 2.26 G multiply-adds per product
    "li6_n6_3b": (3, 3, 6, 3, 2),
}


@pytest.fixture(scope="session")
def problem_root(tmp_path_factory):
    return tmp_path_factory.mktemp("problems")


_cache = {}


@pytest.fixture(scope="session")
def problem(problem_root):
    """problem(name) -> (directory, Z, N, Nmax, nbody)."""
    import jupiterncsm_gb300 as jn

    def get(name):
        if name not in _cache:
            Z, N, nmax, nbody, M2 = PROBLEMS[name]
            d = str(problem_root / name)
            jn.generate(d, Z=Z, N=N, nmax=nmax, nbody=nbody, M2=M2, basis_files=False)
            _cache[name] = (d, Z, N, nmax, nbody)
        return _cache[name]
    return get


# J-scheme problems for the transform: name -> (Z, N, Nmax, 2M)
TRANSFORM_PROBLEMS = {
    "he4_n2": (2, 2, 2, 0),
    "li6_n2": (3, 3, 2, 2),
    "he4_n4": (2, 2, 4, 0),
    "li6_n4": (3, 3, 4, 2),
}
_tcache = {}


@pytest.fixture(scope="session")
def jproblem(problem_root):
    """jproblem(name) -> (directory, Z, N, emax_single, emax_pair): a generated
    problem whose two-body interaction is an Antoine J-scheme file."""
    import jupiterncsm_gb300 as jn

    def get(name):
        if name not in _tcache:
            Z, N, nmax, M2 = TRANSFORM_PROBLEMS[name]
            d = str(problem_root / ("j_" + name))
            s = jn.generate(d, Z=Z, N=N, nmax=nmax, M2=M2, nbody=2, antoine=True)
            _tcache[name] = (d, Z, N, s["emax_single"], s["emax_pair"])
        return _tcache[name]
    return get


def reference_tree_present():
    import oracle
    return oracle.reference_tree_present()
