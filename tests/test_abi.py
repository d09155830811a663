"""The C-ABI library loads and exports every symbol include/*.h declares.
No device call is made here (this suite runs without a GPU); the host-only
plan statistics are checked against the files."""
import ctypes
import glob
import os
import re

import jupiterncsm_gb300 as jn

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        for m in re.finditer(r"\b(jn_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported():
    lib = ctypes.CDLL(jn.GPU_LIB)
    names = declared_functions()
    assert "jn_matvec" in names and "jn_open" in names
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_error_string():
    L = jn.gpu_lib()
    assert L.jn_version().decode().startswith("jncsm-gb300")
    assert isinstance(L.jn_last_error(), bytes)


def test_null_arguments_are_rejected_without_a_device():
    L = jn.gpu_lib()
    h = ctypes.c_void_p()
    assert L.jn_open_files(None, None, None, None, 2, 2, ctypes.byref(h)) == 1
    assert L.jn_matvec(None, None, None) == 1
    assert L.jn_get_plan_stats(None, None) == 1


def test_host_inspect_matches_the_files(problem):
    """jn_inspect_files builds the plan on the host (no device): its statistics
    agree with counts taken from the files and with the oracle's dimension."""
    import numpy as np
    import oracle
    d, Z, N, *_ = problem("li6_n2_3b")
    st = jn.inspect(d, Z, N)
    P = oracle.Port(d)
    assert st["dimension"] == P.dimension
    P.close()
    lists = os.listdir(os.path.join(d, "index_lists"))
    entries = sum(os.path.getsize(os.path.join(d, "index_lists", f)) // 12 for f in lists)
    mes = os.listdir(os.path.join(d, "matrix_elements"))
    elements = sum((os.path.getsize(os.path.join(d, "matrix_elements", f)) - 16) // 8 for f in mes)
    assert st["list_entries"] == entries and st["me_elements"] == elements
    assert 0 < st["me_referenced"] <= st["me_elements"]
    assert st["algorithmic_bytes"] == 12.0 * entries + 8.0 * st["me_referenced"] + 16.0 * st["dimension"]
    assert st["num_work_units"] > 0 and st["num_tiles"] > 0 and st["multiply_adds"] > 0
    assert st["num_instructions"] == sum(1 for l in open(os.path.join(d, "evaluation_order.txt")) if "BLOCK:" in l
                                         and "UNLOAD_" not in l)
    np.testing.assert_equal(jn.inspect(d, Z, N), st)          # deterministic
