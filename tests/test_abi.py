"""The C-ABI library loads and exports every symbol include/*.h declares.
No compute call is made here (this suite runs without a GPU)."""
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
