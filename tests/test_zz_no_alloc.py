"""The allocation-free product (jn_matvec_device_noalloc), for callers that
cannot let the library allocate device memory: it must give what
jn_matvec_device gives, call after call.  Collected last on purpose."""
import ctypes

import numpy as np
import pytest

import jupiterncsm_gb300 as jn

pytestmark = pytest.mark.gpu
TOL = 1e-12   # same relative tolerance as the other FP64 product tests


def test_noalloc_matches_allocating_product_twice(problem):
    torch = pytest.importorskip("torch")
    d, Z, N, *_ = problem("he4_n6_3b")
    H = jn.Hamiltonian.from_dir(d, Z, N)
    L = jn.gpu_lib()
    L.jn_matvec_device_noalloc.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int, ctypes.c_void_p]
    L.jn_matvec_device_noalloc.restype = ctypes.c_int
    dev = torch.device("cuda", 0)
    g = torch.Generator(device=dev).manual_seed(5)
    x = torch.randn(H.dimension, dtype=torch.float64, device=dev, generator=g)
    want = torch.zeros_like(x)
    H.matvec_device(x.data_ptr(), want.data_ptr(), accumulate=False)
    H.synchronize()
    scale = float(want.abs().max())
    for call in range(2):
        y = torch.full_like(x, float("nan"))
        st = L.jn_matvec_device_noalloc(H._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), 0, None)
        assert st == 0, L.jn_last_error().decode()
        H.synchronize()
        assert float((y - want).abs().max()) <= TOL * scale, f"call {call}"
    # accumulate mode adds onto y
    y = want.clone()
    assert L.jn_matvec_device_noalloc(H._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), 1, None) == 0
    H.synchronize()
    assert float((y - 2 * want).abs().max()) <= TOL * 2 * scale
    H.close()
