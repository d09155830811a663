"""The allocation-free product (jn_matvec_device_noalloc), for callers that
cannot let the library allocate device memory: with the block-tile engine
active on the context, it must give bit for bit what jn_matvec_device
gives, call after call, at both precisions and in accumulate mode, and
agree with the default engine to rounding.  Collected last on purpose."""
import ctypes

import pytest

import jupiterncsm_gb300 as jn

pytestmark = pytest.mark.gpu
TOL = {64: 1e-12, 32: 2e-6}   # relative to max|y|, as the other product tests


@pytest.mark.parametrize("bits", [64, 32])
def test_noalloc_matches_allocating_product_twice(problem, bits):
    torch = pytest.importorskip("torch")
    d, Z, N, *_ = problem("he4_n6_3b")
    H = jn.Hamiltonian.from_dir(d, Z, N)
    L = jn.gpu_lib()
    L.jn_matvec_device_noalloc.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int, ctypes.c_void_p]
    L.jn_matvec_device_noalloc.restype = ctypes.c_int
    dev = torch.device("cuda", 0)
    g = torch.Generator(device=dev).manual_seed(5)
    x = torch.randn(H.dimension, dtype=torch.float64, device=dev, generator=g)
    H.set_precision(bits)
    default = torch.zeros_like(x)
    H.matvec_device(x.data_ptr(), default.data_ptr(), accumulate=False)
    H.set_engine(3)                 # the engine the allocation-free product runs
    want = torch.zeros_like(x)
    H.matvec_device(x.data_ptr(), want.data_ptr(), accumulate=False)
    H.synchronize()
    scale = float(want.abs().max())
    assert float((want - default).abs().max()) <= TOL[bits] * scale
    for call in range(2):
        y = torch.full_like(x, float("nan"))
        st = L.jn_matvec_device_noalloc(H._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), 0, None)
        assert st == 0, L.jn_last_error().decode()
        H.synchronize()
        assert torch.equal(y, want), f"call {call}"
    # accumulate mode adds onto y, as the allocating call does
    y, y2 = want.clone(), want.clone()
    assert L.jn_matvec_device_noalloc(H._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), 1, None) == 0
    H.matvec_device(x.data_ptr(), y2.data_ptr(), accumulate=True)
    H.synchronize()
    assert torch.equal(y, y2)
    H.close()
