"""hx_gemm_noalloc through the C ABI: the allocation-free tensor-core GEMM.

It serves callers that cannot allocate device memory when they call it (their
memory belongs to their own pool allocator, or a cudaFree would synchronise
the device under other streams' work). Operands live in device memory
(allocated here by torch, before and outside the call).
Each call must give exactly hx_gemm's result for the same problem, twice in a
row (the static scratch is reused), must not change the device's free memory,
and must reject problems larger than the static scratch.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_DIM = 512            # HX_NOALLOC_MAX_DIM in include/helios_cc.h


@pytest.fixture(scope="module")
def lib():
    from helios_gb300 import build
    build.build()
    from helios_gb300 import api
    lib = api.library()
    lib.hx_gemm_noalloc.restype = ctypes.c_int
    lib.hx_gemm_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                    ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p]
    return lib


def _call(lib, dA, dB, dC, M, N, K, precision):
    return lib.hx_gemm_noalloc(dA.data_ptr(), dB.data_ptr(), dC.data_ptr(), M, N, K, precision, None)


@pytest.mark.parametrize("precision,name", [(1, "mixed"), (2, "high")])
def test_two_calls_match_hx_gemm(lib, precision, name):
    import torch
    from helios_gb300 import api
    rng = np.random.default_rng(17 + precision)
    for (M, N, K) in ((300, 200, 100), (512, 384, 500)):
        A = rng.normal(size=(M, K))
        B = rng.normal(size=(N, K)) * np.exp(rng.normal(size=(N, 1)))       # rows of different scales
        ref, _ = api.gemm(A, B, name)
        dA = torch.from_numpy(A).cuda()
        dB = torch.from_numpy(B).cuda()
        dC = torch.full((M, N), 7.0, dtype=torch.float64, device="cuda")    # C is cleared by the call
        torch.cuda.synchronize()
        assert _call(lib, dA, dB, dC, M, N, K, precision) == 0, api.last_error()
        first = dC.cpu().numpy().copy()
        free0 = torch.cuda.mem_get_info()[0]
        assert _call(lib, dA, dB, dC, M, N, K, precision) == 0, api.last_error()
        torch.cuda.synchronize()
        free1 = torch.cuda.mem_get_info()[0]
        second = dC.cpu().numpy()
        assert np.array_equal(first, ref)
        assert np.array_equal(second, ref)
        assert free1 == free0
        exact = A @ B.T
        tol = 1e-6 if precision == 1 else 1e-10
        assert np.abs(second - exact).max() / np.abs(exact).max() < tol


def test_rejects_problems_above_the_static_limit(lib):
    import torch
    from helios_gb300 import api
    dA = torch.zeros((MAX_DIM + 1, 64), dtype=torch.float64, device="cuda")
    dB = torch.zeros((64, 64), dtype=torch.float64, device="cuda")
    dC = torch.zeros((MAX_DIM + 1, 64), dtype=torch.float64, device="cuda")
    assert _call(lib, dA, dB, dC, MAX_DIM + 1, 64, 64, 1) == -100
    assert "static scratch limit" in api.last_error()
    assert _call(lib, dB, dB, dC, 64, 64, 64, 0) == -100          # FP64 is not offered here
