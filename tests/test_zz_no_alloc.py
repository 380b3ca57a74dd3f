"""tl_gemm_noalloc: the split-k tensor-core GEMM whose scratch is a static device array, for callers
that cannot call cudaMalloc (an application that owns all device memory through its own pool, a
latency-critical path that must not allocate, a caller without a tl_handle).

Called through the C ABI and checked against tl_gemm on the same problem and solution, twice in a
row (the static scratch keeps the previous call's contents, so the second call checks that every
call clears what must start at zero).  Collected last so that a run stopping at the first failure
has already run every other test.
"""
import ctypes

import numpy as np
import pytest

import tensilelite_gb300 as tl
from tests import gpu_util as gu
from tests.golden import gen_golden as gg

pytestmark = pytest.mark.gpu


def _noalloc_fn():
    fn = tl.lib().tl_gemm_noalloc
    fn.argtypes = [ctypes.POINTER(tl.Problem), ctypes.POINTER(tl.Solution), ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return fn


def test_noalloc_matches_tl_gemm_twice():
    import torch
    torch.cuda.init()
    fn = _noalloc_fn()
    h = tl.Handle()
    m, n, k = 480, 1024, 4096
    case = gg.make_case("bf16", "NN", 404, m, n, k, alpha=1.0, beta=0.5)
    A, B = gu.to_dev(case["A_bits"], "bf16"), gu.to_dev(case["B_bits"], "bf16")
    C = gu.to_dev(case["C_bits"], "bf16")
    p = tl.Problem.make(m, n, k, dtype="bf16", alpha=1.0, beta=0.5, lda=case["lda"], ldb=case["ldb"],
                        kernel="tcgen05")
    # split-k 4 over 32 tiles of 128 x 128: 8 MiB of partials in the static scratch
    sol = tl.Solution(kernel=tl.KERNEL_TCGEN05, macro_tile0=128, macro_tile1=128, depth_u=64, stages=4, split_k=4)
    ref = torch.empty(m * n, dtype=torch.bfloat16, device="cuda")
    h.gemm(p, ref, C, A, B, solution=sol)
    h.device_status()
    ref_vals = gu.from_dev(ref, "bf16")
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        D = torch.full((m * n,), float("nan"), dtype=torch.bfloat16, device="cuda")
        st = fn(ctypes.byref(p), ctypes.byref(sol), D.data_ptr(), C.data_ptr(), A.data_ptr(), B.data_ptr(), stream)
        assert st == tl.SUCCESS, tl.lib().tl_last_error_string()
        torch.cuda.synchronize()
        got = gu.from_dev(D, "bf16")
        # same kernel, same split order: the tests' tolerance (one bf16 ulp) and in fact bit-equal
        assert gu.ulp_diff_count(got, ref_vals, "bf16") == 0, f"call {call}"
        assert np.array_equal(got.view(np.uint32), ref_vals.view(np.uint32)), f"call {call}"
    h.close()


def test_noalloc_refuses_oversized_workspace():
    import torch
    torch.cuda.init()
    fn = _noalloc_fn()
    m = n = k = 8192
    A = torch.empty(m * k, dtype=torch.bfloat16, device="cuda")
    B = torch.empty(k * n, dtype=torch.bfloat16, device="cuda")
    D = torch.empty(m * n, dtype=torch.bfloat16, device="cuda")
    p = tl.Problem.make(m, n, k, dtype="bf16", kernel="tcgen05")
    sol = tl.Solution(kernel=tl.KERNEL_TCGEN05, macro_tile0=256, macro_tile1=128, depth_u=64, stages=4, split_k=8)
    st = fn(ctypes.byref(p), ctypes.byref(sol), D.data_ptr(), None, A.data_ptr(), B.data_ptr(),
            torch.cuda.current_stream().cuda_stream)
    assert st == tl.ERR_UNSUPPORTED
    assert b"static scratch" in tl.lib().tl_last_error_string()
