"""tl_gemm_noalloc: the split-k tensor-core GEMM whose scratch is a static device array, for callers
that cannot call cudaMalloc -- an application that owns all device memory through its own pool, a
latency-critical path where an allocation (which can synchronise the device) is not acceptable, or a
caller without a tl_handle (creating one allocates).

Every case runs through the C ABI twice in a row (the static scratch keeps the previous call's
contents, so the second call checks that each call clears what must start at zero) and is checked
against tl_gemm on the same problem and solution -- the same kernel and split order, so the results
are bit-equal, well inside the tests' one-ulp tolerance -- and against the oracle (the restated
reference loop) with the parity tolerance of the other GPU tests.  The calls allocate nothing on the
device (free memory and torch's reserved memory are unchanged across them, after a warm-up), and the
error word reads clean through tl_noalloc_status.  A call made to time out (TL_DEBUG_SKIP_LOADS, a
20 ms wait limit) is reported as TL_ERR_TIMEOUT and the next call is correct.  Collected last so that
a run stopping at the first failure has already run every other test.
"""
import ctypes
import os

import numpy as np
import pytest

import tensilelite_gb300 as tl
from tests import gpu_util as gu
from tests.golden import gen_golden as gg

pytestmark = pytest.mark.gpu


def _noalloc(p, sol, D, C, A, B, stream):
    return tl.lib().tl_gemm_noalloc(ctypes.byref(p), ctypes.byref(sol) if sol is not None else None, D.data_ptr(),
                                    C.data_ptr() if C is not None else None, A.data_ptr(), B.data_ptr(), stream)


# (dtype, layout, m, n, k, solution fields): one SM per tile with split-k 4; a CTA pair (256-row
# tiles) with split-k 3; fp8 operands with split-k 2
CASES = [
    ("bf16", "NN", 480, 1024, 4096, dict(macro_tile0=128, macro_tile1=128, stages=4, split_k=4)),
    ("fp16", "TN", 512, 768, 2048, dict(macro_tile0=256, macro_tile1=256, stages=4, split_k=3)),
    ("fp8", "TN", 384, 512, 2048, dict(macro_tile0=128, macro_tile1=128, stages=4, split_k=2)),
]


@pytest.mark.parametrize("dt,lay,m,n,k,fields", CASES, ids=["bf16_cg1_split4", "fp16_pair_split3", "fp8_split2"])
def test_noalloc_matches_tl_gemm_and_oracle_twice(dt, lay, m, n, k, fields):
    import torch
    torch.cuda.init()
    case = gg.make_case(dt, lay, 404 + CASES.index((dt, lay, m, n, k, fields)), m, n, k, alpha=1.0, beta=0.5)
    od = case["out_dtype"]
    A, B = gu.to_dev(case["A_bits"], dt), gu.to_dev(case["B_bits"], dt)
    C = gu.to_dev(case["C_bits"], od)
    p = tl.Problem.make(m, n, k, dtype=dt, out_dtype=od, trans_a=case["trans_a"], trans_b=case["trans_b"],
                        alpha=1.0, beta=0.5, lda=case["lda"], ldb=case["ldb"], kernel="tcgen05")
    W = 128 if dt == "fp8" else 64
    sol = tl.Solution(kernel=tl.KERNEL_TCGEN05, depth_u=W, **fields)
    h = tl.Handle()
    ref = torch.empty(m * n, dtype=gu.torch_dtype(od), device="cuda")
    h.gemm(p, ref, C, A, B, solution=sol)
    h.device_status()
    ref_vals = gu.from_dev(ref, od)
    h.close()
    stream = torch.cuda.current_stream().cuda_stream
    D = torch.full((m * n,), float("nan"), dtype=gu.torch_dtype(od), device="cuda")
    assert _noalloc(p, sol, D, C, A, B, stream) == tl.SUCCESS, tl.lib().tl_last_error_string()   # warm-up
    torch.cuda.synchronize()
    free0, reserved0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_reserved()
    for call in range(2):
        D.fill_(float("nan"))
        st = _noalloc(p, sol, D, C, A, B, stream)
        assert st == tl.SUCCESS, tl.lib().tl_last_error_string()
        assert tl.lib().tl_noalloc_status(stream) == tl.SUCCESS, tl.lib().tl_last_error_string()
        got = gu.from_dev(D, od)
        assert gu.ulp_diff_count(got, ref_vals, od) == 0, f"call {call}"
        assert np.array_equal(got.view(np.uint32), ref_vals.view(np.uint32)), f"call {call}"
        gu.check_against_oracle(got, case, n_begin=0, n_end=min(n, 128))
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0, "device memory was allocated by tl_gemm_noalloc"
    assert torch.cuda.memory_reserved() == reserved0


def test_noalloc_timeout_reported_then_recovers():
    import torch
    torch.cuda.init()
    m, n, k = 256, 512, 1024
    case = gg.make_case("bf16", "NN", 410, m, n, k, alpha=1.0, beta=0.0)
    A, B = gu.to_dev(case["A_bits"], "bf16"), gu.to_dev(case["B_bits"], "bf16")
    D = torch.empty(m * n, dtype=torch.bfloat16, device="cuda")
    p = tl.Problem.make(m, n, k, dtype="bf16", lda=case["lda"], ldb=case["ldb"], kernel="tcgen05")
    sol = tl.Solution(kernel=tl.KERNEL_TCGEN05, macro_tile0=128, macro_tile1=128, depth_u=64, stages=4, split_k=2,
                      debug_flags=tl.DEBUG_SKIP_LOADS)
    stream = torch.cuda.current_stream().cuda_stream
    old = os.environ.get("TL_WAIT_TIMEOUT_MS")
    os.environ["TL_WAIT_TIMEOUT_MS"] = "20"
    try:
        assert _noalloc(p, sol, D, None, A, B, stream) == tl.SUCCESS
        assert tl.lib().tl_noalloc_status(stream) == tl.ERR_TIMEOUT
        assert b"timed out" in tl.lib().tl_last_error_string()
        assert tl.lib().tl_noalloc_status(stream) == tl.SUCCESS       # read and cleared
    finally:
        if old is None:
            del os.environ["TL_WAIT_TIMEOUT_MS"]
        else:
            os.environ["TL_WAIT_TIMEOUT_MS"] = old
    sol.debug_flags = 0
    for _ in range(2):
        assert _noalloc(p, sol, D, None, A, B, stream) == tl.SUCCESS
        assert tl.lib().tl_noalloc_status(stream) == tl.SUCCESS
        gu.check_against_oracle(gu.from_dev(D, "bf16"), case)


def test_noalloc_refuses_oversized_workspace():
    import torch
    torch.cuda.init()
    m = n = k = 8192
    A = torch.empty(m * k, dtype=torch.bfloat16, device="cuda")
    B = torch.empty(k * n, dtype=torch.bfloat16, device="cuda")
    D = torch.empty(m * n, dtype=torch.bfloat16, device="cuda")
    p = tl.Problem.make(m, n, k, dtype="bf16", kernel="tcgen05")
    sol = tl.Solution(kernel=tl.KERNEL_TCGEN05, macro_tile0=256, macro_tile1=128, depth_u=64, stages=4, split_k=8)
    st = _noalloc(p, sol, D, None, A, B, torch.cuda.current_stream().cuda_stream)
    assert st == tl.ERR_UNSUPPORTED
    assert b"static scratch" in tl.lib().tl_last_error_string()
