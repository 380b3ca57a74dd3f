"""Device errors and the multicast guard, on the GPU, through the C ABI.

* A bounded device wait that runs out is reported (TL_ERR_TIMEOUT) and leaves the context usable.
  The wait is made to run out by the solution's TL_DEBUG_SKIP_LOADS bit: the TMA producer issues no
  copies, so the MMA and epilogue waits expire after the handle's limit (20 ms here).  Nothing is
  issued that could still be in flight when the kernel returns, and nothing faults.  This replaces
  the reference's E_ReturnState reporting (inc/ff_utils.h:44-50) for a kernel that cannot finish.
* The tuner never keeps a candidate that set the error word, and tuning in place (D == C, beta != 0)
  leaves C as it was.
* The cluster-of-four kernel loads through TMA multicast; the library refuses it for operands that
  are not memory of the current GPU (host-pinned buffers here), before anything is launched.
"""
import ctypes

import numpy as np
import pytest

import tensilelite_gb300 as tl
from tests import gpu_util as gu
from tests.golden import gen_golden as gg

pytestmark = pytest.mark.gpu


def _dev_case(case, dt):
    import torch
    A, B = gu.to_dev(case["A_bits"], dt), gu.to_dev(case["B_bits"], dt)
    C = gu.to_dev(case["C_bits"], case["out_dtype"]) if case["beta"] != 0 else None
    D = torch.full((case["ldc"] * case["n"],), float("nan"), dtype=gu.torch_dtype(case["out_dtype"]), device="cuda")
    p = tl.Problem.make(case["m"], case["n"], case["k"], dtype=dt, out_dtype=case["out_dtype"],
                        trans_a=case["trans_a"], trans_b=case["trans_b"], alpha=case["alpha"], beta=case["beta"],
                        lda=case["lda"], ldb=case["ldb"], ldc=case["ldc"], ldd=case["ldc"], kernel="tcgen05")
    return p, A, B, C, D


def test_wait_timeout_reported_and_context_recovers():
    import torch
    torch.cuda.init()
    case = gg.make_case("bf16", "NN", 501, 256, 256, 256, beta=0.0)
    p, A, B, C, D = _dev_case(case, "bf16")
    h = tl.Handle()
    h.set_wait_timeout(20)
    sol = tl.Solution(kernel=tl.KERNEL_TCGEN05, macro_tile0=128, macro_tile1=128, depth_u=64, stages=4, split_k=1,
                      tail_split=1, debug_flags=tl.DEBUG_SKIP_LOADS)
    h.gemm(p, D, C, A, B, solution=sol)
    with pytest.raises(tl.TLError) as e:
        h.device_status()
    assert e.value.status == tl.ERR_TIMEOUT and "timed out" in str(e.value)
    h.device_status()                     # the word was cleared when it was read
    h.close()
    # the context is usable: a normal GEMM on a fresh handle matches the oracle
    h2 = tl.Handle()
    sol.debug_flags = 0
    h2.gemm(p, D, C, A, B, solution=sol)
    h2.device_status()
    gu.check_against_oracle(gu.from_dev(D, "bf16"), case)
    h2.close()


def test_tune_in_place_keeps_c_and_skips_failed_candidates(tmp_path):
    import torch
    torch.cuda.init()
    case = gg.make_case("bf16", "TN", 502, 384, 512, 1024, beta=0.5)
    p, A, B, C, _ = _dev_case(case, "bf16")
    before = C.clone()
    h = tl.Handle()
    best, ms = h.tune(p, C, C, A, B, max_candidates=6, reps=2, cache_path=str(tmp_path / "tl.json"))
    torch.cuda.synchronize()
    assert torch.equal(C.view(torch.int16), before.view(torch.int16)), "tuning in place changed C"
    assert ms > 0 and best.debug_flags == 0
    h.device_status()
    # the tuned solution, in place for real this time, against the oracle
    h.gemm(p, C, C, A, B, solution=best)
    h.device_status()
    gu.check_against_oracle(gu.from_dev(C, "bf16"), case)
    h.close()


def test_multicast_refused_for_host_memory():
    import torch
    torch.cuda.init()
    m = n = k = 1024
    p = tl.Problem.make(m, n, k, dtype="bf16", kernel="tcgen05")
    sol = tl.Solution(kernel=tl.KERNEL_TCGEN05, macro_tile0=256, macro_tile1=512, depth_u=64, stages=6, split_k=1)
    hA = torch.zeros(m * k, dtype=torch.bfloat16).pin_memory()
    hB = torch.zeros(k * n, dtype=torch.bfloat16).pin_memory()
    dA = torch.zeros(m * k, dtype=torch.bfloat16, device="cuda")
    dB = torch.zeros(k * n, dtype=torch.bfloat16, device="cuda")
    D = torch.empty(m * n, dtype=torch.bfloat16, device="cuda")
    h = tl.Handle()
    launches = h.launch_count()
    for A, B in ((hA, dB), (dA, hB), (hA, hB)):
        with pytest.raises(tl.TLError) as e:
            h.gemm(p, D, None, A, B, solution=sol)
        assert e.value.status == tl.ERR_UNSUPPORTED and "multicast" in str(e.value)
    # the allocation-free entry refuses it the same way
    st = tl.lib().tl_gemm_noalloc(ctypes.byref(p), ctypes.byref(sol), D.data_ptr(), None, hA.data_ptr(),
                                  dB.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert st == tl.ERR_UNSUPPORTED
    assert h.launch_count() == launches, "a refused call launched a kernel"
    # on device memory the same solution runs (one GPU) and matches the oracle
    case = gg.make_case("bf16", "NN", 503, m, n, k, beta=0.0)
    p2, A, B, C, D2 = _dev_case(case, "bf16")
    h.gemm(p2, D2, C, A, B, solution=sol)
    h.device_status()
    gu.check_against_oracle(gu.from_dev(D2, "bf16"), case, n_begin=0, n_end=256)
    h.close()
