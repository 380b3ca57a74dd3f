"""Device timeline of the tensor-core kernel (tl_set_trace), on the GPU through the C ABI.

The counterpart of the reference's per-wave thread trace (test/ttrace): each CTA stamps its SM
cycle counter at the kernel's phases.  Checked here: every CTA of a traced launch records its
events in pipeline order, the result is unchanged by tracing, a buffer too small for the grid
records nothing, and switching the trace off leaves the buffer alone.
"""
import numpy as np
import pytest

import tensilelite_gb300 as tl

pytestmark = pytest.mark.gpu

EV = {name: i for i, name in enumerate(tl.TRACE_EVENTS)}


def _problem(m, n, k, beta, split):
    import torch
    g = torch.Generator(device="cuda").manual_seed(7)
    A = torch.randn(m * k, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(k * n, device="cuda", generator=g).to(torch.bfloat16)
    C = torch.randn(m * n, device="cuda", generator=g).to(torch.bfloat16)
    p = tl.Problem.make(m, n, k, dtype="bf16", beta=beta, kernel="tcgen05")
    sol = tl.Solution(kernel=tl.KERNEL_TCGEN05, macro_tile0=128, macro_tile1=128, depth_u=64, stages=4,
                      split_k=split, tail_split=1)
    return p, sol, A, B, C


@pytest.mark.parametrize("split", [1, 4])
def test_trace_records_each_cta_in_pipeline_order(split):
    import torch
    h = tl.Handle()
    m, n, k = 480, 1024, 2048
    p, sol, A, B, C = _problem(m, n, k, 0.5, split)
    ref = torch.empty(m * n, dtype=torch.bfloat16, device="cuda")
    h.gemm(p, ref, C, A, B, solution=sol)
    buf = torch.zeros(1024 * tl.TRACE_SLOTS, dtype=torch.int64, device="cuda")
    h.set_trace(buf)
    D = torch.empty_like(ref)
    h.gemm(p, D, C, A, B, solution=sol)
    h.device_status()
    h.set_trace(None)
    assert torch.equal(D.view(torch.int16), ref.view(torch.int16)), "tracing changed the result"
    t = buf.view(-1, tl.TRACE_SLOTS).cpu().numpy()
    rows = t[t[:, EV["entry"]] != 0]
    tiles = -(-m // 128) * (n // 128) * split
    assert 0 < len(rows) <= tiles
    assert rows[:, EV["tiles"]].sum() == tiles          # every work unit is processed exactly once
    order = ["entry", "setup", "dep", "load_first", "load_last"]
    for a, b in zip(order, order[1:]):
        assert (rows[:, EV[b]] >= rows[:, EV[a]]).all(), (a, b)
    assert (rows[:, EV["mma_first"]] >= rows[:, EV["dep"]]).all()
    assert (rows[:, EV["mma_last"]] >= rows[:, EV["mma_first"]]).all()
    assert (rows[:, EV["acc_ready"]] >= rows[:, EV["dep"]]).all()
    assert (rows[:, EV["stored"]] >= rows[:, EV["acc_ready"]]).all()
    if split > 1:
        assert (rows[:, EV["reduced"]] >= rows[:, EV["stored"]]).all()
    assert (rows[:, EV["exit"]] >= rows[:, EV["epi_end"]]).all()
    assert (rows[:, EV["exit_ns"]] >= rows[:, EV["entry_ns"]]).all()
    assert (rows[:, EV["smid"]] < 1024).all()


def test_trace_buffer_too_small_records_nothing_and_off_is_off():
    import torch
    h = tl.Handle()
    p, sol, A, B, C = _problem(480, 1024, 256, 0.0, 1)
    D = torch.empty(480 * 1024, dtype=torch.bfloat16, device="cuda")
    small = torch.zeros(tl.TRACE_SLOTS, dtype=torch.int64, device="cuda")   # one CTA's words: the grid has 32
    h.set_trace(small)
    h.gemm(p, D, None, A, B, solution=sol)
    h.device_status()
    assert int(small.abs().sum()) == 0
    big = torch.zeros(1024 * tl.TRACE_SLOTS, dtype=torch.int64, device="cuda")
    h.set_trace(big)
    h.set_trace(None)
    h.gemm(p, D, None, A, B, solution=sol)
    h.device_status()
    assert int(big.abs().sum()) == 0
