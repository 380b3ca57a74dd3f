"""Parity at the full sizes of the benchmark configurations, through the C ABI.

The reference checks every run in full against its CPU GEMM (GemmMfmaProblem::verifyResult,
src/gemmMfma.cpp:348-421).  Here each configuration runs at its stated size with the library's own
(heuristic) tile choice, and is checked:

* per element against the oracle's restatement of that CPU loop (oracle/tl_oracle.c,
  src/gemmMfma.cpp:313-346) on sampled column ranges (first, middle and last columns, so whole and
  ragged tiles are both covered), with the tolerance of the other GPU tests:
      |d - r| <= ulp_out(r) + 3 k 2^-24 |alpha| (|op(A)||op(B)|)_mn + 2^-23 |beta c|;
* normwise against an FP64 reference (numpy float64 on the sampled columns, or torch float64 on the
  device for whole matrices), printed and bounded.

Configurations (numpy PCG64 draws in the listed order, in fp64, then cast with RNE):
  fp16/bf16 GEMM, NN/NT/TN, 4096^3 and 480x1024x4096: seed 1, A, B, C ~ N(0,1), alpha 1, beta 0.5;
  FP8 E4M3 8192^3 TN (bf16 output) with per-tensor amax scaling: seed 2, A, B ~ N(0,1);
  grouped bf16, the 256 problems of seed 3 (M, N = 16*U{4..128}, K = 64*U{1..64}), one launch;
  Y = X W forward and dX, dW backward, X 4096x1024, W 1024x4096 ~ N(0,1)*0.02, dY ~ N(0,1), seed 4.
"""
import numpy as np
import pytest

import tensilelite_gb300 as tl
from oracle import oracle as orc
from tests import gpu_util as gu

pytestmark = pytest.mark.gpu

_DRAWS = {}


def _normal_draws(seed, m, n, k, with_c=True):
    key = (seed, m, n, k, with_c)
    if key not in _DRAWS:
        _DRAWS.clear()
        g = np.random.default_rng(seed)
        A = g.standard_normal(m * k).astype(np.float32)
        B = g.standard_normal(k * n).astype(np.float32)
        C = g.standard_normal(m * n).astype(np.float32) if with_c else None
        _DRAWS[key] = (A, B, C)
    return _DRAWS[key]


def _col_ranges(n, width=32):
    mid = max(0, n // 2 - width // 2)
    return [(0, min(width, n)), (mid, min(mid + width, n)), (max(0, n - width), n)]


def _case(dt, lay, m, n, k, seed=1, alpha=1.0, beta=0.5):
    A, B, C = _normal_draws(seed, m, n, k)
    ta, tb = lay[0] == "T", lay[1] == "T"
    Ab, Bb, Cb = orc.encode(A, dt), orc.encode(B, dt), orc.encode(C, dt)
    return dict(trans_a=ta, trans_b=tb, m=m, n=n, k=k, lda=k if ta else m, ldb=n if tb else k, ldc=m, alpha=alpha,
                beta=beta, A_bits=Ab, B_bits=Bb, C_bits=Cb, A=orc.decode(Ab, dt), B=orc.decode(Bb, dt),
                C=orc.decode(Cb, dt), out_dtype=dt)


def _fp64_sampled(case, G_cols, cols):
    """normwise error of the GPU columns against float64 products of the same operand values."""
    m, k = case["m"], case["k"]
    opA = orc.op_matrix(case["A"], case["trans_a"], m, k, case["lda"])
    errs = []
    for (c0, c1), G in zip(cols, G_cols):
        opB = orc.op_matrix(case["B"], case["trans_b"], k, case["n"], case["ldb"])[:, c0:c1]
        R = case["alpha"] * (opA @ opB)
        if case["beta"] != 0:
            R += case["beta"] * gu.mat(case["C"], m, case["n"], case["ldc"]).astype(np.float64)[:, c0:c1]
        errs.append((np.max(np.abs(G - R)), np.max(np.abs(R))))
    return max(e[0] for e in errs) / max(e[1] for e in errs)


@pytest.mark.parametrize("mnk", [(4096, 4096, 4096), (480, 1024, 4096)], ids=["4096cubed", "480x1024x4096"])
@pytest.mark.parametrize("lay", ["NN", "NT", "TN"])
@pytest.mark.parametrize("dt", ["bf16", "fp16"])
def test_half_precision_full_size(dt, lay, mnk):
    import torch
    torch.cuda.init()
    m, n, k = mnk
    case = _case(dt, lay, m, n, k)
    h = tl.Handle()
    got = gu.run_case(h, case, kernel="tcgen05", dtype=dt)
    sol = h.default_solution(tl.Problem.make(m, n, k, dtype=dt, trans_a=case["trans_a"], trans_b=case["trans_b"],
                                             beta=0.5, kernel="tcgen05"))
    h.close()
    cols = _col_ranges(n)
    G_cols = []
    for c0, c1 in cols:
        G, _ = gu.check_against_oracle(got, case, n_begin=c0, n_end=c1, threads=16)
        G_cols.append(np.asarray(G, np.float64))
    nw = _fp64_sampled(case, G_cols, cols)
    print(f"{dt} {lay} {m}x{n}x{k} tile {sol.macro_tile0}x{sol.macro_tile1} split {sol.split_k}: "
          f"normwise vs FP64 {nw:.3e}")
    assert nw < (2.0 ** -7 if dt == "bf16" else 2.0 ** -10)


def test_fp8_8192_per_tensor_scaling():
    import torch
    torch.cuda.init()
    m = n = k = 8192
    A, B, _ = _normal_draws(2, m, n, k, with_c=False)
    h = tl.Handle()
    dA32, dB32 = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    qa = torch.empty(A.size, dtype=torch.uint8, device="cuda")
    qb = torch.empty(B.size, dtype=torch.uint8, device="cuda")
    sa, sb = torch.zeros(1, device="cuda"), torch.zeros(1, device="cuda")
    h.quantize_fp8(dA32, A.size, qa, scale_out=sa)
    h.quantize_fp8(dB32, B.size, qb, scale_out=sb)
    torch.cuda.synchronize()
    del dA32, dB32
    s_a, s_b = sa.item(), sb.item()
    # TN: A stored k x m, B stored k x n (the reference's layout)
    p = tl.Problem.make(m, n, k, dtype="fp8", out_dtype="bf16", trans_a=True, lda=k, ldb=k, kernel="tcgen05",
                        scale_a=s_a, scale_b=s_b)
    D = torch.empty(m * n, dtype=torch.bfloat16, device="cuda")
    h.gemm(p, D, None, qa, qb)
    h.device_status()
    # whole-matrix FP64 error on the device: dequantised operands, float64 product
    deqA = (qa.view(torch.float8_e4m3fn).double() * s_a).view(m, k)          # row i = column i of op(A)^T
    deqB = (qb.view(torch.float8_e4m3fn).double() * s_b).view(n, k)
    R = deqB @ deqA.T                                                         # (n, m): column-major D
    Dg = D.view(n, m).double()
    nw = float((Dg - R).abs().max() / R.abs().max())
    del deqA, deqB, R, Dg
    print(f"fp8 e4m3 TN 8192^3 (scales {s_a:.3e}, {s_b:.3e}): normwise vs FP64 {nw:.3e}")
    assert nw < 2.0 ** -7
    # per element against the oracle's loop on the quantised values (alpha = scale_a * scale_b)
    qa_h, qb_h = qa.cpu().numpy(), qb.cpu().numpy()
    case = dict(trans_a=True, trans_b=False, m=m, n=n, k=k, lda=k, ldb=k, ldc=m, alpha=float(np.float32(s_a) * np.float32(s_b)),
                beta=0.0, A=orc.e4m3_to_f32(qa_h), B=orc.e4m3_to_f32(qb_h), C=None, out_dtype="bf16")
    got = gu.from_dev(D, "bf16")
    for c0, c1 in _col_ranges(n, 16):
        gu.check_against_oracle(got, case, n_begin=c0, n_end=c1, threads=16)
    h.close()


def test_grouped_256_seed3_one_launch():
    import torch
    torch.cuda.init()
    _, sizes = orc.grouped_sizes(3, 256)
    assert sizes[:3] == [(1680, 880, 3840), (224, 576, 832), (416, 1040, 1408)]
    gen = torch.Generator(device="cuda").manual_seed(3)
    probs, A, B, D = [], [], [], []
    for (m, n, k) in sizes:
        A.append(torch.randn(m * k, device="cuda", generator=gen).to(torch.bfloat16))
        B.append(torch.randn(k * n, device="cuda", generator=gen).to(torch.bfloat16))
        D.append(torch.full((m * n,), float("nan"), device="cuda", dtype=torch.bfloat16))
        probs.append(tl.Problem.make(m, n, k, dtype="bf16", kernel="tcgen05"))
    h = tl.Handle()
    l0 = h.launch_count()
    plan = h.grouped_plan(probs, D, None, A, B)
    plan.launch()
    h.device_status()
    assert h.launch_count() - l0 == 1
    worst = 0.0
    for i, (m, n, k) in enumerate(sizes):
        Ah = gu.from_dev(A[i], "bf16")
        got = gu.from_dev(D[i], "bf16")
        for c0, c1 in ((0, 4), (n - 4, n)):
            Bh = gu.from_dev(B[i][c0 * k:c1 * k], "bf16")
            case = dict(trans_a=False, trans_b=False, m=m, n=c1 - c0, k=k, lda=m, ldb=k, ldc=m, alpha=1.0, beta=0.0,
                        A=Ah, B=Bh, C=None, out_dtype="bf16")
            G, R = gu.check_against_oracle(got[c0 * m:c1 * m], case, ldd=m, threads=16)
            worst = max(worst, orc.normwise_error(G, R))
    print(f"grouped 256 problems (seed 3), 8 columns each: worst normwise vs the oracle {worst:.3e}")
    plan.close()
    h.close()


def test_fwd_bwd_4096x1024x4096_fp64_gradient():
    import torch
    torch.cuda.init()
    M, K, N = 4096, 1024, 4096
    g = np.random.default_rng(4)
    Xh = (g.standard_normal(M * K) * 0.02).astype(np.float32).reshape(M, K)
    Wh = (g.standard_normal(K * N) * 0.02).astype(np.float32).reshape(K, N)
    dYh = g.standard_normal(M * N).astype(np.float32).reshape(M, N)
    X = torch.from_numpy(Xh).cuda().to(torch.bfloat16).requires_grad_()
    W = torch.from_numpy(Wh).cuda().to(torch.bfloat16).requires_grad_()
    dY = torch.from_numpy(dYh).cuda().to(torch.bfloat16)
    Y = tl.matmul(X, W)
    Y.backward(dY)
    tl.default_handle().device_status()
    Xd, Wd, dYd = X.detach().double(), W.detach().double(), dY.double()
    errs = {}
    for name, got, ref in (("Y", Y, Xd @ Wd), ("dX", X.grad, dYd @ Wd.T), ("dW", W.grad, Xd.T @ dYd)):
        errs[name] = float((got.detach().double() - ref).abs().max() / ref.abs().max())
    print("fwd/bwd 4096x1024x4096 normwise vs FP64:", {k: f"{v:.2e}" for k, v in errs.items()})
    assert all(v < 1e-2 for v in errs.values()), errs
