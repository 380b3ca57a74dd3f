"""GPU parity: every kernel path through the C ABI against the oracle (the restated reference loop
and the FP64 oracle) on the same seeded inputs.

Tolerance (written here; both sides accumulate in fp32, in different orders):
  per element  |d - r| <= ulp_out(r) + 3 * k * 2^-24 * |alpha| * (|op(A)| |op(B)|)_mn + 2^-23 |beta c|
where r is the oracle's fp32 loop result and ulp_out the unit in the last place of the output type
(the epilogue rounds once, to nearest even).  The k * 2^-24 term is the standard bound of an fp32
dot product; any indexing, layout or pipeline error is O(1) and fails it.  In addition, the
normwise error against the oracle must be below the output type's half-ulp (2^-9 bf16, 2^-12 fp16)
plus the accumulation allowance.
"""
import math
import os

import numpy as np
import pytest

import tensilelite_gb300 as tl
from oracle import oracle as orc
from tests import gpu_util as gu
from tests.golden import gen_golden as gg

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MANT = {"fp32": 23, "fp16": 10, "bf16": 7}


@pytest.fixture(scope="module")
def h():
    import torch
    torch.cuda.init()
    os.environ.setdefault("TL_WAIT_TIMEOUT_MS", "2000")
    hd = tl.Handle()
    yield hd
    hd.close()


def fp32_tol(k):
    return 2e-6 * math.sqrt(max(k, 512) / 512.0)


ulp_out = gu.ulp_out
assert_close = gu.assert_close
absprod_of = gu.absprod_of


def check_case(h, case, dt, kernel="auto", solution=None, rounding="rne"):
    got = gu.run_case(h, case, kernel=kernel, dtype=dt, solution=solution, rounding=rounding)
    ref = gu.oracle_ref(case)
    m, n = case["m"], case["n"]
    G = gu.mat(got, m, n, case["ldc"])
    R = gu.mat(ref, m, n, m)
    od = case["out_dtype"]
    Cm = gu.mat(case["C"], m, n, case["ldc"]) if case["beta"] != 0 else None
    assert_close(G, R, absprod_of(case), case["k"], case["alpha"], case["beta"], Cm, od, rounding)
    return G, R


# ---------------------------------------------------------------------------- CUDA-core FP32 kernel
def test_simt_fp32_480x512x512_nn(h):
    """Plain FP32 GEMM, NN, 480x512x512, A/B uniform[-1,1) seed 0, alpha 1, beta 0."""
    g = orc.rng(0)
    M, N, K = 480, 512, 512
    A = orc.uniform_pm1(g, M * K).astype(np.float32)
    B = orc.uniform_pm1(g, K * N).astype(np.float32)
    case = dict(trans_a=False, trans_b=False, m=M, n=N, k=K, lda=M, ldb=K, ldc=M, alpha=1.0, beta=0.0, A_bits=A,
                B_bits=B, C_bits=np.zeros(M * N, np.float32), A=A, B=B, C=np.zeros(M * N, np.float32),
                out_dtype="fp32")
    G, R = check_case(h, case, "fp32", kernel="simt")
    D64 = gu.mat(gu.oracle_f64(case), M, N, M)
    assert orc.normwise_error(G, D64) < 1e-6


@pytest.mark.parametrize("lay", gg.LAYOUTS)
def test_simt_fp32_layouts_edges(h, lay):
    case = gg.make_case("fp32", lay, 21 + gg.LAYOUTS.index(lay), 131, 67, 45)
    check_case(h, case, "fp32", kernel="simt")


def test_simt_kat_integer_pattern_tn(h):
    """The reference's own fixture (TN, padding 64, alpha 0.314, beta 0.2718) at 768x640x256."""
    import torch
    M, N, K = 768, 640, 256
    A, B, C, lda, ldb, ldc = gg.kat_case(M, N, K, 64)
    dA, dB, dC = (torch.from_numpy(x).cuda() for x in (A, B, C))
    D = torch.zeros(ldc * N, dtype=torch.float32, device="cuda")
    p = tl.Problem.make(M, N, K, dtype="fp32", trans_a=True, alpha=float(gg.ALPHA_KAT), beta=float(gg.BETA_KAT),
                        lda=lda, ldb=ldb, ldc=ldc, ldd=ldc, kernel="simt")
    h.gemm(p, D, dC, dA, dB)
    got = gu.mat(D.cpu().numpy(), M, N, ldc)
    exp = gu.mat(gg.kat_expected(M, N, K, 64), M, N, ldc)
    # integer sums are exact on both sides; only the final alpha/beta step may differ by one ulp (fma)
    assert gu.ulp_diff_count(got, exp, "fp32") == 0


# ---------------------------------------------------------------------------- tcgen05 kernel
@pytest.mark.parametrize("dt", ["bf16", "fp16"])
@pytest.mark.parametrize("lay", ["TN", "NN", "NT", "TT"])
def test_tc_small_golden(h, dt, lay):
    """Small seeded cases; the oracle's output is also a committed golden fixture."""
    gold = np.load(os.path.join(GOLD, "gemm_small.npz"))
    seed = 1000 + gg.DTYPES.index(dt) * 10 + gg.LAYOUTS.index(lay)
    case = gg.make_case(dt, lay, seed, **gg.SMALL)
    assert np.array_equal(gu.oracle_ref(case).view(np.uint32), gold[f"{dt}_{lay}"])
    check_case(h, case, dt, kernel="tcgen05")


@pytest.mark.parametrize("dt", ["bf16", "fp16"])
@pytest.mark.parametrize("lay", ["TN", "NN", "NT", "TT"])
@pytest.mark.parametrize("mnk", [(256, 384, 320), (130, 200, 72), (480, 1024, 256), (64, 64, 64), (1, 1, 64),
                                 (300, 129, 1000)])
def test_tc_layouts_sizes(h, dt, lay, mnk):
    m, n, k = mnk
    seed = 7 + m + 3 * n + k
    case = gg.make_case(dt, lay, seed, m, n, k, ld_align=8)    # TMA: leading dims in 16-byte units
    check_case(h, case, dt, kernel="tcgen05")


@pytest.mark.parametrize("bm", [64, 128, 192, 256])
@pytest.mark.parametrize("stages", [2, 4])
@pytest.mark.parametrize("split", [1, 3])
def test_tc_solutions(h, bm, stages, split):
    case = gg.make_case("bf16", "NN", 99, 333, 300, 640, ld_align=8)
    sol = tl.Solution(kernel=tl.KERNEL_TCGEN05, macro_tile0=bm, macro_tile1=128, depth_u=64, stages=stages,
                      split_k=split, raster=4)
    check_case(h, case, "bf16", kernel="tcgen05", solution=sol)


@pytest.mark.parametrize("dt", ["bf16", "fp16", "fp8"])
@pytest.mark.parametrize("lay", ["TN", "NN", "NT", "TT"])
@pytest.mark.parametrize("bm,split", [(256, 1), (128, 1), (256, 3)])
def test_tc_cta_pair(h, dt, lay, bm, split):
    """macro_tile1 = 256: a cluster of two CTAs per 256-row tile (tcgen05 cta_group::2)."""
    if dt == "fp8" and lay[0] == "N" and bm == 128:
        pytest.skip("MN-major fp8 A needs 128 m rows per CTA")
    m, n, k = 520, 600, 704
    case = gg.make_case(dt, lay, 300 + bm + split, m, n, k, ld_align=16)
    sol = tl.Solution(kernel=tl.KERNEL_TCGEN05, macro_tile0=bm, macro_tile1=256,
                      depth_u=128 if dt == "fp8" else 64, stages=4, split_k=split)
    check_case(h, case, dt, kernel="tcgen05", solution=sol)


def test_tc_cta_pair_promoted_bf16x6(h):
    """The FP32-accurate path on a CTA pair with promotion (bm 128)."""
    import torch
    M, N, K = 512, 640, 2048
    g = orc.rng(9)
    A = orc.uniform_pm1(g, M * K).astype(np.float32)
    B = orc.uniform_pm1(g, K * N).astype(np.float32)
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    D = torch.empty(M * N, dtype=torch.float32, device="cuda")
    sol = tl.Solution(kernel=tl.KERNEL_BF16X6, macro_tile0=128, macro_tile1=256, depth_u=64, stages=4,
                      split_k=1, promote_k=256)
    h.gemm(tl.Problem.make(M, N, K, dtype="fp32", kernel="bf16x6"), D, None, dA, dB, solution=sol)
    ref = A.reshape(K, M).T.astype(np.float64) @ B.reshape(N, K).T.astype(np.float64)
    got = D.cpu().numpy().reshape(N, M).T
    assert orc.normwise_error(got, ref) < 1e-6


def test_grouped_cta_pair(h):
    probs, cases, D, C, A, B = _grouped_setup(16, 13)
    sol = tl.Solution(kernel=tl.KERNEL_TCGEN05, macro_tile0=256, macro_tile1=256, depth_u=64, stages=6)
    plan = h.grouped_plan(probs, D, C, A, B, solution=sol)
    plan.launch()
    h.device_status()
    _check_grouped(cases, D)
    plan.close()


@pytest.mark.parametrize("cg,bm", [(1, 256), (2, 256), (1, 128), (4, 256)])
def test_tail_split_last_wave(h, cg, bm):
    """More tiles than persistent workers with a small remainder: the last wave's k-blocks are
    spread evenly over all workers (auto tail_split: balanced pieces, one or two per worker) or its
    tiles cut into 3 equal k-slices (tail_split 3), and reduced through the workspace."""
    m, n, k = 1024, 5120, 1024
    case = gg.make_case("bf16", "NN", 500 + cg + bm, m, n, k)
    sol = tl.Solution(kernel=tl.KERNEL_TCGEN05, macro_tile0=bm, macro_tile1=128 * cg, depth_u=64,
                      stages=4, split_k=1, tail_split=0)
    check_case(h, case, "bf16", kernel="tcgen05", solution=sol)
    sol.tail_split = 3
    check_case(h, case, "bf16", kernel="tcgen05", solution=sol)
    sol.tail_split = -1
    check_case(h, case, "bf16", kernel="tcgen05", solution=sol)


@pytest.mark.parametrize("cg,bm,split", [(1, 128, 3), (2, 256, 2), (1, 64, 4)])
def test_split_k_reductions(h, cg, bm, split):
    """Explicit split-k with few units (all resident: the splits of a tile reduce one share each in
    parallel) and with many (more units than workers: the last split to arrive reduces the tile);
    both sum in split order."""
    for (m, n, k) in ((480, 1024, 2048), (2048, 2048, 512)):
        case = gg.make_case("bf16", "NN", 700 + cg + bm + split + m % 7, m, n, k, alpha=1.25, beta=0.5)
        sol = tl.Solution(kernel=tl.KERNEL_TCGEN05, macro_tile0=bm, macro_tile1=128 * cg, depth_u=64,
                          stages=4, split_k=split)
        check_case(h, case, "bf16", kernel="tcgen05", solution=sol)


@pytest.mark.parametrize("od", ["bf16", "fp16", "fp32"])
@pytest.mark.parametrize("m,n,k", [(1000, 600, 2048), (2048, 2048, 4096), (4096, 264, 2048)])
def test_nn_runs_transposed(h, od, m, n, k):
    """NN with beta = 0 and k >= 2048 runs as the transposed TT product with a transposed store
    (32 x 32 TMA boxes; ragged edges; 2048^2 leaves a partial wave, whose balanced split finishes
    its tiles element by element).  Every output type against the oracle."""
    dt = "fp16" if od == "fp16" else "bf16"
    case = gg.make_case(dt, "NN", 1500 + m + n, m, n, k, alpha=1.5, beta=0.0, ld_align=8)
    got = gu.run_case(h, case, kernel="tcgen05", dtype=dt, out_dtype=od)
    G = gu.mat(got, m, n, case["ldc"])
    R = gu.mat(gu.oracle_ref(case), m, n, m)
    assert_close(G, R, absprod_of(case), k, case["alpha"], 0.0, None, od)


@pytest.mark.parametrize("od", ["bf16", "fp16", "fp32"])
@pytest.mark.parametrize("m", [480, 479])
def test_parallel_split_k_c_staging(h, od, m):
    """Parallel split-k with beta: a split copies the C rows of the chunk it finishes into shared
    memory while the tile accumulates, when the row segment is whole and 16-byte aligned, else it
    reads C at the end.  m = 479 (odd leading dimension of C and D, ragged last m-tile) mixes both
    in one launch; every output type."""
    dt = "fp16" if od == "fp16" else "bf16"
    case = gg.make_case(dt, "NN", 1300 + m, m, 1024, 2048, alpha=1.25, beta=0.5, ld_align=8)
    sol = tl.Solution(kernel=tl.KERNEL_TCGEN05, macro_tile0=128, macro_tile1=128, depth_u=64, stages=4,
                      split_k=4)
    got = gu.run_case(h, case, kernel="tcgen05", dtype=dt, out_dtype=od, solution=sol)
    n, k = case["n"], case["k"]
    G = gu.mat(got, m, n, case["ldc"])
    R = gu.mat(gu.oracle_ref(case), m, n, m)
    assert_close(G, R, absprod_of(case), k, case["alpha"], case["beta"], gu.mat(case["C"], m, n, case["ldc"]), od)


@pytest.mark.parametrize("cg,bm", [(1, 256), (2, 256), (4, 256), (2, 128)])
@pytest.mark.parametrize("m,n,k", [(256, 512, 8192), (1000, 3008, 1344), (2048, 4608, 576)])
def test_balanced_split_shapes(h, cg, bm, m, n, k):
    """Balanced split of a partial wave at shapes where the pieces straddle tile boundaries, where
    no whole wave follows (single partial wave, long k) and with ragged edges; C and beta on."""
    case = gg.make_case("bf16", "NN", 900 + cg + bm + m % 97, m, n, k, alpha=0.75, beta=0.5, ld_align=8)
    for tail in (0, -1):        # automatic, and the balanced split forced on
        sol = tl.Solution(kernel=tl.KERNEL_TCGEN05, macro_tile0=bm, macro_tile1=128 * cg, depth_u=64,
                          stages=4, split_k=1, tail_split=tail)
        check_case(h, case, "bf16", kernel="tcgen05", solution=sol)


def test_tc_fp32_output_and_truncation(h):
    case = gg.make_case("bf16", "TN", 5, 200, 160, 512)
    got = gu.run_case(h, case, kernel="tcgen05", dtype="bf16", out_dtype="fp32")
    # fp32 output of a bf16 GEMM: the oracle's fp32 loop on the same exact inputs, per-element bound
    assert_close(gu.mat(got, 200, 160, 200), gu.mat(gu.oracle_ref(case), 200, 160, 200), absprod_of(case), 512,
                 1.0, 0.5, gu.mat(case["C"], 200, 160, 200), "fp32")
    # reference bf16 store mode: truncation (src/gemmMfmaKernelWriter.h:1661-1665)
    check_case(h, case, "bf16", kernel="tcgen05", rounding="trunc")


def test_tc_batched(h):
    import torch
    m, n, k, batch = 96, 130, 192, 3
    g = np.random.default_rng(17)
    A = orc.encode(g.standard_normal(m * k * batch).astype(np.float32), "bf16")
    B = orc.encode(g.standard_normal(k * n * batch).astype(np.float32), "bf16")
    C = orc.encode(g.standard_normal(m * n * batch).astype(np.float32), "bf16")
    Af, Bf, Cf = (orc.decode(x, "bf16") for x in (A, B, C))
    dA, dB, dC = gu.to_dev(A, "bf16"), gu.to_dev(B, "bf16"), gu.to_dev(C, "bf16")
    dD = torch.empty(m * n * batch, dtype=torch.bfloat16, device="cuda")
    p = tl.Problem.make(m, n, k, dtype="bf16", alpha=1.5, beta=-0.5, batch=batch, kernel="tcgen05")
    h.gemm(p, dD, dC, dA, dB)
    got = gu.from_dev(dD, "bf16")
    ref = orc.gemm_ref_f32(0, 0, m, n, k, 1.5, Af, m, Bf, k, -0.5, Cf, m, m, batch=batch, stride_a=m * k,
                           stride_b=k * n, stride_c=m * n, stride_d=m * n)
    for b in range(batch):
        sl = slice(b * m * n, (b + 1) * m * n)
        ap = np.abs(Af[b * m * k:(b + 1) * m * k].reshape(k, m).T.astype(np.float64)) @ \
            np.abs(Bf[b * k * n:(b + 1) * k * n].reshape(n, k).T.astype(np.float64))
        assert_close(gu.mat(got[sl], m, n, m), gu.mat(ref[sl], m, n, m), ap, k, 1.5, -0.5,
                     gu.mat(Cf[sl], m, n, m), "bf16")


def test_tc_in_place_beta_and_k0(h):
    import torch
    case = gg.make_case("fp16", "TN", 3, 128, 128, 128)
    C = gu.to_dev(case["C_bits"], "fp16")
    D = C.clone()
    p = tl.Problem.make(128, 128, 128, dtype="fp16", trans_a=True, alpha=1.0, beta=0.5, kernel="tcgen05")
    A, B = gu.to_dev(case["A_bits"], "fp16"), gu.to_dev(case["B_bits"], "fp16")
    h.gemm(p, D, D, A, B)        # D == C in place
    assert_close(gu.mat(gu.from_dev(D, "fp16"), 128, 128, 128), gu.mat(gu.oracle_ref(case), 128, 128, 128),
                 absprod_of(case), 128, 1.0, 0.5, gu.mat(case["C"], 128, 128, 128), "fp16")
    # k == 0: D = beta * C
    p0 = tl.Problem.make(128, 128, 0, dtype="fp16", trans_a=True, alpha=1.0, beta=0.5, lda=1, kernel="tcgen05")
    D0 = torch.empty_like(C)
    h.gemm(p0, D0, C, A, B)
    exp = gu.quantize_out(0.5 * case["C"], "fp16")
    assert np.array_equal(gu.from_dev(D0, "fp16"), exp)


def test_unaligned_ld_falls_back_to_simt(h):
    """lda*2 bytes not a multiple of 16: TMA cannot describe it; AUTO routes to the CUDA-core kernel,
    an explicit TCGEN05 request is refused."""
    case = gg.make_case("bf16", "NN", 4, 61, 33, 47)      # lda = 61, ldb = 47
    check_case(h, case, "bf16", kernel="auto")
    with pytest.raises(tl.TLError) as e:
        gu.run_case(h, case, kernel="tcgen05", dtype="bf16")
    assert e.value.status == tl.ERR_UNSUPPORTED


# ---------------------------------------------------------------------------- bf16x3 and fp8
def _fp32_paths_errors(h, M, N, K, cols):
    """Errors of the three fp32 paths against FP64 on `cols` output columns of an M x N x K NN GEMM
    with A, B uniform[-1,1) (seed 2)."""
    import torch
    g = orc.rng(2)
    A = orc.uniform_pm1(g, M * K).astype(np.float32)
    B = orc.uniform_pm1(g, K * N).astype(np.float32)
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    sel = np.sort(np.random.default_rng(0).choice(N, cols, replace=False))
    opA = A.reshape(K, M).T.astype(np.float64)
    opB = B.reshape(N, K)[sel].T.astype(np.float64)
    ref = opA @ opB
    absprod = np.abs(opA) @ np.abs(opB)
    errs = {}
    for kern in ("bf16x6", "bf16x3", "simt"):
        D = torch.empty(M * N, dtype=torch.float32, device="cuda")
        h.gemm(tl.Problem.make(M, N, K, dtype="fp32", kernel=kern), D, None, dA, dB)
        got = D.cpu().numpy().reshape(N, M)[sel].T
        errs[kern] = (orc.normwise_error(got, ref), orc.componentwise_error(got, ref, absprod))
    return errs


def test_fp32_accurate_paths_1024(h):
    errs = _fp32_paths_errors(h, 1024, 1024, 1024, 256)
    print("fp32 paths 1024^3 (normwise, componentwise):", errs)
    assert errs["bf16x6"][0] < 1e-6
    assert errs["bf16x3"][0] < 6e-6          # two-piece split: products good to ~2^-17
    assert errs["simt"][0] < 4e-6
    assert all(e[1] < 2e-6 for e in errs.values())


@pytest.mark.parametrize("promote,split", [(256, 1), (128, 1), (256, 2), (64, 3)])
def test_promotion_chains(h, promote, split):
    """bf16 inputs, fp32 output, the dominant product promoted out of TMEM every `promote` k."""
    import torch
    M, N, K = 256, 384, 2048
    case = gg.make_case("bf16", "NN", 71, M, N, K)
    sol = tl.Solution(kernel=tl.KERNEL_TCGEN05, macro_tile0=128, macro_tile1=128, depth_u=64, stages=4,
                      split_k=split, promote_k=promote)
    got = gu.run_case(h, case, kernel="tcgen05", dtype="bf16", out_dtype="fp32", solution=sol)
    ref = gu.mat(gu.oracle_f64(case), M, N, M)
    G = gu.mat(got, M, N, M)
    assert_close(G, gu.mat(gu.oracle_ref(case), M, N, M), absprod_of(case), K, 1.0, 0.5,
                 gu.mat(case["C"], M, N, M), "fp32")
    assert orc.normwise_error(G, ref) < 1e-6


def test_fp32_accurate_paths_8192(h):
    """The FP32-accurate configuration: 8192^3 NN, checked on 128 output columns against FP64."""
    errs = _fp32_paths_errors(h, 8192, 8192, 8192, 128)
    print("fp32 paths 8192^3 (normwise, componentwise):", errs)
    assert errs["bf16x6"][0] <= 1e-6
    assert errs["bf16x6"][0] < errs["simt"][0]


def test_split_bf16_pieces_exact(h):
    import torch
    g = np.random.default_rng(8)
    x = (g.standard_normal(10001) * 10).astype(np.float32)
    dx = torch.from_numpy(x).cuda()
    hi = torch.empty(x.size, dtype=torch.bfloat16, device="cuda")
    lo = torch.empty_like(hi)
    h.split_bf16x2(dx, x.size, hi, lo)
    hb = gu.from_dev(hi, "bf16")
    lb = gu.from_dev(lo, "bf16")
    assert np.array_equal(hb, orc.decode(orc.f32_to_bf16(x), "bf16"))
    assert np.array_equal(lb, orc.decode(orc.f32_to_bf16(x - hb), "bf16"))


def test_fp8_quantize_bit_exact(h):
    import torch
    g = np.random.default_rng(12)
    x = g.standard_normal(50000).astype(np.float32)
    dx = torch.from_numpy(x).cuda()
    q = torch.empty(x.size, dtype=torch.uint8, device="cuda")
    scale = torch.zeros(1, dtype=torch.float32, device="cuda")
    amax = torch.zeros(1, dtype=torch.float32, device="cuda")
    h.quantize_fp8(dx, x.size, q, scale_out=scale, amax_out=amax)
    a = np.float32(np.max(np.abs(x)))
    s = np.float32(448.0) / a
    assert amax.item() == a
    assert scale.item() == np.float32(a / np.float32(448.0))
    assert np.array_equal(q.cpu().numpy(), orc.f32_to_e4m3((x * s).astype(np.float32)))


@pytest.mark.parametrize("lay", ["TN", "NN", "NT", "TT"])
def test_fp8_gemm(h, lay):
    case = gg.make_case("fp8", lay, 31 + gg.LAYOUTS.index(lay), 256, 200, 384, ld_align=16)
    check_case(h, case, "fp8", kernel="tcgen05")
    # with dequantisation scales folded into alpha
    got = gu.run_case(h, case, kernel="tcgen05", dtype="fp8", scale_a=0.5, scale_b=0.25)
    c2 = dict(case)
    c2["alpha"] = case["alpha"] * 0.125
    m, n = case["m"], case["n"]
    assert_close(gu.mat(got, m, n, m), gu.mat(gu.oracle_ref(c2), m, n, m), absprod_of(case), case["k"],
                 c2["alpha"], case["beta"], gu.mat(case["C"], m, n, m), "bf16")


# ---------------------------------------------------------------------------- grouped + graphs
def _grouped_setup(count, seed, dt="bf16", lay="NN"):
    import torch
    g = np.random.default_rng(seed)
    probs, cases, D, C, A, B = [], [], [], [], [], []
    for i in range(count):
        m = int(16 * g.integers(1, 20))
        n = int(16 * g.integers(1, 20))
        k = int(64 * g.integers(1, 8))
        case = gg.make_case(dt, lay, seed * 1000 + i, m, n, k, alpha=1.0, beta=0.5 if i % 2 else 0.0)
        cases.append(case)
        A.append(gu.to_dev(case["A_bits"], dt))
        B.append(gu.to_dev(case["B_bits"], dt))
        C.append(gu.to_dev(case["C_bits"], case["out_dtype"]))
        D.append(torch.full((m * n,), float("nan"), dtype=gu.torch_dtype(case["out_dtype"]), device="cuda"))
        probs.append(tl.Problem.make(m, n, k, dtype=dt, out_dtype=case["out_dtype"], trans_a=case["trans_a"],
                                     trans_b=case["trans_b"], alpha=case["alpha"], beta=case["beta"], lda=case["lda"],
                                     ldb=case["ldb"], ldc=m, ldd=m, kernel="tcgen05"))
    return probs, cases, D, C, A, B


def _check_grouped(cases, D):
    for case, d in zip(cases, D):
        m, n = case["m"], case["n"]
        got = gu.mat(gu.from_dev(d, case["out_dtype"]), m, n, m)
        Cm = gu.mat(case["C"], m, n, m) if case["beta"] != 0 else None
        assert_close(got, gu.mat(gu.oracle_ref(case), m, n, m), absprod_of(case), case["k"], case["alpha"],
                     case["beta"], Cm, case["out_dtype"])


@pytest.mark.parametrize("lay", ["NN", "TN"])
def test_grouped_one_launch(h, lay):
    probs, cases, D, C, A, B = _grouped_setup(24, 5, lay=lay)
    n0 = h.launch_count()
    plan = h.grouped_plan(probs, D, C, A, B)
    plan.launch()
    h.device_status()
    assert h.launch_count() - n0 == 1
    _check_grouped(cases, D)
    plan.close()


def test_grouped_graph_replay(h):
    import torch
    probs, cases, D, C, A, B = _grouped_setup(12, 9)
    plan = h.grouped_plan(probs, D, C, A, B)
    s = torch.cuda.Stream()
    graph = plan.capture(s)
    for d in D:
        d.fill_(float("nan"))
    torch.cuda.synchronize()
    graph.launch(s)
    graph.launch(s)
    s.synchronize()
    h.device_status()
    _check_grouped(cases, D)
    graph.close()
    plan.close()


def test_gemm_graph_capture(h):
    import torch
    case = gg.make_case("bf16", "NT", 77, 512, 256, 512)
    A, B = gu.to_dev(case["A_bits"], "bf16"), gu.to_dev(case["B_bits"], "bf16")
    C = gu.to_dev(case["C_bits"], "bf16")
    D = torch.empty(512 * 256, dtype=torch.bfloat16, device="cuda")
    p = tl.Problem.make(512, 256, 512, dtype="bf16", trans_b=True, alpha=1.0, beta=0.5, lda=case["lda"],
                        ldb=case["ldb"], kernel="tcgen05")
    s = torch.cuda.Stream()
    graph = h.capture_gemm(p, D, C, A, B, stream=s)
    graph.launch(s)
    s.synchronize()
    assert_close(gu.mat(gu.from_dev(D, "bf16"), 512, 256, 512), gu.mat(gu.oracle_ref(case), 512, 256, 512),
                 absprod_of(case), 512, 1.0, 0.5, gu.mat(case["C"], 512, 256, 512), "bf16")
    graph.close()


def _split_case(seed, m, n, k):
    import torch
    case = gg.make_case("bf16", "NN", seed, m, n, k, alpha=1.0, beta=0.0)
    A, B = gu.to_dev(case["A_bits"], "bf16"), gu.to_dev(case["B_bits"], "bf16")
    D = torch.empty(m * n, dtype=torch.bfloat16, device="cuda")
    p = tl.Problem.make(m, n, k, dtype="bf16", lda=case["lda"], ldb=case["ldb"], kernel="tcgen05")
    return case, A, B, D, p


def test_graph_survives_workspace_growth():
    """A captured split-k GEMM keeps its workspace after a larger problem grows the handle's buffer."""
    import torch
    h = tl.Handle()
    sol = tl.Solution(kernel=tl.KERNEL_TCGEN05, macro_tile0=128, macro_tile1=128, depth_u=64, stages=4, split_k=2)
    case, A, B, D, p = _split_case(91, 256, 256, 1024)
    s = torch.cuda.Stream()
    graph = h.capture_gemm(p, D, None, A, B, solution=sol, stream=s)
    # a bigger split-k problem grows the workspace (the captured buffer is retired, not freed)
    big, A2, B2, D2, p2 = _split_case(92, 1024, 1024, 2048)
    sol2 = tl.Solution(kernel=tl.KERNEL_TCGEN05, macro_tile0=128, macro_tile1=128, depth_u=64, stages=4, split_k=8)
    h.gemm(p2, D2, None, A2, B2, solution=sol2, stream=s)
    D.fill_(float("nan"))
    graph.launch(s)
    s.synchronize()
    h.device_status(s)
    assert_close(gu.mat(gu.from_dev(D, "bf16"), 256, 256, 256), gu.mat(gu.oracle_ref(case), 256, 256, 256),
                 absprod_of(case), 1024, 1.0, 0.0, None, "bf16")
    assert_close(gu.mat(gu.from_dev(D2, "bf16"), 1024, 1024, 1024), gu.mat(gu.oracle_ref(big), 1024, 1024, 1024),
                 absprod_of(big), 2048, 1.0, 0.0, None, "bf16")
    graph.close()
    h.close()


def test_capture_refuses_workspace_growth():
    """Inside a stream capture a problem whose workspace is not yet allocated fails with a clear error
    (an allocation is not capturable); after one eager call the same problem captures."""
    import torch
    h = tl.Handle()
    sol = tl.Solution(kernel=tl.KERNEL_TCGEN05, macro_tile0=128, macro_tile1=128, depth_u=64, stages=4, split_k=4)
    case, A, B, D, p = _split_case(93, 512, 512, 2048)
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with pytest.raises(tl.TLError) as ei:
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                h.gemm(p, D, None, A, B, solution=sol, stream=s)
    assert ei.value.status == tl.ERR_UNSUPPORTED
    assert b"stream capture" in tl.lib().tl_last_error_string()
    torch.cuda.synchronize()
    h.gemm(p, D, None, A, B, solution=sol, stream=s)       # sizes the workspace
    g2 = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g2, stream=s):
            h.gemm(p, D, None, A, B, solution=sol, stream=s)
    D.fill_(float("nan"))
    g2.replay()
    torch.cuda.synchronize()
    h.device_status()
    assert_close(gu.mat(gu.from_dev(D, "bf16"), 512, 512, 512), gu.mat(gu.oracle_ref(case), 512, 512, 512),
                 absprod_of(case), 2048, 1.0, 0.0, None, "bf16")
    h.close()


def test_kernel_timing_counts_gemm_launches():
    """tl_kernel_timing: one event pair per GEMM kernel (not the split pre-pass); the summed kernel
    time lies inside the stream time around the same launches."""
    import torch
    h = tl.Handle()
    case, A, B, D, p = _split_case(94, 1024, 1024, 1024)
    s = torch.cuda.Stream()
    h.gemm(p, D, None, A, B, stream=s)
    h.set_kernel_timing(True)
    h.kernel_timing(reset=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(5):
        h.gemm(p, D, None, A, B, stream=s)
    e1.record(s)
    ms, n = h.kernel_timing(reset=True)
    assert n == 5
    assert 0 < ms <= e0.elapsed_time(e1) * 1.01 + 0.01
    # fp32 operands on the split path: 2 split launches + 1 GEMM per call, only the GEMM is timed
    Af = torch.randn(512 * 512, device="cuda")
    Bf = torch.randn(512 * 512, device="cuda")
    Df = torch.empty(512 * 512, device="cuda")
    pf = tl.Problem.make(512, 512, 512, dtype="fp32", kernel="bf16x3")
    l0 = h.launch_count()
    h.gemm(pf, Df, None, Af, Bf, stream=s)
    assert h.launch_count() - l0 == 3
    ms, n = h.kernel_timing(reset=True)
    assert n == 1 and ms > 0
    h.set_kernel_timing(False)
    h.gemm(p, D, None, A, B, stream=s)
    assert h.kernel_timing()[1] == 0
    h.close()


# ---------------------------------------------------------------------------- tuner, norms, autograd
def test_tune_and_cache(h, tmp_path):
    import torch
    case = gg.make_case("bf16", "NN", 55, 480, 1024, 1024)
    A, B = gu.to_dev(case["A_bits"], "bf16"), gu.to_dev(case["B_bits"], "bf16")
    D = torch.empty(480 * 1024, dtype=torch.bfloat16, device="cuda")
    p = tl.Problem.make(480, 1024, 1024, dtype="bf16", kernel="tcgen05")
    path = str(tmp_path / "tuned.json")
    sol, ms = h.tune(p, D, None, A, B, max_candidates=6, reps=3, cache_path=path)
    assert ms > 0
    h.check_solution(p, sol)
    h2 = tl.Handle()
    assert h2.load_solutions(path) == 1
    c = dict(case)
    c["beta"] = 0.0
    check_case(h2, c, "bf16", kernel="tcgen05")
    h2.close()


def test_error_norms_device(h):
    import torch
    g = np.random.default_rng(1)
    m, n = 300, 200
    R = g.standard_normal(m * n)
    Dv = (R + g.standard_normal(m * n) * 1e-3).astype(np.float32)
    W = np.abs(g.standard_normal(m * n)) + 0.5
    out = h.error_norms(tl.FP32, torch.from_numpy(Dv).cuda(), m, torch.from_numpy(R).cuda(), m, m, n,
                        W=torch.from_numpy(W).cuda())
    diff = np.abs(Dv.astype(np.float64) - R)
    assert out[0] == pytest.approx(diff.max(), rel=0, abs=0)
    assert out[1] == pytest.approx(np.abs(R).max(), rel=0, abs=0)
    assert out[2] == pytest.approx((diff / W).max(), rel=1e-15)


def test_autograd_finite_differences_fp64():
    """Y = X W at M=64, K=48, N=32 (bf16 kernels); gradients vs central differences of the fp64
    function, relative error below 1e-2."""
    import torch
    g = torch.Generator().manual_seed(4)
    M, K, N = 64, 48, 32
    X64 = torch.randn(M, K, generator=g, dtype=torch.float64) * 0.02 * 50
    W64 = torch.randn(K, N, generator=g, dtype=torch.float64) * 0.02 * 50
    dY = torch.randn(M, N, generator=g, dtype=torch.float64)
    Xb = X64.to(torch.bfloat16).cuda().requires_grad_()
    Wb = W64.to(torch.bfloat16).cuda().requires_grad_()
    Y = tl.matmul(Xb, Wb)
    Y.backward(dY.to(torch.bfloat16).cuda())
    Xe, We = Xb.detach().double().cpu(), Wb.detach().double().cpu()
    dYe = dY.to(torch.bfloat16).double()

    def loss(X, W):
        return float((X @ W * dYe).sum())

    eps = 1e-3
    for name, T, grad in (("X", Xe, Xb.grad), ("W", We, Wb.grad)):
        gnum = torch.zeros_like(T)
        for i in range(T.shape[0]):
            for j in range(T.shape[1]):
                Tp, Tm = T.clone(), T.clone()
                Tp[i, j] += eps
                Tm[i, j] -= eps
                gnum[i, j] = (loss(Tp, We) - loss(Tm, We)) / (2 * eps) if name == "X" else \
                    (loss(Xe, Tp) - loss(Xe, Tm)) / (2 * eps)
        ga = grad.double().cpu()
        rel = float((ga - gnum).abs().max() / gnum.abs().max())
        assert rel < 1e-2, (name, rel)


def test_autograd_layouts_match_fp64_gradient():
    import torch
    g = torch.Generator().manual_seed(4)
    M, K, N = 512, 256, 384
    X = (torch.randn(M, K, generator=g) * 0.02).to(torch.bfloat16).cuda().requires_grad_()
    W = (torch.randn(K, N, generator=g) * 0.02).to(torch.bfloat16).cuda().requires_grad_()
    dY = torch.randn(M, N, generator=g).to(torch.bfloat16).cuda()
    Y = tl.matmul(X, W)
    Y.backward(dY)
    Xd, Wd, dYd = X.detach().double(), W.detach().double(), dY.double()
    for got, ref in ((Y, Xd @ Wd), (X.grad, dYd @ Wd.T), (W.grad, Xd.T @ dYd)):
        rel = float((got.double() - ref).abs().max() / ref.abs().max())
        assert rel < 1e-2


# ---------------------------------------------------------------------------- Tensile layout, CLI
@pytest.mark.parametrize("dt,name", [("fp32", "Cijk_Alik_Bljk_SB"), ("fp16", "Cijk_Alik_Bljk_HBH_MT64x64x16"),
                                     ("bf16", "Cijk_Alik_Bljk_BBH")])
def test_tensile_layout_launch_matches_gemm(h, dt, name):
    """tl_tensile_launch decodes the reference's Tensile-layout argument buffer (padded TN problem,
    batch 2) into the same GEMM tl_gemm runs: bit-equal outputs; bad names, short buffers and
    declared sizes the strides overrun are refused."""
    import torch
    m, n, k, batch, pad = 192, 160, 256, 2, 64
    lda = ldb = k + pad
    ldc = ldd = m + pad
    sa, sb, sc, sd = lda * m, ldb * n, ldc * n, ldd * n
    tdt = {"fp32": torch.float32, "fp16": torch.float16, "bf16": torch.bfloat16}[dt]
    gen = torch.Generator(device="cuda").manual_seed(61)
    A = torch.randn(sa * batch, device="cuda", generator=gen).to(tdt)
    B = torch.randn(sb * batch, device="cuda", generator=gen).to(tdt)
    C = torch.randn(sc * batch, device="cuda", generator=gen).to(tdt)
    D1 = torch.full((sd * batch,), float("nan"), device="cuda", dtype=tdt)
    D2 = D1.clone()
    alpha, beta = 0.314, 0.2718
    if dt == "fp16":         # the HBH kernel takes fp16 scalars
        alpha, beta = float(np.float16(alpha)), float(np.float16(beta))
    p = tl.Problem.make(m, n, k, dtype=dt, trans_a=True, alpha=alpha, beta=beta, lda=lda, ldb=ldb, ldc=ldc, ldd=ldd,
                        batch=batch, stride_a=sa, stride_b=sb, stride_c=sc, stride_d=sd,
                        rounding="trunc" if dt == "bf16" else "rne")
    h.gemm(p, D1, C, A, B)
    kw = dict(batch=batch, alpha=alpha, beta=beta, half_scalars=dt == "fp16", stride_d0=ldd, stride_d1=sd,
              stride_c0=ldc, stride_c1=sc, stride_a0=lda, stride_a1=sa, stride_b0=ldb, stride_b1=sb)
    buf = tl.tensile_kernarg(D2, C, A, B, m, n, k, size_c=sc * batch, size_a=sa * batch, size_b=sb * batch, **kw)
    h.tensile_launch(name, buf)
    torch.cuda.synchronize()
    h.device_status()
    view = torch.int32 if dt == "fp32" else torch.int16
    assert torch.equal(D1.view(view), D2.view(view))
    # and against the oracle's restated reference loop, batch by batch (bf16 stores truncate, as the
    # reference's BBH kernel does)
    rounding = "trunc" if dt == "bf16" else "rne"
    Af, Bf, Cf = (gu.from_dev(x, dt) for x in (A, B, C))
    got = gu.from_dev(D2, dt)
    for b in range(batch):
        case = dict(trans_a=True, trans_b=False, m=m, n=n, k=k, lda=lda, ldb=ldb, ldc=ldc, alpha=alpha, beta=beta,
                    A=Af[b * sa:(b + 1) * sa], B=Bf[b * sb:(b + 1) * sb], C=Cf[b * sc:(b + 1) * sc], out_dtype=dt)
        gu.check_against_oracle(got[b * sd:(b + 1) * sd], case, ldd=ldd, rounding=rounding)
    with pytest.raises(tl.TLError) as e:
        h.tensile_launch("Cijk_Ailk_Bljk_SB", buf)
    assert e.value.status == tl.ERR_UNSUPPORTED
    with pytest.raises(tl.TLError) as e:
        h.tensile_launch(name, buf[:120])
    assert e.value.status == tl.ERR_INVALID_ARG
    small = tl.tensile_kernarg(D2, C, A, B, m, n, k, size_c=sc * batch, size_a=sa, size_b=sb * batch, **kw)
    with pytest.raises(tl.TLError) as e:
        h.tensile_launch(name, small)
    assert e.value.status == tl.ERR_INVALID_ARG


_CLI_CASES = [
    ["-d", "1", "-m", "256", "-n", "192", "-k", "128", "-l", "3"],
    ["-d", "2", "-m", "384", "-n", "256", "-k", "192", "-l", "3"],
    ["-d", "3", "-m", "512", "-n", "512", "-k", "256", "-l", "3", "-z", "32", "-r", "4", "-x", "2", "-s", "4",
     "-y", "1", "-f", "4"],
    ["-d", "3", "-m", "256", "-n", "256", "-k", "128", "-l", "3", "-t", "1"],
    ["--data-type", "2", "--gemm-m", "128", "--gemm-n", "128", "--gemm-k", "64", "--loop", "2", "-b", "2"],
]


@pytest.mark.parametrize("args", _CLI_CASES)
def test_cli_runs_and_verifies(args):
    """The command-line runner with the reference's options: runs, verifies against the CUDA-core
    kernel (integer-pattern data, exact), prints the performance summary."""
    import subprocess
    cli = os.path.join(ROOT, "tensilelite_gb300", "tensilelite")
    if not os.path.exists(cli):
        pytest.skip("CLI not built")
    out = subprocess.run([cli] + args, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "Performance =" in out.stdout
    if "-t" not in args:
        assert "Verify Success" in out.stdout, out.stdout


# ---------------------------------------------------------------------------- device data init
@pytest.mark.parametrize("dt", ["fp32", "fp16", "bf16", "fp8"])
def test_fill_pattern_matches_init_real_data(h, dt):
    """tl_fill_pattern (device) against the oracle's InitRealData (ff_gpu_src/ff_gpu.cpp:110-148),
    bit for bit: every flat-index code, converted to the buffer type with round-to-nearest-even
    (saturating for fp8); the shape-dependent codes 2.2 / -2.2 are refused."""
    import torch
    count = 100003
    nbytes = {"fp32": 4, "fp16": 2, "bf16": 2, "fp8": 1}[dt]
    code_of = {"fp32": tl.FP32, "fp16": tl.FP16, "bf16": tl.BF16, "fp8": tl.FP8}[dt]
    L = tl.lib()
    buf = torch.empty(count * nbytes, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for code in (0.0, 0.5, 1.0, 2.0, 2.1, 2.3, 2.4, -1.0, -2.0, -2.1, -2.3, -2.4, 3.25):
        tl.check(L.tl_fill_pattern(code_of, buf.data_ptr(), count, code, stream))
        torch.cuda.synchronize()
        want = orc.encode(orc.init_pattern(code, count, 1), dt)
        got = buf.cpu().numpy().view(want.dtype)
        assert np.array_equal(got, want), f"code {code}: {int(np.count_nonzero(got != want))} elements differ"
    for code in (2.2, -2.2):
        assert L.tl_fill_pattern(code_of, buf.data_ptr(), count, code, stream) == tl.ERR_UNSUPPORTED


# ---------------------------------------------------------------------------- fused epilogue
def _epi_ref(o, bias, act):
    o = o.astype(np.float32)
    if bias is not None:
        o = (o + bias.astype(np.float32)[:, None]).astype(np.float32)
    if act == "relu":
        o = np.maximum(o, 0)
    elif act == "gelu":
        x = o.astype(np.float64)
        o = (0.5 * x * (1 + np.tanh(0.7978845608028654 * (x + 0.044715 * x ** 3)))).astype(np.float32)
    elif act == "silu":
        x = o.astype(np.float64)
        o = (x / (1 + np.exp(-x))).astype(np.float32)
    return o


@pytest.mark.parametrize("dt,lay,act,cg,bm,split", [
    ("bf16", "NN", "gelu", 2, 256, 1), ("bf16", "TN", "relu", 4, 256, 1), ("fp16", "NT", "silu", 1, 128, 1),
    ("bf16", "NN", "none", 1, 128, 3), ("fp16", "TN", "gelu", 2, 128, 2)])
def test_fused_epilogue(h, dt, lay, act, cg, bm, split):
    """tl_gemm_ex: act(alpha*AB + beta*C + bias[m]) and max |D| against the same kernel's fp32-output
    result with the epilogue applied on the host (one output ulp), ragged sizes, whole tiles (TMA
    stores) and split-k reductions."""
    import torch
    m, n, k = 1000, 600, 320
    case = gg.make_case(dt, lay, 321 + cg + bm + split, m, n, k, alpha=0.75, beta=0.5, ld_align=8)
    A, B = gu.to_dev(case["A_bits"], dt), gu.to_dev(case["B_bits"], dt)
    C = gu.to_dev(case["C_bits"], dt)
    tdt = {"bf16": torch.bfloat16, "fp16": torch.float16}[dt]
    g = np.random.default_rng(5)
    bias = g.standard_normal(m).astype(np.float32)
    dbias = torch.from_numpy(bias).cuda()
    sol = tl.Solution(kernel=tl.KERNEL_TCGEN05, macro_tile0=bm, macro_tile1=128 * cg, depth_u=0, stages=4,
                      split_k=split)
    kw = dict(trans_a=lay[0] == "T", trans_b=lay[1] == "T", alpha=0.75, beta=0.5, lda=case["lda"], ldb=case["ldb"],
              kernel="tcgen05")
    # the pre-epilogue values: same kernel and solution with fp32 output (C widened exactly)
    p32 = tl.Problem.make(m, n, k, dtype=dt, out_dtype="fp32", **kw)
    C32 = torch.from_numpy(case["C"].astype(np.float32)).cuda()
    D32 = torch.empty(m * n, dtype=torch.float32, device="cuda")
    h.gemm(p32, D32, C32, A, B, solution=sol)
    p = tl.Problem.make(m, n, k, dtype=dt, **kw)
    D = torch.empty(m * n, dtype=tdt, device="cuda")
    amax = torch.zeros(1, dtype=torch.float32, device="cuda")
    h.gemm_ex(p, D, C, A, B, bias=dbias, activation=act, amax=amax, solution=sol)
    torch.cuda.synchronize()
    h.device_status()
    ref = _epi_ref(D32.cpu().numpy().reshape(n, m).T, bias, act)
    got = D.float().cpu().numpy().reshape(n, m).T
    # one output ulp, with an absolute floor for the activations' flat tails (gelu / silu of large
    # negative inputs cancel to ~1e-10 in float64 but to 0 on the device)
    mant = {"bf16": 7, "fp16": 10}[dt]
    mag = np.maximum(np.abs(ref).astype(np.float64), 2.0 ** -126)
    ulp = 2.0 ** (np.floor(np.log2(mag)) - mant)
    bad = np.abs(got.astype(np.float64) - ref) > ulp + 1e-6 * np.abs(ref).max()
    assert int(bad.sum()) == 0, (got[bad][:5], ref[bad][:5])
    assert abs(amax.item() - np.abs(ref).max()) <= 1e-5 * np.abs(ref).max()
    # against the oracle: the restated reference loop (alpha*AB + beta*C in fp32), then bias and the
    # activation on the host; the activations are 1.13-Lipschitz at most, so the accumulation
    # allowance carries over scaled by that
    R0 = gu.mat(gu.oracle_ref(case), m, n, m)
    Ro = _epi_ref(R0, bias, act).astype(np.float64)
    acc = 3.0 * k * 2.0 ** -24 * 0.75 * gu.absprod_of(case) + 2.0 ** -23 * np.abs(0.5 * gu.mat(case["C"], m, n, m))
    bound = 2.0 * ulp_out(Ro, dt) + 1.13 * acc + 1e-6 * np.abs(Ro).max()
    bad = np.abs(got.astype(np.float64) - Ro) > bound
    assert int(bad.sum()) == 0, (got[bad][:5], Ro[bad][:5])


@pytest.mark.parametrize("dt,lay,act,cg,bm,split", [
    ("bf16", "NN", "none", 1, 128, 1), ("bf16", "TN", "gelu", 2, 256, 1), ("fp16", "NT", "relu", 1, 64, 1),
    ("fp8", "TN", "silu", 1, 256, 1), ("bf16", "NN", "relu", 1, 128, 3), ("fp8", "TN", "none", 2, 128, 2)])
def test_fp8_output_epilogue(h, dt, lay, act, cg, bm, split):
    """E4M3 output from the fused epilogue: D = e4m3(d_scale * act(alpha*AB + bias)), round to nearest
    even, saturating.  Checked against the oracle's loop with the epilogue applied on the host and the
    oracle's E4M3 quantiser (orc_f32_to_e4m3): every element within one E4M3 step of the quantised
    oracle value, and nearly all bit-equal; the amax is of the values before d_scale.  Whole tiles
    through TMA stores (macro_tile0 128 / 256), 64-wide tiles through direct stores, split-k
    reductions; m is ragged against every tile width and its leading dimension a multiple of 16 bytes."""
    import torch
    m, n, k = 1008, 600, 320
    case = gg.make_case(dt, lay, 901 + cg + bm + split, m, n, k, alpha=0.75, beta=0.0, ld_align=16)
    A, B = gu.to_dev(case["A_bits"], dt), gu.to_dev(case["B_bits"], dt)
    g = np.random.default_rng(6)
    bias = g.standard_normal(m).astype(np.float32)
    dbias = torch.from_numpy(bias).cuda()
    d_scale = 3.5
    W = 128 if dt == "fp8" else 64
    sol = tl.Solution(kernel=tl.KERNEL_TCGEN05, macro_tile0=bm, macro_tile1=128 * cg, depth_u=W, stages=4,
                      split_k=split)
    p = tl.Problem.make(m, n, k, dtype=dt, out_dtype="fp8", trans_a=lay[0] == "T", trans_b=lay[1] == "T",
                        alpha=0.75, lda=case["lda"], ldb=case["ldb"], kernel="tcgen05")
    D = torch.full((m * n,), 0x7f, dtype=torch.uint8, device="cuda")
    amax = torch.zeros(1, dtype=torch.float32, device="cuda")
    h.gemm_ex(p, D, None, A, B, bias=dbias, activation=act, amax=amax, d_scale=d_scale, solution=sol)
    h.device_status()
    got = orc.e4m3_to_f32(D.cpu().numpy()).reshape(n, m).T
    pre = _epi_ref(gu.mat(gu.oracle_ref(case), m, n, m), bias, act)       # before d_scale
    want = orc.e4m3_to_f32(orc.f32_to_e4m3((pre * np.float32(d_scale)).astype(np.float32)))
    # accumulation-order differences may move a value across a rounding boundary: one E4M3 step
    mag = np.maximum(np.abs(want.astype(np.float64)), 2.0 ** -6)
    step = 2.0 ** (np.floor(np.log2(mag)) - 3)
    assert np.all(np.abs(got - want) <= step + 1e-12)
    assert np.mean(got == want) > 0.99
    assert abs(amax.item() - np.abs(pre).max()) <= 1e-4 * np.abs(pre).max()
    # tl_gemm with an fp8 output: the same without bias and activation, d_scale 1
    D2 = torch.zeros(m * n, dtype=torch.uint8, device="cuda")
    h.gemm(p, D2, None, A, B, solution=sol)
    h.device_status()
    got2 = orc.e4m3_to_f32(D2.cpu().numpy()).reshape(n, m).T
    want2 = orc.e4m3_to_f32(orc.f32_to_e4m3(gu.mat(gu.oracle_ref(case), m, n, m).astype(np.float32)))
    mag2 = np.maximum(np.abs(want2.astype(np.float64)), 2.0 ** -6)
    assert np.all(np.abs(got2 - want2) <= 2.0 ** (np.floor(np.log2(mag2)) - 3) + 1e-12)


def test_fp8_output_refusals(h):
    import torch
    A = torch.zeros(128 * 128, dtype=torch.bfloat16, device="cuda")
    D = torch.zeros(128 * 128, dtype=torch.uint8, device="cuda")
    p = tl.Problem.make(128, 128, 128, dtype="bf16", out_dtype="fp8", beta=0.5)
    with pytest.raises(tl.TLError) as e:
        h.gemm(p, D, D, A, A)
    assert e.value.status == tl.ERR_UNSUPPORTED and "beta" in str(e.value)
    q = tl.Problem.make(128, 128, 128, dtype="bf16", out_dtype="fp8", kernel="simt")
    with pytest.raises(tl.TLError) as e:
        h.gemm(q, D, None, A, A)
    assert e.value.status == tl.ERR_UNSUPPORTED


def test_fused_epilogue_errors_and_linear(h):
    import torch
    p = tl.Problem.make(64, 64, 64, dtype="fp32")
    X = torch.randn(64 * 64, device="cuda")
    with pytest.raises(tl.TLError) as e:
        h.gemm_ex(p, torch.empty_like(X), None, X, X, activation="relu")      # CUDA-core kernel
    assert e.value.status == tl.ERR_UNSUPPORTED
    pb = tl.Problem.make(64, 64, 64, dtype="bf16")
    Xb = X.to(torch.bfloat16)
    with pytest.raises(tl.TLError) as e:
        h.gemm_ex(pb, torch.empty_like(Xb), None, Xb, Xb, activation=7)
    assert e.value.status == tl.ERR_INVALID_ARG
    # row-major fused linear layer against torch in fp32
    g = torch.Generator(device="cuda").manual_seed(9)
    Xr = torch.randn(512, 384, device="cuda", generator=g).to(torch.bfloat16)
    Wr = (torch.randn(384, 768, device="cuda", generator=g) * 0.05).to(torch.bfloat16)
    br = torch.randn(768, device="cuda", generator=g).to(torch.bfloat16)
    Y = tl.linear(Xr, Wr, br, "gelu")
    ref = torch.nn.functional.gelu(Xr.float() @ Wr.float() + br.float(), approximate="tanh")
    assert float((Y.float() - ref).abs().max() / ref.abs().max()) < 1e-2
