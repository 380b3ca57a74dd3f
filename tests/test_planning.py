"""Solution planning without a GPU: a planning handle (tl_init_host) for a described GB300 runs the
tile heuristic (GemmMfmaSolver::generateSolver's role, src/gemmMfma.cpp) and the legality check
(checkKernelParameters, src/gemmMfmaKernelWriter.h:321-405), and refuses every call that would
launch, allocate or time work."""
import ctypes

import pytest

import tensilelite_gb300 as tl
from tensilelite_gb300 import Problem, Solution, TLError


@pytest.fixture(scope="module")
def gb300():
    h = tl.Handle.planning()          # 152 SMs, 227 KB opt-in shared memory, 36 clusters of four
    yield h
    h.close()


def test_planning_handle_describes_the_device(gb300):
    assert gb300.device_info() == {"sm_count": 152, "cc": (10, 3), "smem_optin": 232448}


@pytest.mark.parametrize("args", [(0, 232448, 0), (152, 1024, 0), (152, 232448, 39), (152, 232448, -1)])
def test_planning_handle_rejects_bad_descriptions(args):
    h = ctypes.c_void_p()
    assert tl.lib().tl_init_host(*args, ctypes.byref(h)) == tl.ERR_INVALID_ARG
    assert not h.value
    assert tl.lib().tl_init_host(152, 232448, 36, None) == tl.ERR_INVALID_ARG


def test_planning_handle_refuses_device_work(gb300):
    L, h = tl.lib(), gb300.ptr
    p = Problem.make(256, 256, 256, dtype="bf16")
    s = gb300.default_solution(p)
    pp, sp = ctypes.byref(p), ctypes.byref(s)
    out = ctypes.c_void_p()
    f = ctypes.c_float()
    dbl = (ctypes.c_double * 3)()
    n64 = ctypes.c_int64()
    calls = {
        "tl_gemm": lambda: L.tl_gemm(h, pp, sp, None, None, None, None, None),
        "tl_gemm_ex": lambda: L.tl_gemm_ex(h, pp, None, sp, None, None, None, None, None),
        "tl_tune": lambda: L.tl_tune(h, pp, None, None, None, None, 4, 1, None, sp, ctypes.byref(f)),
        "tl_tensile_launch": lambda: L.tl_tensile_launch(h, b"Cijk_Alik_Bljk_SB", None, 0, None),
        "tl_grouped_plan_create": lambda: L.tl_grouped_plan_create(h, pp, 1, None, None, None, None, None,
                                                                   ctypes.byref(out)),
        "tl_gemm_grouped": lambda: L.tl_gemm_grouped(h, pp, 1, None, None, None, None, None),
        "tl_tune_grouped": lambda: L.tl_tune_grouped(h, pp, 1, None, None, None, None, 1, sp, ctypes.byref(f)),
        "tl_graph_capture_gemm": lambda: L.tl_graph_capture_gemm(h, pp, sp, None, None, None, None, None,
                                                                 ctypes.byref(out)),
        "tl_quantize_fp8": lambda: L.tl_quantize_fp8(h, tl.FP32, None, 0, None, None, None, None),
        "tl_split_bf16x2": lambda: L.tl_split_bf16x2(h, None, 0, None, None, None),
        "tl_error_norms": lambda: L.tl_error_norms(h, tl.BF16, None, 1, None, None, 1, 1, 1, dbl, None),
        "tl_set_kernel_timing": lambda: L.tl_set_kernel_timing(h, 1),
        "tl_kernel_timing": lambda: L.tl_kernel_timing(h, dbl, ctypes.byref(n64), 0),
        "tl_device_status": lambda: L.tl_device_status(h, None),
    }
    for name, call in calls.items():
        assert call() == tl.ERR_INVALID_ARG, name
        assert b"planning handle" in L.tl_last_error_string(), name
    # bookkeeping calls are fine
    assert L.tl_launch_count(h, ctypes.byref(n64)) == tl.SUCCESS and n64.value == 0
    assert L.tl_set_wait_timeout(h, 100) == tl.SUCCESS


# Tiles the device handle picked for these problems on a GB300 (recorded in the benchmark and
# tile-sweep runs there): (macro_tile0, macro_tile1, split_k, stages, raster, promote_k, depth_u).
DEVICE_PICKS = [
    ("bf16 4096^3 NN beta 0.5", dict(m=4096, n=4096, k=4096, beta=0.5), (256, 256, 1, 6, 0, 0, 64)),
    ("bf16 4096x4096x1024 NN", dict(m=4096, n=4096, k=1024), (256, 512, 1, 6, 0, 0, 64)),
    ("bf16 dX 1024x4096x4096 TN", dict(m=1024, n=4096, k=4096, trans_a=True), (256, 512, 1, 6, 0, 0, 64)),
    ("bf16 dW 4096x1024x4096 NT", dict(m=4096, n=1024, k=4096, trans_b=True), (256, 512, 1, 6, 0, 0, 64)),
    ("bf16 1024x4096x4096 NN", dict(m=1024, n=4096, k=4096), (256, 512, 1, 6, 0, 0, 64)),
    ("bf16 480x1024x4096 NN", dict(m=480, n=1024, k=4096), (128, 128, 4, 6, 0, 0, 64)),
    ("bf16 1024^3 NN", dict(m=1024, n=1024, k=1024), (128, 256, 1, 6, 0, 0, 64)),
    ("bf16 1024x1024x4096 NN", dict(m=1024, n=1024, k=4096), (192, 128, 3, 5, 0, 0, 64)),
    ("fp8 8192^3 TN", dict(m=8192, n=8192, k=8192, dtype="fp8", trans_a=True), (256, 512, 1, 6, 8, 0, 128)),
    ("bf16x6 8192^3 NN", dict(m=8192, n=8192, k=8192, dtype="fp32", kernel="bf16x6"), (128, 256, 1, 6, 8, 256, 64)),
]


@pytest.mark.parametrize("name,kw,want", DEVICE_PICKS, ids=[d[0] for d in DEVICE_PICKS])
def test_heuristic_matches_the_device_handle(gb300, name, kw, want):
    kw = dict(kw)
    m, n, k = kw.pop("m"), kw.pop("n"), kw.pop("k")
    p = Problem.make(m, n, k, dtype=kw.pop("dtype", "bf16"), **kw)
    s = gb300.default_solution(p)
    got = (s.macro_tile0, s.macro_tile1, s.split_k, s.stages, s.raster, s.promote_k, s.depth_u)
    assert got == want
    gb300.check_solution(p, s)


@pytest.mark.parametrize("dtype", ["bf16", "fp16", "fp8"])
@pytest.mark.parametrize("ta,tb", [(False, False), (True, False), (False, True), (True, True)])
def test_heuristic_solutions_are_legal(gb300, dtype, ta, tb):
    for m, n, k in [(1, 1, 1), (64, 64, 64), (100, 300, 17), (480, 1024, 4096), (2048, 512, 8192),
                    (4096, 4096, 4096), (12288, 1024, 256), (256, 8192, 65536)]:
        p = Problem.make(m, n, k, dtype=dtype, trans_a=ta, trans_b=tb)
        s = gb300.default_solution(p)
        assert s.kernel == tl.KERNEL_TCGEN05
        gb300.check_solution(p, s)


def test_nn_plans_as_its_transposed_view(gb300):
    """An NN problem with beta = 0 and k >= 2048 is planned (and run) as the TT problem with m and n
    exchanged; with beta != 0 or short k it is planned as it is."""
    nn = Problem.make(1024, 4096, 4096, dtype="bf16")
    tt = Problem.make(4096, 1024, 4096, dtype="bf16", trans_a=True, trans_b=True)
    assert gb300.default_solution(nn).as_dict() == gb300.default_solution(tt).as_dict()
    gb300.check_solution(nn, gb300.default_solution(nn))
    # with beta, or k below 2048, the NN problem keeps its own shape: a pick that is legal only for
    # it (MN-major A needs whole 128-byte chunks of m per CTA) is accepted
    for p in (Problem.make(1024, 4096, 4096, dtype="bf16", beta=0.5), Problem.make(1024, 4096, 1024, dtype="bf16")):
        s = gb300.default_solution(p)
        gb300.check_solution(p, s)


def test_heuristic_is_deterministic_and_simt_for_fp32(gb300):
    p = Problem.make(3000, 2000, 1000, dtype="bf16")
    assert gb300.default_solution(p).as_dict() == gb300.default_solution(p).as_dict()
    s = gb300.default_solution(Problem.make(480, 512, 512, dtype="fp32"))
    assert (s.kernel, s.macro_tile0, s.macro_tile1) == (tl.KERNEL_SIMT, 128, 128)


def _sol(**kw):
    s = Solution()
    s.kernel, s.macro_tile0, s.macro_tile1, s.depth_u, s.stages, s.split_k = tl.KERNEL_TCGEN05, 256, 256, 64, 6, 1
    for key, v in kw.items():
        setattr(s, key, v)
    return s


ILLEGAL = [
    ("macro_tile1 384", dict(macro_tile1=384), tl.ERR_UNSUPPORTED),
    ("macro_tile0 96", dict(macro_tile0=96), tl.ERR_UNSUPPORTED),
    ("pair with macro_tile0 64", dict(macro_tile0=64), tl.ERR_UNSUPPORTED),
    ("two pairs with macro_tile0 128", dict(macro_tile0=128, macro_tile1=512), tl.ERR_UNSUPPORTED),
    ("depth_u 32", dict(depth_u=32), tl.ERR_UNSUPPORTED),
    ("one stage", dict(stages=1), tl.ERR_UNSUPPORTED),
    ("nine stages", dict(stages=9), tl.ERR_UNSUPPORTED),
    ("shared memory", dict(macro_tile1=128, stages=8), tl.ERR_UNSUPPORTED),
    ("split_k beyond k blocks", dict(split_k=65), tl.ERR_UNSUPPORTED),
    ("negative raster", dict(raster=-1), tl.ERR_INVALID_ARG),
    ("tail_split 9", dict(tail_split=9), tl.ERR_INVALID_ARG),
    ("promotion with macro_tile0 256", dict(promote_k=256), tl.ERR_UNSUPPORTED),
    ("unresolved kernel", dict(kernel=tl.KERNEL_AUTO), tl.ERR_INVALID_ARG),
    ("SIMT 64x64", dict(kernel=tl.KERNEL_SIMT, macro_tile0=64, macro_tile1=64, depth_u=8), tl.ERR_UNSUPPORTED),
]


@pytest.mark.parametrize("name,kw,status", ILLEGAL, ids=[c[0] for c in ILLEGAL])
def test_check_solution_rejects(gb300, name, kw, status):
    p = Problem.make(4096, 4096, 4096, dtype="bf16")
    with pytest.raises(TLError) as e:
        gb300.check_solution(p, _sol(**kw))
    assert e.value.status == status


def test_check_solution_accepts_the_documented_tiles(gb300):
    p = Problem.make(4096, 4096, 4096, dtype="bf16")
    for mt0, mt1, stages in [(64, 128, 6), (128, 128, 6), (192, 128, 4), (256, 128, 4), (128, 256, 6),
                             (256, 256, 6), (256, 512, 6)]:
        gb300.check_solution(p, _sol(macro_tile0=mt0, macro_tile1=mt1, stages=stages))
    gb300.check_solution(p, _sol(split_k=64))
    gb300.check_solution(p, _sol(tail_split=-1))


def test_dtype_rules(gb300):
    with pytest.raises(TLError) as e:
        gb300.check_solution(Problem.make(256, 256, 256, dtype="fp32"), _sol())
    assert e.value.status == tl.ERR_UNSUPPORTED
    with pytest.raises(TLError) as e:
        gb300.check_solution(Problem.make(256, 256, 256, dtype="bf16"), _sol(kernel=tl.KERNEL_BF16X3, macro_tile0=128))
    assert e.value.status == tl.ERR_UNSUPPORTED
    gb300.check_solution(Problem.make(256, 256, 256, dtype="fp32"),
                         _sol(kernel=tl.KERNEL_BF16X3, macro_tile0=128, promote_k=256))


@pytest.mark.parametrize("m,n,k", [(1, 1, 1), (64, 64, 64), (128, 128, 64), (64, 64, 1), (256, 256, 63)])
def test_single_tile_single_k_block_plans(gb300, m, n, k):
    # one tile of one k-block leaves no worker for a split of the last wave; the cost model used to
    # divide by that zero worker count (SIGFPE on x86 hosts)
    for dtype in ("bf16", "fp8"):
        p = Problem.make(m, n, k, dtype=dtype)
        s = gb300.default_solution(p)
        assert s.split_k == 1
        gb300.check_solution(p, s)


def test_mn_major_rules(gb300):
    # MN-major A (problem NN: A stored m-contiguous) is staged in 128-byte chunks of m per CTA
    fp8_nn = Problem.make(520, 600, 704, dtype="fp8")
    with pytest.raises(TLError) as e:     # a pair of 128 m rows leaves 64 fp8 rows (half a chunk) per CTA
        gb300.check_solution(fp8_nn, _sol(macro_tile0=128, depth_u=128))
    assert e.value.status == tl.ERR_UNSUPPORTED
    gb300.check_solution(fp8_nn, _sol(macro_tile0=256, depth_u=128))
    gb300.check_solution(Problem.make(520, 600, 704, dtype="fp8", trans_a=True), _sol(macro_tile0=128, depth_u=128))
    with pytest.raises(TLError) as e:     # two pairs: each CTA needs two 128-byte chunks of m
        gb300.check_solution(fp8_nn, _sol(macro_tile0=256, macro_tile1=512, depth_u=128))
    assert e.value.status == tl.ERR_UNSUPPORTED
    gb300.check_solution(Problem.make(520, 600, 704, dtype="bf16"), _sol(macro_tile0=256, macro_tile1=512))
