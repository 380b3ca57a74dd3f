"""The oracle pinned against the reference: converters vs the reference's own compiled code
(golden vectors), the GEMM loop vs the reference's integer-pattern known answers, and the FP64
oracle / error metrics vs numpy."""
import hashlib
import os

import numpy as np
import pytest

from oracle import oracle as orc
from tests.golden import gen_golden as gg

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def conv():
    return np.load(os.path.join(GOLD, "converters.npz"))


def test_f32_to_f16_matches_reference(conv):
    assert np.array_equal(orc.f32_to_f16(conv["x"]), conv["ref_f16"])


def test_f32_to_bf16_truncation_matches_reference(conv):
    assert np.array_equal(orc.f32_to_bf16(conv["x"], "trunc"), conv["ref_bf16"])


def test_reference_f16_decode_all_patterns(conv):
    h = np.arange(65536, dtype=np.uint16)
    assert np.array_equal(orc.f16_to_f32(h, reference_decode=True).view(np.uint32), conv["ref_f16_decode"])


def test_bf16_decode_all_patterns(conv):
    h = np.arange(65536, dtype=np.uint16)
    assert np.array_equal(orc.bf16_to_f32(h).view(np.uint32), conv["ref_bf16_decode"])


def test_reference_decode_differs_only_on_subnormal_inf_nan(conv):
    """The reference's fp16 decode is exact on normal values (its 2^112 factor is pow(1.0, 112))."""
    h = np.arange(65536, dtype=np.uint16)
    exact = orc.f16_to_f32(h)
    ref = orc.f16_to_f32(h, reference_decode=True)
    e = (h >> 10) & 0x1F
    normal = (e > 0) & (e < 31)
    assert np.array_equal(exact[normal].view(np.uint32), ref[normal].view(np.uint32))
    zero = (h & 0x7FFF) == 0
    assert np.array_equal(exact[zero].view(np.uint32), ref[zero].view(np.uint32))


def test_f16_roundtrip_exact_for_halves():
    h = np.arange(65536, dtype=np.uint16)
    e = (h >> 10) & 0x1F
    keep = e < 31
    assert np.array_equal(orc.f32_to_f16(orc.f16_to_f32(h[keep])), h[keep])


def test_bf16_rne_properties():
    g = np.random.default_rng(5)
    x = g.standard_normal(100000).astype(np.float32)
    b = orc.f32_to_bf16(x, "rne")
    y = orc.bf16_to_f32(b)
    # within half an ulp of bf16 (2^-8 relative)
    assert np.all(np.abs(y - x) <= np.abs(x) * 2.0 ** -8)
    # torch agrees (IEEE RNE)
    torch = pytest.importorskip("torch")
    tb = torch.from_numpy(x).to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16)
    assert np.array_equal(tb, b)


def test_e4m3_codec_matches_torch():
    torch = pytest.importorskip("torch")
    g = np.random.default_rng(7)
    x = np.concatenate([g.standard_normal(50000) * 100, g.standard_normal(5000) * 1e-3,
                        [0, 448, 464, 465, 2 ** -9, 2 ** -10, 0.75 * 2 ** -9]]).astype(np.float32)
    xc = np.clip(x, -448, 448)
    tq = torch.from_numpy(xc).to(torch.float8_e4m3fn).view(torch.uint8).numpy()
    assert np.array_equal(orc.f32_to_e4m3(x), tq)
    allq = np.arange(256, dtype=np.uint8)
    dec = torch.from_numpy(allq).view(torch.float8_e4m3fn).float().numpy()
    assert np.array_equal(np.nan_to_num(orc.e4m3_to_f32(allq), nan=7.0), np.nan_to_num(dec, nan=7.0))


def test_kat_small_exact():
    kat = np.load(os.path.join(GOLD, "kat.npz"))
    A, B, C, lda, ldb, ldc = gg.kat_case(64, 48, 40, 16)
    D = orc.gemm_ref_f32(1, 0, 64, 48, 40, gg.ALPHA_KAT, A, lda, B, ldb, gg.BETA_KAT, C, ldc, ldc)
    D = D.reshape(48, ldc)
    ref = kat["small"].view(np.float32).reshape(48, ldc)
    assert np.array_equal(D[:, :64].view(np.uint32), ref[:, :64].view(np.uint32))


@pytest.mark.parametrize("M,N,K,key", [(768, 640, 256, "sha_768x640x256"), (960, 1024, 1024, "sha_960x1024x1024")])
def test_kat_reference_sizes(M, N, K, key):
    """The reference's functional-matrix size (fuction_test.xlsx) and build smoke size (build.py:43-46),
    default padding 64 (inc/ff_utils.h:351)."""
    kat = np.load(os.path.join(GOLD, "kat.npz"))
    A, B, C, lda, ldb, ldc = gg.kat_case(M, N, K, 64)
    D = orc.gemm_ref_f32(1, 0, M, N, K, gg.ALPHA_KAT, A, lda, B, ldb, gg.BETA_KAT, C, ldc, ldc, threads=os.cpu_count())
    full = np.zeros(ldc * N, np.float32)
    full.reshape(N, ldc)[:, :M] = D.reshape(N, ldc)[:, :M]
    assert hashlib.sha256(full.tobytes()).hexdigest() == str(kat[key])


@pytest.mark.parametrize("dt", gg.DTYPES)
@pytest.mark.parametrize("lay", gg.LAYOUTS)
def test_small_cases_stable(dt, lay):
    gold = np.load(os.path.join(GOLD, "gemm_small.npz"))
    seed = 1000 + gg.DTYPES.index(dt) * 10 + gg.LAYOUTS.index(lay)
    c = gg.make_case(dt, lay, seed, **gg.SMALL)
    assert np.array_equal(gg.small_reference(c).view(np.uint32), gold[f"{dt}_{lay}"])


@pytest.mark.parametrize("lay", gg.LAYOUTS)
def test_f64_oracle_matches_numpy(lay):
    c = gg.make_case("fp32", lay, 9, 33, 17, 29)
    D64 = orc.gemm_f64(c["trans_a"], c["trans_b"], c["m"], c["n"], c["k"], c["alpha"], c["A"], c["lda"], c["B"],
                       c["ldb"], c["beta"], c["C"], c["ldc"], c["m"])
    ref, _ = orc.gemm_f64_numpy(c["trans_a"], c["trans_b"], c["m"], c["n"], c["k"], c["alpha"], c["A"], c["lda"],
                                c["B"], c["ldb"], c["beta"], c["C"], c["ldc"])
    assert np.allclose(D64.reshape(c["n"], c["m"]).T, ref, rtol=1e-13, atol=1e-12)


def test_threaded_loop_is_bit_identical():
    c = gg.make_case("fp32", "NN", 11, 70, 45, 33)
    args = (c["trans_a"], c["trans_b"], 70, 45, 33, 1.0, c["A"], c["lda"], c["B"], c["ldb"], 0.5, c["C"], 70, 70)
    d1 = orc.gemm_ref_f32(*args, threads=1)
    d4 = orc.gemm_ref_f32(*args, threads=4)
    assert np.array_equal(d1.view(np.uint32), d4.view(np.uint32))


def test_batched_and_column_subset():
    g = np.random.default_rng(3)
    M, N, K, batch = 12, 10, 9, 3
    A = g.standard_normal(M * K * batch).astype(np.float32)
    B = g.standard_normal(K * N * batch).astype(np.float32)
    D = orc.gemm_ref_f32(0, 0, M, N, K, 1.0, A, M, B, K, batch=batch, stride_a=M * K, stride_b=K * N,
                         stride_d=M * N)
    for b in range(batch):
        ref = (A[b * M * K:(b + 1) * M * K].reshape(K, M).T.astype(np.float64) @
               B[b * K * N:(b + 1) * K * N].reshape(N, K).T.astype(np.float64))
        got = D[b * M * N:(b + 1) * M * N].reshape(N, M).T
        assert np.allclose(got, ref, rtol=1e-5, atol=1e-5)
    part = orc.gemm_ref_f32(0, 0, M, N, K, 1.0, A, M, B, K, n_begin=3, n_end=6)
    full = orc.gemm_ref_f32(0, 0, M, N, K, 1.0, A, M, B, K)
    assert np.array_equal(part.reshape(N, M)[3:6], full.reshape(N, M)[3:6])
    assert np.all(part.reshape(N, M)[:3] == 0)


def test_error_metrics():
    r = np.array([1.0, -2.0, 4.0])
    d = np.array([1.0, -2.5, 4.0])
    assert orc.normwise_error(d, r) == pytest.approx(0.125)
    assert orc.componentwise_error(d, r, np.array([1.0, 5.0, 1.0])) == pytest.approx(0.1)


def test_init_pattern_codes():
    x = orc.init_pattern(2.4, 8, 3)
    assert np.array_equal(x, (np.arange(24) % 7).astype(np.float32))
    y = orc.init_pattern(-2.4, 8, 3)
    assert np.array_equal(y, -(np.arange(24) % 11).astype(np.float32))


def test_grouped_sizes_seed3():
    _, sizes = orc.grouped_sizes()
    assert sizes[:3] == [(1680, 880, 3840), (224, 576, 832), (416, 1040, 1408)]
    assert sum(2 * m * n * k for m, n, k in sizes) == 1147123695616
