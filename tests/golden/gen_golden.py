"""Generates the golden fixtures under tests/golden/ (run from the repository root).

  converters.npz  the reference's OWN host converters (inc/ff_utils.h:90-127, compiled in place from
                  the reference tree into oracle/_ref/libffref.so) applied to a fixed sample of fp32
                  values and to every fp16 bit pattern -- pins the oracle's restated converters.
  kat.npz         the reference's integer-pattern known answer (InitRealData codes 2.4 / -2.4,
                  ff_gpu_src/ff_gpu.cpp:131,137; alpha = 0.314, beta = 0.2718, src/gemmMfma.cpp:229-235)
                  for TN GEMMs: exact integer sums, then alpha*s + beta*c rounded in fp32 as the
                  reference's loop does (src/gemmMfma.cpp:325-345).  Small case stored in full, the
                  reference's functional-matrix size (768x640x256) and its build smoke size
                  (960x1024x1024) as SHA-256 of the result bits.
  gemm_small.npz  the oracle's reference-parity loop on small seeded problems for every
                  dtype x layout (inputs are regenerated from the seed by ``make_case``).

Needs the reference tree for converters.npz (set TL_REFERENCE_TREE); the rest needs only the oracle.
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as orc  # noqa: E402

ALPHA_KAT = np.float32(0.314)
BETA_KAT = np.float32(0.2718)
SMALL = dict(m=40, n=24, k=56)
LAYOUTS = ["NN", "NT", "TN", "TT"]
DTYPES = ["fp32", "fp16", "bf16", "fp8"]


def kat_case(M, N, K, pad):
    """Buffers of the reference's TN problem: A is M rows of K+pad, B is N rows of K+pad, C is N
    columns of M+pad (src/gemmMfma.cpp:210-217)."""
    lda, ldb, ldc = K + pad, K + pad, M + pad
    A = orc.init_pattern(2.4, lda, M)
    B = orc.init_pattern(-2.4, ldb, N)
    C = orc.init_pattern(2.4, ldc, N)
    return A, B, C, lda, ldb, ldc


def kat_expected(M, N, K, pad):
    """Exact integer products, then the reference's fp32 alpha/beta step -> D (ldc x N flat)."""
    A, B, C, lda, ldb, ldc = kat_case(M, N, K, pad)
    Ai = A.reshape(M, lda)[:, :K].astype(np.int64)
    Bi = B.reshape(N, ldb)[:, :K].astype(np.int64)
    S = Ai @ Bi.T
    assert np.abs(S).max() < 2 ** 24
    Cm = C.reshape(N, ldc)[:, :M].T
    Dm = (ALPHA_KAT * S.astype(np.float32) + BETA_KAT * Cm).astype(np.float32)
    D = np.zeros(ldc * N, np.float32)
    D.reshape(N, ldc)[:, :M] = Dm.T
    return D


def make_case(dtype, layout, seed, m, n, k, alpha=1.0, beta=0.5, ld_align=1):
    """Seeded column-major buffers: A, B ~ N(0,1) drawn in that order, then C; cast to dtype (RNE).
    Leading dimensions are the stored row counts rounded up to ``ld_align`` elements (the padding
    holds values too).  Returns dict with storage bits, their exact fp32 values and leading dims."""
    ta, tb = layout[0] == "T", layout[1] == "T"
    g = np.random.default_rng(seed)
    a_rows, a_cols = (k, m) if ta else (m, k)
    b_rows, b_cols = (n, k) if tb else (k, n)
    a_rows = -(-a_rows // ld_align) * ld_align
    b_rows = -(-b_rows // ld_align) * ld_align
    A = g.standard_normal(a_rows * a_cols)
    B = g.standard_normal(b_rows * b_cols)
    C = g.standard_normal(m * n)
    out_dt = "bf16" if dtype == "fp8" else dtype
    if dtype == "fp8":
        A, B = A * 4.0, B * 4.0
    Ab = orc.encode(A.astype(np.float32), dtype)
    Bb = orc.encode(B.astype(np.float32), dtype)
    Cb = orc.encode(C.astype(np.float32), out_dt)
    return dict(trans_a=ta, trans_b=tb, m=m, n=n, k=k, lda=a_rows, ldb=b_rows, ldc=m, alpha=alpha, beta=beta,
                A_bits=Ab, B_bits=Bb, C_bits=Cb, A=orc.decode(Ab, dtype), B=orc.decode(Bb, dtype),
                C=orc.decode(Cb, out_dt), out_dtype=out_dt)


def small_reference(case):
    return orc.gemm_ref_f32(case["trans_a"], case["trans_b"], case["m"], case["n"], case["k"], case["alpha"],
                            case["A"], case["lda"], case["B"], case["ldb"], case["beta"], case["C"], case["ldc"],
                            case["m"])


def main():
    # converters: the reference's own code
    R = orc.ref_lib()
    if R is not None:
        g = np.random.default_rng(123)
        u = g.integers(0, 2 ** 32, 20000, dtype=np.uint64).astype(np.uint32)
        normals = (g.standard_normal(20000) * np.exp2(g.integers(-30, 17, 20000))).astype(np.float32)
        special = np.array([0.0, -0.0, 1.0, -2.5, 65504.0, 65519.0, 65520.0, 65536.0, 6.0e-8, 2.98e-8, 5.96e-8,
                            1e-8, np.inf, -np.inf, 3.14159265, 0.1, 448.0], np.float32)
        x = np.concatenate([u.view(np.float32), normals, special])
        halves = np.arange(65536, dtype=np.uint16)
        np.savez_compressed(os.path.join(HERE, "converters.npz"), x=x,
                            ref_f16=orc.ref_convert("f32_to_f16", x),
                            ref_bf16=orc.ref_convert("f32_to_bf16", x),
                            ref_f16_decode=orc.ref_convert("f16_to_f32", halves).view(np.uint32),
                            ref_bf16_decode=orc.ref_convert("bf16_to_f32", halves).view(np.uint32))
        print("converters.npz written from", orc._HERE + "/_ref/libffref.so")
    else:
        print("reference tree absent: converters.npz left as is")

    # KAT
    small = kat_expected(64, 48, 40, 16)
    h1 = hashlib.sha256(kat_expected(768, 640, 256, 64).tobytes()).hexdigest()
    h2 = hashlib.sha256(kat_expected(960, 1024, 1024, 64).tobytes()).hexdigest()
    np.savez_compressed(os.path.join(HERE, "kat.npz"), small=small.view(np.uint32), sha_768x640x256=h1,
                        sha_960x1024x1024=h2)
    print("kat.npz written")

    # small seeded cases through the restated loop
    out = {}
    for dt in DTYPES:
        for lay in LAYOUTS:
            seed = 1000 + DTYPES.index(dt) * 10 + LAYOUTS.index(lay)
            c = make_case(dt, lay, seed, **SMALL)
            out[f"{dt}_{lay}"] = small_reference(c).view(np.uint32)
    np.savez_compressed(os.path.join(HERE, "gemm_small.npz"), **out)
    print("gemm_small.npz written")


if __name__ == "__main__":
    main()
