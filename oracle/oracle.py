"""oracle.py -- TEST INFRASTRUCTURE ONLY.

Python side of the oracle: loads ``liboracle.so`` (tl_oracle.c, the C restatement of
TensileLite's CPU GEMM ``GemmMfmaProblem::cpuCompute``, src/gemmMfma.cpp:313-346, and of its host
converters, inc/ff_utils.h:90-127) and adds the seeded input generators and the FP64 error metrics
the tests use.  Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this module; the product library never does.

``ref_lib()`` loads ``_ref/libffref.so`` -- the reference's own converters compiled in place --
when it was built (it needs the reference tree, so it exists only where that tree does).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None

_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)
_u16p = ctypes.POINTER(ctypes.c_uint16)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_i64 = ctypes.c_int64


def build(quiet: bool = True) -> str:
    """Compile liboracle.so in place (gcc, a few seconds)."""
    out = subprocess.run(["make", "-C", _HERE, "liboracle.so"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return os.path.join(_HERE, "liboracle.so")


def build_ref(ref_tree: str | None = None) -> str | None:
    """Compile the reference's converters from the reference tree: `ref_tree`, else the environment
    variable TL_REFERENCE_TREE.  Raises when neither names a tree holding inc/ff_utils.h."""
    ref = ref_tree or os.environ.get("TL_REFERENCE_TREE")
    if not ref:
        raise RuntimeError("the reference tree is not set: pass ref_tree or set TL_REFERENCE_TREE")
    if not os.path.isfile(os.path.join(ref, "inc", "ff_utils.h")):
        raise RuntimeError(f"no reference tree at {ref} (inc/ff_utils.h missing)")
    out = subprocess.run(["make", "-C", _HERE, "ref", "REF=" + ref], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("reference converter build failed:\n" + out.stdout + out.stderr)
    return os.path.join(_HERE, "_ref", "libffref.so")


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        for name, argt in [("orc_f32_to_f16_n", (_f32p, _u16p, _i64)),
                           ("orc_f16_to_f32_n", (_u16p, _f32p, _i64)),
                           ("orc_ref_f16_to_f32_n", (_u16p, _f32p, _i64)),
                           ("orc_f32_to_bf16_trunc_n", (_f32p, _u16p, _i64)),
                           ("orc_f32_to_bf16_rne_n", (_f32p, _u16p, _i64)),
                           ("orc_bf16_to_f32_n", (_u16p, _f32p, _i64)),
                           ("orc_f32_to_e4m3_n", (_f32p, _u8p, _i64)),
                           ("orc_e4m3_to_f32_n", (_u8p, _f32p, _i64))]:
            fn = getattr(L, name)
            fn.argtypes = argt
            fn.restype = None
        L.orc_init_pattern.argtypes = (ctypes.c_float, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, _f32p)
        L.orc_init_pattern.restype = ctypes.c_int
        common = (ctypes.c_int, ctypes.c_int, _i64, _i64, _i64, _i64, ctypes.c_float,
                  _f32p, _i64, _i64, _f32p, _i64, _i64, ctypes.c_float, _f32p, _i64, _i64)
        L.orc_gemm_ref_f32.argtypes = common + (_f32p, _i64, _i64, _i64, _i64, ctypes.c_int)
        L.orc_gemm_ref_f32.restype = ctypes.c_int
        L.orc_gemm_f64.argtypes = common + (_f64p, _i64, _i64, _i64, _i64, ctypes.c_int)
        L.orc_gemm_f64.restype = ctypes.c_int
        L.orc_gemm_ref_f32_packed.argtypes = (_i64, _i64, _i64, ctypes.c_float, _f32p, _f32p, ctypes.c_float,
                                              _f32p, _i64, _f32p, _i64, _i64, _i64, ctypes.c_int)
        L.orc_gemm_ref_f32_packed.restype = ctypes.c_int
        _LIB = L
    return _LIB


def ref_lib():
    """The reference's converters (compiled from the reference tree), or None."""
    global _REF
    if _REF is None:
        path = os.path.join(_HERE, "_ref", "libffref.so")
        if not os.path.exists(path):
            try:
                path = build_ref()
            except RuntimeError:
                path = None
        if not path or not os.path.exists(path):
            return None
        R = ctypes.CDLL(path)
        R.ref_cvt_f32_to_f16.argtypes = (ctypes.c_float,)
        R.ref_cvt_f32_to_f16.restype = ctypes.c_uint16
        R.ref_cvt_f16_to_f32.argtypes = (ctypes.c_uint16,)
        R.ref_cvt_f16_to_f32.restype = ctypes.c_float
        R.ref_cvt_f32_to_bf16.argtypes = (ctypes.c_float,)
        R.ref_cvt_f32_to_bf16.restype = ctypes.c_uint16
        R.ref_cvt_bf16_to_f32.argtypes = (ctypes.c_uint16,)
        R.ref_cvt_bf16_to_f32.restype = ctypes.c_float
        for name, argt in [("ref_cvt_f32_to_f16_n", (_f32p, _u16p, ctypes.c_long)),
                           ("ref_cvt_f16_to_f32_n", (_u16p, _f32p, ctypes.c_long)),
                           ("ref_cvt_f32_to_bf16_n", (_f32p, _u16p, ctypes.c_long)),
                           ("ref_cvt_bf16_to_f32_n", (_u16p, _f32p, ctypes.c_long))]:
            fn = getattr(R, name)
            fn.argtypes = argt
            fn.restype = None
        _REF = R
    return _REF


def _p(a, t):
    return a.ctypes.data_as(t)


def ref_convert(kind, x):
    """Run one of the reference's own converters over an array (needs ``ref_lib()``).
    kind: 'f32_to_f16', 'f16_to_f32', 'f32_to_bf16', 'bf16_to_f32'."""
    R = ref_lib()
    if R is None:
        raise RuntimeError("reference converters not built")
    src_t, dst_t = {"f32_to_f16": (np.float32, np.uint16), "f16_to_f32": (np.uint16, np.float32),
                    "f32_to_bf16": (np.float32, np.uint16), "bf16_to_f32": (np.uint16, np.float32)}[kind]
    x = np.ascontiguousarray(x, dtype=src_t)
    y = np.empty(x.shape, dst_t)
    pt = {np.float32: _f32p, np.uint16: _u16p}
    getattr(R, "ref_cvt_" + kind + "_n")(_p(x, pt[src_t]), _p(y, pt[dst_t]), x.size)
    return y


# ---------------------------------------------------------------------------------------------
# converters (bulk)
# ---------------------------------------------------------------------------------------------
def f32_to_f16(x):
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty(x.shape, np.uint16)
    lib().orc_f32_to_f16_n(_p(x, _f32p), _p(y, _u16p), x.size)
    return y


def f16_to_f32(h, reference_decode=False):
    h = np.ascontiguousarray(h, dtype=np.uint16)
    y = np.empty(h.shape, np.float32)
    fn = lib().orc_ref_f16_to_f32_n if reference_decode else lib().orc_f16_to_f32_n
    fn(_p(h, _u16p), _p(y, _f32p), h.size)
    return y


def f32_to_bf16(x, rounding="rne"):
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty(x.shape, np.uint16)
    fn = lib().orc_f32_to_bf16_rne_n if rounding == "rne" else lib().orc_f32_to_bf16_trunc_n
    fn(_p(x, _f32p), _p(y, _u16p), x.size)
    return y


def bf16_to_f32(b):
    b = np.ascontiguousarray(b, dtype=np.uint16)
    y = np.empty(b.shape, np.float32)
    lib().orc_bf16_to_f32_n(_p(b, _u16p), _p(y, _f32p), b.size)
    return y


def f32_to_e4m3(x):
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty(x.shape, np.uint8)
    lib().orc_f32_to_e4m3_n(_p(x, _f32p), _p(y, _u8p), x.size)
    return y


def e4m3_to_f32(q):
    q = np.ascontiguousarray(q, dtype=np.uint8)
    y = np.empty(q.shape, np.float32)
    lib().orc_e4m3_to_f32_n(_p(q, _u8p), _p(y, _f32p), q.size)
    return y


def encode(x_f32, dtype, bf16_rounding="rne"):
    """fp32 values -> storage bits of ``dtype`` ('fp32','fp16','bf16','fp8')."""
    if dtype == "fp32":
        return np.ascontiguousarray(x_f32, dtype=np.float32)
    if dtype == "fp16":
        return f32_to_f16(x_f32)
    if dtype == "bf16":
        return f32_to_bf16(x_f32, bf16_rounding)
    if dtype == "fp8":
        return f32_to_e4m3(x_f32)
    raise ValueError(dtype)


def decode(bits, dtype, reference_decode=False):
    """storage bits -> exact fp32 values."""
    if dtype == "fp32":
        return np.asarray(bits, dtype=np.float32)
    if dtype == "fp16":
        return f16_to_f32(bits, reference_decode)
    if dtype == "bf16":
        return bf16_to_f32(bits)
    if dtype == "fp8":
        return e4m3_to_f32(bits)
    raise ValueError(dtype)


def init_pattern(code, dim0, dim1, dim2=1):
    """InitRealData (ff_gpu_src/ff_gpu.cpp:110-148): flat buffer of dim0*dim1*dim2 floats."""
    out = np.empty(dim0 * dim1 * dim2, np.float32)
    lib().orc_init_pattern(ctypes.c_float(code), dim0, dim1, dim2, _p(out, _f32p))
    return out


# ---------------------------------------------------------------------------------------------
# GEMM oracles (column-major, flat float buffers)
# ---------------------------------------------------------------------------------------------
def _flat32(a):
    return np.ascontiguousarray(a, dtype=np.float32).reshape(-1)


def gemm_ref_f32(trans_a, trans_b, M, N, K, alpha, A, lda, B, ldb, beta=0.0, C=None, ldc=None, ldd=None,
                 batch=1, stride_a=0, stride_b=0, stride_c=0, stride_d=None, n_begin=0, n_end=-1, threads=1):
    """The reference loop (src/gemmMfma.cpp:325-345) through op(A)/op(B); returns flat float32 D."""
    ldd = ldd or M
    ldc = ldc or ldd
    stride_d = stride_d if stride_d is not None else ldd * N
    A = _flat32(A)
    B = _flat32(B)
    Cf = _flat32(C) if C is not None else None
    D = np.zeros(max(1, (batch - 1) * stride_d + ldd * N), np.float32)
    rc = lib().orc_gemm_ref_f32(int(trans_a), int(trans_b), M, N, K, batch, ctypes.c_float(alpha),
                                _p(A, _f32p), lda, stride_a, _p(B, _f32p), ldb, stride_b, ctypes.c_float(beta),
                                _p(Cf, _f32p) if Cf is not None else None, ldc, stride_c,
                                _p(D, _f32p), ldd, stride_d, n_begin, n_end, threads)
    if rc != 0:
        raise MemoryError("oracle allocation failed")
    return D


def gemm_f64(trans_a, trans_b, M, N, K, alpha, A, lda, B, ldb, beta=0.0, C=None, ldc=None, ldd=None,
             batch=1, stride_a=0, stride_b=0, stride_c=0, stride_d=None, threads=None):
    """FP64 host oracle with the same indexing (loop in C; use for small/medium sizes)."""
    ldd = ldd or M
    ldc = ldc or ldd
    stride_d = stride_d if stride_d is not None else ldd * N
    threads = threads or os.cpu_count() or 1
    A = _flat32(A)
    B = _flat32(B)
    Cf = _flat32(C) if C is not None else None
    D = np.zeros(max(1, (batch - 1) * stride_d + ldd * N), np.float64)
    rc = lib().orc_gemm_f64(int(trans_a), int(trans_b), M, N, K, batch, ctypes.c_float(alpha),
                            _p(A, _f32p), lda, stride_a, _p(B, _f32p), ldb, stride_b, ctypes.c_float(beta),
                            _p(Cf, _f32p) if Cf is not None else None, ldc, stride_c,
                            _p(D, _f64p), ldd, stride_d, 0, -1, threads)
    if rc != 0:
        raise MemoryError("oracle allocation failed")
    return D


def op_matrix(flat, trans, rows, cols, ld, dtype=np.float64):
    """Dense op(X) (rows x cols) from a column-major flat buffer; op = X or X^T."""
    flat = np.ascontiguousarray(flat)
    if not trans:      # X stored rows x cols column-major: X[r + c*ld]
        return np.lib.stride_tricks.as_strided(flat, shape=(rows, cols),
                                               strides=(flat.itemsize, flat.itemsize * ld)).astype(dtype)
    # op(X) = X^T where X is cols x rows column-major: op(X)[r, c] = X[c + r*ld]
    return np.lib.stride_tricks.as_strided(flat, shape=(rows, cols),
                                           strides=(flat.itemsize * ld, flat.itemsize)).astype(dtype)


def gemm_f64_numpy(trans_a, trans_b, M, N, K, alpha, A, lda, B, ldb, beta=0.0, C=None, ldc=None):
    """FP64 oracle through numpy's float64 matmul (multi-threaded BLAS) for large sizes.
    Returns (D as an M x N float64 array, |op(A)| @ |op(B)| for the componentwise metric)."""
    opA = op_matrix(A, trans_a, M, K, lda)
    opB = op_matrix(B, trans_b, K, N, ldb)
    D = alpha * (opA @ opB)
    if beta != 0.0 and C is not None:
        D += beta * op_matrix(C, False, M, N, ldc or M)
    absprod = np.abs(opA) @ np.abs(opB)
    return D, absprod


# ---------------------------------------------------------------------------------------------
# error metrics (host, FP64)
# ---------------------------------------------------------------------------------------------
def normwise_error(d, r):
    """max|d - r| / max|r|  (the headline metric)."""
    d = np.asarray(d, np.float64)
    r = np.asarray(r, np.float64)
    den = np.max(np.abs(r)) if r.size else 0.0
    num = np.max(np.abs(d - r)) if r.size else 0.0
    return float(num / den) if den > 0 else float(num)


def componentwise_error(d, r, absprod, alpha=1.0):
    """max |d - r| / (|alpha| * sum_k |a_mk| |b_kn|)."""
    d = np.asarray(d, np.float64)
    r = np.asarray(r, np.float64)
    den = abs(alpha) * np.asarray(absprod, np.float64) + 1e-300
    return float(np.max(np.abs(d - r) / den)) if r.size else 0.0


# ---------------------------------------------------------------------------------------------
# seeded synthetic inputs: numpy PCG64, drawn in fp64 in the listed order, then cast
# ---------------------------------------------------------------------------------------------
def rng(seed):
    return np.random.default_rng(seed)


def uniform_pm1(g, n):
    return g.uniform(-1.0, 1.0, n)


def normal(g, n, scale=1.0):
    return g.standard_normal(n) * scale


def grouped_sizes(seed=3, count=256):
    """Grouped workload: M = 16*U{4..128}, then N likewise, then K = 64*U{1..64} (all ``count``
    draws of one dimension before the next)."""
    g = np.random.default_rng(seed)
    M = 16 * g.integers(4, 129, count)
    N = 16 * g.integers(4, 129, count)
    K = 64 * g.integers(1, 65, count)
    return g, [(int(m), int(n), int(k)) for m, n, k in zip(M, N, K)]
