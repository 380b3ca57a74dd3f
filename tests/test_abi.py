"""The C ABI without a GPU: the library loads, exports every function include/tensilelite.h declares,
its structs match the header's layout, and the host-only entry points behave (no compute call)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import tensilelite_gb300 as tl
from oracle import oracle as orc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol():
    declared = tl.exported_symbols()
    assert len(declared) >= 40
    L = tl.lib()
    missing = [s for s in declared if not hasattr(L, s)]
    assert not missing, missing


def test_no_undeclared_exports():
    out = subprocess.run(["nm", "-D", "--defined-only", tl.LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line and line.split()[-1].startswith("tl_")}
    assert exported == set(tl.exported_symbols())


def _c_sizeof(expr):
    src = f'#include "include/tensilelite.h"\n#include <stdio.h>\n#include <stddef.h>\nint main(){{printf("%zu", (size_t)({expr}));}}'
    build = os.path.join(ROOT, "tensilelite_gb300", "_build")     # the package's (git-ignored) build folder
    os.makedirs(build, exist_ok=True)
    exe = os.path.join(build, "tl_sizeof_probe")
    r = subprocess.run(["gcc", "-x", "c", "-I", ROOT, "-o", exe, "-"], input=src, text=True, capture_output=True,
                       cwd=ROOT)
    assert r.returncode == 0, r.stderr
    return int(subprocess.run([exe], capture_output=True, text=True).stdout)


def test_struct_layout_matches_header():
    assert ctypes.sizeof(tl.Problem) == _c_sizeof("sizeof(tl_gemm_problem)")
    assert ctypes.sizeof(tl.Solution) == _c_sizeof("sizeof(tl_gemm_solution)")
    assert tl.Problem.alpha.offset == _c_sizeof("offsetof(tl_gemm_problem, alpha)")
    assert tl.Problem.out_rounding.offset == _c_sizeof("offsetof(tl_gemm_problem, out_rounding)")
    assert tl.Solution.ctas.offset == _c_sizeof("offsetof(tl_gemm_solution, ctas)")
    assert tl.Solution.debug_flags.offset == _c_sizeof("offsetof(tl_gemm_solution, debug_flags)")
    assert tl.DEBUG_SKIP_LOADS == _c_sizeof("TL_DEBUG_SKIP_LOADS")


def test_tensile_kernarg_layout():
    """tl_tensile_kernarg matches the reference's Tensile argument table (src/gemmMfmaKernelWriter.h:
    321-338 with the 24-byte size prefix of src/gemmMfma.cpp:70-103): pointers at 24..56, alpha/beta
    at 56/60, strides from 64, sizes from 96; 148 bytes used."""
    offs = {"size_c": 0, "size_a": 8, "size_b": 16, "d": 24, "c": 32, "a": 40, "b": 48, "alpha_bits": 56,
            "beta_bits": 60, "stride_d0": 64, "stride_d1": 68, "stride_c0": 72, "stride_c1": 76, "stride_a0": 80,
            "stride_a1": 84, "stride_b0": 88, "stride_b1": 92, "sizes_free0": 96, "sizes_free1": 100,
            "sizes_free2": 104, "sizes_sum0": 108, "padding": 144}
    for field, off in offs.items():
        assert _c_sizeof(f"offsetof(tl_tensile_kernarg, {field})") == off, field
    assert _c_sizeof("TL_TENSILE_KERNARG_BYTES") == 148 == tl.TENSILE_KERNARG_BYTES
    buf = tl.tensile_kernarg(0x1000, 0x2000, 0x3000, 0x4000, 96, 80, 64, batch=2, alpha=0.5, beta=0.25,
                             stride_d0=160, stride_d1=12800, stride_c0=160, stride_c1=12800, stride_a0=128,
                             stride_a1=12288, stride_b0=128, stride_b1=10240)
    import struct
    assert struct.unpack_from("<4Q", buf, 24) == (0x1000, 0x2000, 0x3000, 0x4000)
    assert struct.unpack_from("<2f", buf, 56) == (0.5, 0.25)
    assert struct.unpack_from("<4I", buf, 96) == (96, 80, 2, 64)


def test_cli_help_lists_reference_options():
    """The command-line runner takes the reference's options (inc/ff_utils.h:347-361); -h needs no GPU."""
    import subprocess
    cli = os.path.join(ROOT, "tensilelite_gb300", "tensilelite")
    if not os.path.exists(cli):
        pytest.skip("CLI not built")
    out = subprocess.run([cli, "-h"], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0
    for opt in ("-d --data-type", "-m --gemm-m", "-n --gemm-n", "-k --gemm-k", "-p --padding", "-r --mfma-pttn0",
                "-s --mfma-pttn1", "-x --wave-pttn0", "-y --wave-pttn1", "-z --mfma-mn", "-u --depth-u",
                "-v --verify", "-l --loop", "-f --buffer", "-t --tensile"):
        assert opt in out.stdout, opt
    bad = subprocess.run([cli, "-q", "1"], capture_output=True, text=True, timeout=60)
    assert bad.returncode == 1 and "unknown" in bad.stderr


def test_problem_init_defaults():
    p = tl.Problem()
    tl.check(tl.lib().tl_problem_init(ctypes.byref(p), tl.BF16, tl.BF16, tl.OP_N, tl.OP_T, 480, 1024, 4096))
    assert (p.m, p.n, p.k, p.batch) == (480, 1024, 4096, 1)
    assert (p.lda, p.ldb, p.ldc, p.ldd) == (480, 1024, 480, 480)
    assert p.alpha == 1.0 and p.beta == 0.0 and p.scale_a == 1.0
    q = tl.Problem.make(64, 32, 16, dtype="fp16", trans_a=True, alpha=2.0, beta=0.5, ldd=80)
    assert q.lda == 16 and q.ldb == 16 and q.ldd == 80 and q.ldc == 80 and q.trans_a == tl.OP_T


def test_status_strings_and_errors():
    L = tl.lib()
    assert L.tl_status_string(0) == b"TL_SUCCESS"
    assert L.tl_status_string(18) == b"TL_ERR_TIMEOUT"
    assert L.tl_version() >= 10000
    with pytest.raises(tl.TLError) as e:
        tl.check(L.tl_problem_init(None, 1, 1, 0, 0, 1, 1, 1))
    assert e.value.status == tl.ERR_INVALID_ARG
    assert b"NULL" in L.tl_last_error_string()


def test_trace_argument_checks():
    """tl_set_trace needs a handle and an 8-byte aligned buffer; NULL switches it off (no GPU use)."""
    L = tl.lib()
    assert tl.TRACE_SLOTS == 16 and len(tl.TRACE_EVENTS) == tl.TRACE_SLOTS
    assert L.tl_set_trace(None, None, 0) == tl.ERR_INVALID_ARG
    h = ctypes.c_void_p()
    tl.check(L.tl_init_host(152, 232448, 0, ctypes.byref(h)))
    try:
        assert L.tl_set_trace(h, ctypes.c_void_p(0x1004), 4096) == tl.ERR_INVALID_ARG
        assert L.tl_set_trace(h, ctypes.c_void_p(0x1000), -8) == tl.ERR_INVALID_ARG
        tl.check(L.tl_set_trace(h, None, 0))
    finally:
        tl.check(L.tl_destroy(h))


@pytest.mark.parametrize("rounding", [tl.ROUND_RNE, tl.ROUND_TRUNCATE])
def test_host_convert_bf16(rounding):
    conv = np.load(os.path.join(ROOT, "tests", "golden", "converters.npz"))
    x = conv["x"]
    out = np.empty(x.shape, np.uint16)
    tl.check(tl.lib().tl_convert_host(x.ctypes.data, x.size, tl.BF16, rounding, out.ctypes.data))
    if rounding == tl.ROUND_TRUNCATE:
        assert np.array_equal(out, conv["ref_bf16"])            # the reference's cvtFP32toBF16
    else:
        assert np.array_equal(out, orc.f32_to_bf16(x, "rne"))


def test_host_convert_fp16_matches_reference():
    conv = np.load(os.path.join(ROOT, "tests", "golden", "converters.npz"))
    x = conv["x"]
    out = np.empty(x.shape, np.uint16)
    tl.check(tl.lib().tl_convert_host(x.ctypes.data, x.size, tl.FP16, tl.ROUND_RNE, out.ctypes.data))
    assert np.array_equal(out, conv["ref_f16"])                # the reference's cvtFP32toFP16


def test_header_compiles_as_c_and_cpp():
    for lang, comp in (("c", "gcc"), ("c++", "g++")):
        r = subprocess.run([comp, "-x", lang, "-fsyntax-only", "-Wall", "-Werror", "-I", ROOT, "-"],
                           input='#include "include/tensilelite.h"\n', text=True, capture_output=True, cwd=ROOT)
        assert r.returncode == 0, r.stderr


def test_header_cites_reference():
    text = open(os.path.join(ROOT, "include", "tensilelite.h")).read()
    for cite in ("src/gemmMfma.cpp", "inc/ff_gpu.h", "inc/ff_utils.h", "src/gemmMfmaKernelWriter.h"):
        assert cite in text
    assert re.search(r"TL_API tl_status tl_gemm\(", text)
