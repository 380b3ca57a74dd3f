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
    src = f'#include "include/tensilelite.h"\n#include <stdio.h>\n#include <stddef.h>\nint main(){{printf("%zu", {expr});}}'
    exe = os.path.join("/tmp", "tl_sizeof_probe")
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
