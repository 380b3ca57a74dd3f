"""Helpers for the GPU parity tests: move oracle cases to the device, run them through the C ABI,
bring results back and score them against the oracle."""
import numpy as np

import tensilelite_gb300 as tl
from oracle import oracle as orc

TORCH_DT = None


def torch_dtype(name):
    import torch
    return {"fp32": torch.float32, "fp16": torch.float16, "bf16": torch.bfloat16, "fp8": torch.uint8}[name]


def to_dev(bits, name):
    """Storage bits (numpy) -> flat CUDA tensor of the storage dtype."""
    import torch
    if name == "fp32":
        return torch.from_numpy(np.ascontiguousarray(bits, np.float32)).cuda()
    if name == "fp8":
        return torch.from_numpy(np.ascontiguousarray(bits, np.uint8)).cuda()
    t = torch.from_numpy(np.ascontiguousarray(bits, np.uint16).view(np.int16)).cuda()
    return t.view(torch_dtype(name))


def from_dev(t, name):
    """CUDA tensor -> exact fp32 values (numpy)."""
    import torch
    torch.cuda.synchronize()
    if name == "fp32":
        return t.cpu().numpy().astype(np.float32)
    bits = t.view(torch.int16).cpu().numpy().view(np.uint16)
    return orc.decode(bits, name)


def run_case(handle, case, kernel="auto", dtype=None, solution=None, rounding="rne", out_dtype=None,
             ldd=None, scale_a=1.0, scale_b=1.0):
    """Runs an oracle case (gen_golden.make_case layout) on the GPU; returns D as fp32 (flat, ldd)."""
    import torch
    dt = dtype or case.get("dtype")
    od = out_dtype or case["out_dtype"]
    m, n, k = case["m"], case["n"], case["k"]
    ldd = ldd or case["ldc"]
    A = to_dev(case["A_bits"], dt)
    B = to_dev(case["B_bits"], dt)
    C_bits = case["C_bits"] if od == case["out_dtype"] else orc.encode(case["C"], od)
    C = to_dev(C_bits, od) if case["beta"] != 0 else None
    D = torch.full((ldd * n,), float("nan"), dtype=torch_dtype(od), device="cuda")
    p = tl.Problem.make(m, n, k, dtype=dt, out_dtype=od, trans_a=case["trans_a"], trans_b=case["trans_b"],
                        alpha=case["alpha"], beta=case["beta"], lda=case["lda"], ldb=case["ldb"], ldc=case["ldc"],
                        ldd=ldd, kernel=kernel, rounding=rounding, scale_a=scale_a, scale_b=scale_b)
    handle.gemm(p, D, C, A, B, solution=solution)
    handle.device_status()
    return from_dev(D, od)


def oracle_ref(case, ldd=None):
    return orc.gemm_ref_f32(case["trans_a"], case["trans_b"], case["m"], case["n"], case["k"], case["alpha"],
                            case["A"], case["lda"], case["B"], case["ldb"], case["beta"], case["C"], case["ldc"],
                            ldd or case["m"])


def oracle_f64(case):
    return orc.gemm_f64(case["trans_a"], case["trans_b"], case["m"], case["n"], case["k"], case["alpha"],
                        case["A"], case["lda"], case["B"], case["ldb"], case["beta"], case["C"], case["ldc"],
                        case["m"])


def mat(flat, m, n, ld):
    return np.asarray(flat).reshape(n, ld)[:, :m].T


def ulp_diff_count(got, ref, out_dtype):
    """Elements whose value differs from the oracle's by more than one ulp of the output type."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    mant = {"fp32": 23, "fp16": 10, "bf16": 7}[out_dtype]
    mag = np.maximum(np.abs(ref), {"fp32": 2.0 ** -126, "fp16": 2.0 ** -14, "bf16": 2.0 ** -126}[out_dtype])
    ulp = 2.0 ** (np.floor(np.log2(mag)) - mant)
    return int(np.count_nonzero(np.abs(got - ref) > 1.0 * ulp + 1e-30))


def quantize_out(vals_f32, out_dtype, rounding="rne"):
    """Round oracle fp32 results the way the kernel's epilogue does (for ulp comparisons)."""
    if out_dtype == "fp32":
        return np.asarray(vals_f32, np.float32)
    bits = orc.encode(np.asarray(vals_f32, np.float32), out_dtype, bf16_rounding=rounding)
    return orc.decode(bits, out_dtype)
