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


# ---- the parity tolerance (both sides accumulate in fp32, in different orders) ----
MANT = {"fp32": 23, "fp16": 10, "bf16": 7}


def ulp_out(x, od):
    mag = np.maximum(np.abs(x), {"fp32": 2.0 ** -126, "fp16": 2.0 ** -14, "bf16": 2.0 ** -126}[od])
    return 2.0 ** (np.floor(np.log2(mag)) - MANT[od])


def assert_close(G, R, absprod, k, alpha, beta, Cm, od, rounding="rne"):
    """G: GPU result (m x n, exact fp32 values of the output), R: oracle fp32 result.  Truncating
    output rounding may lose a whole ulp instead of half of one."""
    G = np.asarray(G, np.float64)
    R = np.asarray(R, np.float64)
    bound = ulp_out(R, od) + 3.0 * k * 2.0 ** -24 * abs(alpha) * absprod
    if beta != 0.0 and Cm is not None:
        bound = bound + 2.0 ** -23 * np.abs(beta * np.asarray(Cm, np.float64))
    err = np.abs(G - R)
    bad = int(np.count_nonzero(err > bound))
    assert np.all(np.isfinite(G)), "non-finite output"
    assert bad == 0, f"{bad} elements beyond the bound; worst excess {float(np.max(err - bound)):.3e}"
    nw = orc.normwise_error(G, R)
    allowance = 2.0 ** -(MANT[od] + (0 if rounding == "trunc" else 1)) + 3.0 * k * 2.0 ** -24 * abs(alpha) * float(np.max(absprod)) / max(
        float(np.max(np.abs(R))), 1e-30)
    assert nw <= allowance, f"normwise {nw:.3e} > {allowance:.3e}"


def absprod_of(case):
    opA = orc.op_matrix(case["A"], case["trans_a"], case["m"], case["k"], case["lda"])
    opB = orc.op_matrix(case["B"], case["trans_b"], case["k"], case["n"], case["ldb"])
    return np.abs(opA) @ np.abs(opB)


def check_against_oracle(got_flat, case, ldd=None, rounding="rne", n_begin=0, n_end=None, threads=8):
    """Scores a GPU result (flat, exact fp32 values, leading dimension ldd) against the oracle's
    restated reference loop on columns [n_begin, n_end) with the tolerance of assert_close."""
    m, n, k = case["m"], case["n"], case["k"]
    ldd = ldd or case["ldc"]
    n_end = n if n_end is None else n_end
    ref = orc.gemm_ref_f32(case["trans_a"], case["trans_b"], m, n, k, case["alpha"], case["A"], case["lda"],
                           case["B"], case["ldb"], case["beta"], case["C"], case["ldc"], m, n_begin=n_begin,
                           n_end=n_end, threads=threads)
    G = mat(got_flat, m, n, ldd)[:, n_begin:n_end]
    R = mat(ref, m, n, m)[:, n_begin:n_end]
    opA = orc.op_matrix(case["A"], case["trans_a"], m, k, case["lda"])
    opB = orc.op_matrix(case["B"], case["trans_b"], k, n, case["ldb"])[:, n_begin:n_end]
    Cm = mat(case["C"], m, n, case["ldc"])[:, n_begin:n_end] if case["beta"] != 0 else None
    assert_close(G, R, np.abs(opA) @ np.abs(opB), k, case["alpha"], case["beta"], Cm, case["out_dtype"], rounding)
    return G, R
