"""tensilelite_gb300 -- GEMM library for one GB300 (sm_103a), Python side.

The compute lives in ``libtensilelite_gb300.so`` (hand-written CUDA: tcgen05/TMEM/TMA tensor-core
GEMM, a CUDA-core FP32 GEMM, split/quantise helpers) behind the C ABI declared in
``include/tensilelite.h``.  This module binds that ABI with ctypes and adds:

* ``Problem`` / ``Solution`` -- the reference's problem and solution description
  (T_GemmMfmaKernelParam, src/gemmMfmaKernelWriter.h:11-22, plus transpose flags and alpha/beta);
* ``Handle.gemm`` -- one GEMM on raw device pointers (the reference's launch,
  src/gemmMfma.cpp:104-168 + ff_gpu_src/ff_hip_runtime.cpp:278-320);
* ``gemm_colmajor`` -- the same on torch tensors holding column-major buffers;
* ``matmul`` -- a ``torch.autograd.Function`` whose forward and backward run on the NN/TN/NT
  kernels (forward Y = X W is NN, dX is TN, dW is NT).

There is no fallback: if the library is not built, importing raises.  Build it with
``tensilelite_gb300._build.build()`` (``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libtensilelite_gb300.so")

# status codes (include/tensilelite.h)
SUCCESS, WARN, ERR, FATAL = 0, 1, 2, 3
ERR_INVALID_ARG, ERR_UNSUPPORTED, ERR_TIMEOUT, ERR_CUDA, ERR_ALLOC = 16, 17, 18, 19, 20

# dtype codes: 1..3 are the reference's -d codes
FP32, FP16, BF16, FP8 = 1, 2, 3, 4
OP_N, OP_T = 0, 1
KERNEL_AUTO, KERNEL_SIMT, KERNEL_TCGEN05, KERNEL_BF16X3, KERNEL_BF16X6 = 0, 1, 2, 3, 4
ROUND_RNE, ROUND_TRUNCATE = 0, 1
DEBUG_SKIP_LOADS = 1   # tl_gemm_solution.debug_flags: the producer issues no copies (timeout-path tests)
# device timeline (Handle.set_trace): words per CTA and their events (include/tensilelite.h)
TRACE_SLOTS = 16
TRACE_EVENTS = ("entry", "entry_ns", "setup", "dep", "load_first", "load_last", "mma_first", "mma_last",
                "acc_ready", "stored", "reduced", "epi_end", "exit", "exit_ns", "smid", "tiles")

DTYPE_BYTES = {FP32: 4, FP16: 2, BF16: 2, FP8: 1}
DTYPE_NAMES = {"fp32": FP32, "fp16": FP16, "bf16": BF16, "fp8": FP8, "fp8_e4m3": FP8}
KERNEL_NAMES = {"auto": KERNEL_AUTO, "simt": KERNEL_SIMT, "tcgen05": KERNEL_TCGEN05, "bf16x3": KERNEL_BF16X3,
                "bf16x6": KERNEL_BF16X6}


class TLError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{_status_name(status)}: {msg}")
        self.status = status


def _status_name(st):
    return {0: "TL_SUCCESS", 1: "TL_WARN", 2: "TL_ERR", 3: "TL_FATAL", 16: "TL_ERR_INVALID_ARG",
            17: "TL_ERR_UNSUPPORTED", 18: "TL_ERR_TIMEOUT", 19: "TL_ERR_CUDA", 20: "TL_ERR_ALLOC"}.get(st, str(st))


class Problem(ctypes.Structure):
    """tl_gemm_problem.  Sizes/strides in elements; column-major; op(A) m x k, op(B) k x n."""
    _fields_ = [("dtype_a", ctypes.c_int32), ("dtype_b", ctypes.c_int32), ("dtype_c", ctypes.c_int32),
                ("dtype_d", ctypes.c_int32), ("trans_a", ctypes.c_int32), ("trans_b", ctypes.c_int32),
                ("m", ctypes.c_int64), ("n", ctypes.c_int64), ("k", ctypes.c_int64), ("batch", ctypes.c_int64),
                ("lda", ctypes.c_int64), ("ldb", ctypes.c_int64), ("ldc", ctypes.c_int64), ("ldd", ctypes.c_int64),
                ("stride_a", ctypes.c_int64), ("stride_b", ctypes.c_int64), ("stride_c", ctypes.c_int64),
                ("stride_d", ctypes.c_int64), ("alpha", ctypes.c_float), ("beta", ctypes.c_float),
                ("scale_a", ctypes.c_float), ("scale_b", ctypes.c_float), ("kernel", ctypes.c_int32),
                ("out_rounding", ctypes.c_int32)]

    @classmethod
    def make(cls, m, n, k, *, dtype="bf16", out_dtype=None, trans_a=False, trans_b=False, alpha=1.0, beta=0.0,
             lda=None, ldb=None, ldc=None, ldd=None, batch=1, stride_a=None, stride_b=None, stride_c=None,
             stride_d=None, kernel="auto", rounding="rne", scale_a=1.0, scale_b=1.0):
        p = cls()
        dt = DTYPE_NAMES[dtype] if isinstance(dtype, str) else dtype
        od = dt if out_dtype is None else (DTYPE_NAMES[out_dtype] if isinstance(out_dtype, str) else out_dtype)
        if od == FP8 and out_dtype is None:
            od = BF16          # fp8 operands default to a bf16 output; ask for out_dtype="fp8" explicitly
        ta, tb = OP_T if trans_a else OP_N, OP_T if trans_b else OP_N
        check(lib().tl_problem_init(ctypes.byref(p), dt, od, ta, tb, m, n, k))
        p.batch = batch
        for name, val in (("lda", lda), ("ldb", ldb), ("ldc", ldc), ("ldd", ldd)):
            if val is not None:
                setattr(p, name, val)
        if ldd is not None and ldc is None:
            p.ldc = ldd
        p.stride_a = stride_a if stride_a is not None else p.lda * (k if ta == OP_N else m)
        p.stride_b = stride_b if stride_b is not None else p.ldb * (n if tb == OP_N else k)
        p.stride_c = stride_c if stride_c is not None else p.ldc * n
        p.stride_d = stride_d if stride_d is not None else p.ldd * n
        p.alpha, p.beta = alpha, beta
        p.scale_a, p.scale_b = scale_a, scale_b
        p.kernel = KERNEL_NAMES[kernel] if isinstance(kernel, str) else kernel
        p.out_rounding = ROUND_TRUNCATE if rounding in ("trunc", "truncate", ROUND_TRUNCATE) else ROUND_RNE
        return p

    def flops(self):
        return 2.0 * self.m * self.n * self.k * self.batch


ACTIVATIONS = {"none": 0, "relu": 1, "gelu": 2, "silu": 3}


class Epilogue(ctypes.Structure):
    """tl_epilogue: D = act(alpha*op(A)*op(B) + beta*C + bias[row]); max |D| into *amax."""
    _fields_ = [("bias", ctypes.c_void_p), ("bias_dtype", ctypes.c_int32), ("activation", ctypes.c_int32),
                ("amax", ctypes.c_void_p), ("d_scale", ctypes.c_float), ("reserved", ctypes.c_int32 * 3)]


class Solution(ctypes.Structure):
    """tl_gemm_solution: macro tile MT0 x MT1, depth_u, stages (lds_buffer_num), wave tile, split_k."""
    _fields_ = [("kernel", ctypes.c_int32), ("macro_tile0", ctypes.c_int32), ("macro_tile1", ctypes.c_int32),
                ("depth_u", ctypes.c_int32), ("stages", ctypes.c_int32), ("wave_tile0", ctypes.c_int32),
                ("wave_tile1", ctypes.c_int32), ("split_k", ctypes.c_int32), ("raster", ctypes.c_int32),
                ("ctas", ctypes.c_int32), ("promote_k", ctypes.c_int32),
                ("tail_split", ctypes.c_int32), ("debug_flags", ctypes.c_int32), ("reserved", ctypes.c_int32 * 3)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved"}

    def __repr__(self):
        return "Solution(%s)" % ", ".join(f"{k}={v}" for k, v in self.as_dict().items())


_LIB = None
_vp = ctypes.c_void_p


def lib():
    """The loaded C library; raises if it was not built (there is no fallback path)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is not built; run tensilelite_gb300._build.build() first")
    L = ctypes.CDLL(LIB_PATH)
    P, S = ctypes.POINTER(Problem), ctypes.POINTER(Solution)
    i64, i32, f32 = ctypes.c_int64, ctypes.c_int, ctypes.c_float
    sig = {
        "tl_init": [ctypes.POINTER(_vp)], "tl_init_host": [i32, ctypes.c_size_t, i32, ctypes.POINTER(_vp)],
        "tl_destroy": [_vp], "tl_device_info": [_vp, ctypes.POINTER(i32),
        ctypes.POINTER(i32), ctypes.POINTER(i32), ctypes.POINTER(ctypes.c_size_t)],
        "tl_problem_init": [P, i32, i32, i32, i32, i64, i64, i64],
        "tl_default_solution": [_vp, P, S], "tl_check_solution": [_vp, P, S],
        "tl_gemm": [_vp, P, S, _vp, _vp, _vp, _vp, _vp],
        "tl_tune": [_vp, P, _vp, _vp, _vp, _vp, i32, i32, ctypes.c_char_p, S, ctypes.POINTER(f32)],
        "tl_load_solutions": [_vp, ctypes.c_char_p, ctypes.POINTER(i32)],
        "tl_grouped_plan_create": [_vp, P, i32, ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_vp),
                                   ctypes.POINTER(_vp), S, ctypes.POINTER(_vp)],
        "tl_grouped_plan_launch": [_vp, _vp], "tl_grouped_plan_destroy": [_vp],
        "tl_grouped_plan_info": [_vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(i64), S],
        "tl_gemm_grouped": [_vp, P, i32, ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_vp),
                            ctypes.POINTER(_vp), _vp],
        "tl_tune_grouped": [_vp, P, i32, ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_vp),
                            ctypes.POINTER(_vp), i32, S, ctypes.POINTER(f32)],
        "tl_graph_capture_grouped": [_vp, _vp, ctypes.POINTER(_vp)],
        "tl_graph_capture_gemm": [_vp, P, S, _vp, _vp, _vp, _vp, _vp, ctypes.POINTER(_vp)],
        "tl_graph_launch": [_vp, _vp], "tl_graph_destroy": [_vp],
        "tl_quantize_fp8": [_vp, i32, _vp, i64, _vp, _vp, _vp, _vp],
        "tl_split_bf16x2": [_vp, _vp, i64, _vp, _vp, _vp],
        "tl_error_norms": [_vp, i32, _vp, i64, _vp, _vp, i64, i64, i64, ctypes.POINTER(ctypes.c_double), _vp],
        "tl_malloc": [ctypes.POINTER(_vp), ctypes.c_size_t], "tl_free": [_vp],
        "tl_host_malloc": [ctypes.POINTER(_vp), ctypes.c_size_t], "tl_host_free": [_vp],
        "tl_memcpy_h2d": [_vp, _vp, ctypes.c_size_t, _vp], "tl_memcpy_d2h": [_vp, _vp, ctypes.c_size_t, _vp],
        "tl_memcpy_d2d": [_vp, _vp, ctypes.c_size_t, _vp], "tl_memset": [_vp, i32, ctypes.c_size_t, _vp],
        "tl_stream_create": [ctypes.POINTER(_vp)], "tl_stream_destroy": [_vp], "tl_stream_synchronize": [_vp],
        "tl_fill_pattern": [i32, _vp, i64, f32, _vp],
        "tl_convert_host": [_vp, i64, i32, i32, _vp],
        "tl_timer_create": [ctypes.POINTER(_vp)], "tl_timer_start": [_vp, _vp], "tl_timer_stop": [_vp, _vp],
        "tl_timer_elapsed_ms": [_vp, ctypes.POINTER(f32)], "tl_timer_destroy": [_vp],
        "tl_launch_count": [_vp, ctypes.POINTER(i64)], "tl_device_status": [_vp, _vp],
        "tl_set_kernel_timing": [_vp, i32],
        "tl_gemm_ex": [_vp, P, ctypes.POINTER(Epilogue), S, _vp, _vp, _vp, _vp, _vp],
        "tl_tensile_launch": [_vp, ctypes.c_char_p, _vp, ctypes.c_size_t, _vp],
        "tl_kernel_timing": [_vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(i64), i32],
        "tl_set_wait_timeout": [_vp, ctypes.c_uint32],
        "tl_set_trace": [_vp, _vp, ctypes.c_int64],
        "tl_gemm_noalloc": [P, S, _vp, _vp, _vp, _vp, _vp],
        "tl_noalloc_status": [_vp],
    }
    for name, argt in sig.items():
        fn = getattr(L, name)
        fn.argtypes = argt
        fn.restype = ctypes.c_int
    L.tl_last_error_string.restype = ctypes.c_char_p
    L.tl_last_error_string.argtypes = []
    L.tl_status_string.restype = ctypes.c_char_p
    L.tl_status_string.argtypes = [ctypes.c_int]
    L.tl_version.restype = ctypes.c_int
    L.tl_version.argtypes = []
    _LIB = L
    return L


TENSILE_KERNARG_BYTES = 148


def tensile_kernarg(D, C, A, B, m, n, k, *, batch=1, alpha=1.0, beta=0.0, half_scalars=False, stride_d0, stride_d1,
                    stride_c0, stride_c1, stride_a0, stride_a1, stride_b0, stride_b1, size_c=0, size_a=0, size_b=0):
    """Packs the reference's Tensile-layout argument buffer (148 bytes; tl_tensile_kernarg)."""
    import struct
    import numpy as np
    if half_scalars:
        ab = [int(np.array(x, np.float16).view(np.uint16)) for x in (alpha, beta)]
    else:
        ab = [int(np.array(x, np.float32).view(np.uint32)) for x in (alpha, beta)]
    buf = struct.pack("<3Q4Q2I8I4I9I", size_c, size_a, size_b, _ptr(D) or 0, _ptr(C) or 0, _ptr(A) or 0,
                      _ptr(B) or 0, ab[0], ab[1], stride_d0, stride_d1, stride_c0, stride_c1, stride_a0, stride_a1,
                      stride_b0, stride_b1, m, n, batch, k, *([0] * 9))
    assert len(buf) == TENSILE_KERNARG_BYTES
    return buf


def exported_symbols() -> list:
    """Every function include/tensilelite.h declares (used to check the library's exports)."""
    import re
    hdr = os.path.join(os.path.dirname(_HERE), "include", "tensilelite.h")
    with open(hdr) as f:
        text = f.read()
    return sorted(set(re.findall(r"TL_API\s+[\w\s\*]+?\b(tl_\w+)\s*\(", text)))


def check(status: int):
    if status != SUCCESS:
        msg = lib().tl_last_error_string().decode(errors="replace")
        raise TLError(status, msg)


def _ptr(x) -> Optional[int]:
    """Device address of a torch tensor / int / None."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    return x.data_ptr()


def _stream_ptr(stream) -> Optional[int]:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


class Handle:
    """tl_handle on the current CUDA device (the reference's GpuRuntime, per device not global)."""

    def __init__(self):
        h = _vp()
        check(lib().tl_init(ctypes.byref(h)))
        self._h = h

    @classmethod
    def planning(cls, sm_count=152, smem_optin=232448, clusters4=36):
        """A planning handle for a described device (tl_init_host; defaults: a GB300): solution
        heuristics and legality checks without a GPU.  Calls that launch, allocate or time work raise."""
        self = cls.__new__(cls)
        h = _vp()
        check(lib().tl_init_host(sm_count, smem_optin, clusters4, ctypes.byref(h)))
        self._h = h
        return self

    def close(self):
        if getattr(self, "_h", None):
            lib().tl_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def ptr(self):
        return self._h

    def device_info(self):
        sm, ma, mi, sh = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_size_t()
        check(lib().tl_device_info(self._h, ctypes.byref(sm), ctypes.byref(ma), ctypes.byref(mi), ctypes.byref(sh)))
        return {"sm_count": sm.value, "cc": (ma.value, mi.value), "smem_optin": sh.value}

    def default_solution(self, p: Problem) -> Solution:
        s = Solution()
        check(lib().tl_default_solution(self._h, ctypes.byref(p), ctypes.byref(s)))
        return s

    def check_solution(self, p: Problem, s: Solution) -> None:
        check(lib().tl_check_solution(self._h, ctypes.byref(p), ctypes.byref(s)))

    def gemm(self, p: Problem, D, C, A, B, solution: Optional[Solution] = None, stream=None):
        check(lib().tl_gemm(self._h, ctypes.byref(p), ctypes.byref(solution) if solution is not None else None,
                            _ptr(D), _ptr(C), _ptr(A), _ptr(B), _stream_ptr(stream)))

    def tune(self, p: Problem, D, C, A, B, max_candidates=16, reps=10, cache_path=None):
        s, ms = Solution(), ctypes.c_float()
        check(lib().tl_tune(self._h, ctypes.byref(p), _ptr(D), _ptr(C), _ptr(A), _ptr(B), max_candidates, reps,
                            cache_path.encode() if cache_path else None, ctypes.byref(s), ctypes.byref(ms)))
        return s, ms.value

    def load_solutions(self, path):
        n = ctypes.c_int()
        check(lib().tl_load_solutions(self._h, path.encode(), ctypes.byref(n)))
        return n.value

    def quantize_fp8(self, src, n, dst, scale_out=None, amax_out=None, src_dtype=FP32, stream=None):
        check(lib().tl_quantize_fp8(self._h, src_dtype, _ptr(src), n, _ptr(dst), _ptr(scale_out), _ptr(amax_out),
                                    _stream_ptr(stream)))

    def split_bf16x2(self, src, n, hi, lo, stream=None):
        check(lib().tl_split_bf16x2(self._h, _ptr(src), n, _ptr(hi), _ptr(lo), _stream_ptr(stream)))

    def error_norms(self, dtype_d, D, ldd, R, ldr, m, n, W=None, stream=None):
        out = (ctypes.c_double * 3)()
        check(lib().tl_error_norms(self._h, dtype_d, _ptr(D), ldd, _ptr(R), _ptr(W), ldr, m, n, out,
                                   _stream_ptr(stream)))
        return out[0], out[1], out[2]

    def launch_count(self):
        n = ctypes.c_int64()
        check(lib().tl_launch_count(self._h, ctypes.byref(n)))
        return n.value

    def gemm_ex(self, p: Problem, D, C, A, B, bias=None, bias_dtype=None, activation="none", amax=None,
                d_scale=0.0, solution: Optional[Solution] = None, stream=None):
        """tl_gemm_ex: tl_gemm with a fused bias / activation / amax epilogue (and, for an fp8 output,
        the quantisation scale d_scale)."""
        e = Epilogue()
        e.d_scale = d_scale
        e.bias = _ptr(bias)
        if bias is not None and bias_dtype is None:
            bias_dtype = torch_dtype_code(bias.dtype)
        e.bias_dtype = (DTYPE_NAMES[bias_dtype] if isinstance(bias_dtype, str) else bias_dtype) or FP32
        e.activation = ACTIVATIONS[activation] if isinstance(activation, str) else int(activation)
        e.amax = _ptr(amax)
        check(lib().tl_gemm_ex(self._h, ctypes.byref(p), ctypes.byref(e),
                               ctypes.byref(solution) if solution is not None else None,
                               _ptr(D), _ptr(C), _ptr(A), _ptr(B), _stream_ptr(stream)))

    def tensile_launch(self, kernel_name: str, kernarg: bytes, stream=None):
        """tl_tensile_launch: the GEMM a Tensile-layout (Cijk_Alik_Bljk) argument buffer describes."""
        buf = ctypes.create_string_buffer(bytes(kernarg), len(kernarg))
        check(lib().tl_tensile_launch(self._h, kernel_name.encode(), ctypes.cast(buf, _vp), len(kernarg),
                                      _stream_ptr(stream)))

    def set_kernel_timing(self, enable: bool):
        """Record an event pair around every GEMM kernel launch (see tl_set_kernel_timing)."""
        check(lib().tl_set_kernel_timing(self._h, 1 if enable else 0))

    def kernel_timing(self, reset=True):
        """(summed kernel milliseconds, timed launches) since the last reset; waits for them."""
        ms, n = ctypes.c_double(), ctypes.c_int64()
        check(lib().tl_kernel_timing(self._h, ctypes.byref(ms), ctypes.byref(n), 1 if reset else 0))
        return ms.value, n.value

    def device_status(self, stream=None):
        check(lib().tl_device_status(self._h, _stream_ptr(stream)))

    def set_wait_timeout(self, ms):
        check(lib().tl_set_wait_timeout(self._h, ms))

    def set_trace(self, buffer=None):
        """Device timeline of the tensor-core kernel (tl_set_trace): `buffer` is an int64 device tensor
        of at least grid x TRACE_SLOTS elements, or None to switch it off."""
        if buffer is None:
            check(lib().tl_set_trace(self._h, None, 0))
        else:
            check(lib().tl_set_trace(self._h, _ptr(buffer), buffer.numel() * buffer.element_size()))

    # ---- grouped ----
    def grouped_plan(self, problems: Sequence[Problem], D, C, A, B, solution: Optional[Solution] = None):
        return GroupedPlan(self, problems, D, C, A, B, solution)

    def tune_grouped(self, problems, D, C, A, B, reps=5):
        n = len(problems)
        arr = (Problem * n)(*problems)
        s, ms = Solution(), ctypes.c_float()
        check(lib().tl_tune_grouped(self._h, arr, n, _ptr_array(D), _ptr_array(C), _ptr_array(A), _ptr_array(B),
                                    reps, ctypes.byref(s), ctypes.byref(ms)))
        return s, ms.value

    def capture_gemm(self, p: Problem, D, C, A, B, solution=None, stream=None):
        g = _vp()
        check(lib().tl_graph_capture_gemm(self._h, ctypes.byref(p), ctypes.byref(solution) if solution else None,
                                          _ptr(D), _ptr(C), _ptr(A), _ptr(B), _stream_ptr(stream), ctypes.byref(g)))
        return Graph(g)


def _ptr_array(xs):
    if xs is None:
        return None
    arr = (_vp * len(xs))()
    for i, x in enumerate(xs):
        arr[i] = _ptr(x)
    return arr


class Graph:
    def __init__(self, g):
        self._g = g

    def launch(self, stream=None):
        check(lib().tl_graph_launch(self._g, _stream_ptr(stream)))

    def close(self):
        if self._g:
            lib().tl_graph_destroy(self._g)
            self._g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GroupedPlan:
    """tl_grouped_plan: one persistent launch over many independent problems."""

    def __init__(self, handle: Handle, problems, D, C, A, B, solution=None):
        n = len(problems)
        self._keep = (problems, D, C, A, B)
        arr = (Problem * n)(*problems)
        plan = _vp()
        check(lib().tl_grouped_plan_create(handle.ptr, arr, n, _ptr_array(D), _ptr_array(C), _ptr_array(A),
                                           _ptr_array(B), ctypes.byref(solution) if solution else None,
                                           ctypes.byref(plan)))
        self._plan = plan
        self.handle = handle

    def launch(self, stream=None):
        check(lib().tl_grouped_plan_launch(self._plan, _stream_ptr(stream)))

    def capture(self, stream) -> Graph:
        g = _vp()
        check(lib().tl_graph_capture_grouped(self._plan, _stream_ptr(stream), ctypes.byref(g)))
        return Graph(g)

    def info(self):
        fl, tiles, s = ctypes.c_double(), ctypes.c_int64(), Solution()
        check(lib().tl_grouped_plan_info(self._plan, ctypes.byref(fl), ctypes.byref(tiles), ctypes.byref(s)))
        return fl.value, tiles.value, s

    def close(self):
        if self._plan:
            lib().tl_grouped_plan_destroy(self._plan)
            self._plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def gemm_noalloc(p: Problem, D, C, A, B, solution: Optional[Solution] = None, stream=None):
    """tl_gemm_noalloc: the tensor-core GEMM with its split-k scratch in the library's static device
    array (no allocation, no handle)."""
    check(lib().tl_gemm_noalloc(ctypes.byref(p), ctypes.byref(solution) if solution is not None else None,
                                _ptr(D), _ptr(C), _ptr(A), _ptr(B), _stream_ptr(stream)))


def noalloc_status(stream=None):
    """tl_noalloc_status: raises TLError(ERR_TIMEOUT) when the last tl_gemm_noalloc call on the current
    device ran out a device wait (and clears the record)."""
    check(lib().tl_noalloc_status(_stream_ptr(stream)))


_DEFAULT_HANDLE = {}


def default_handle() -> Handle:
    import torch
    dev = torch.cuda.current_device()
    h = _DEFAULT_HANDLE.get(dev)
    if h is None:
        h = Handle()
        _DEFAULT_HANDLE[dev] = h
    return h


def torch_dtype_code(t) -> int:
    import torch
    return {torch.float32: FP32, torch.float16: FP16, torch.bfloat16: BF16,
            torch.float8_e4m3fn: FP8, torch.uint8: FP8}[t]


def gemm_colmajor(A, B, m, n, k, *, C=None, D=None, alpha=1.0, beta=0.0, trans_a=False, trans_b=False,
                  lda=None, ldb=None, ldc=None, ldd=None, out_dtype=None, kernel="auto", rounding="rne",
                  scale_a=1.0, scale_b=1.0, solution=None, handle=None, stream=None):
    """D = alpha op(A) op(B) + beta C on torch CUDA tensors holding column-major buffers."""
    import torch
    dt = torch_dtype_code(A.dtype)
    od = out_dtype if out_dtype is not None else (dt if dt != FP8 else BF16)
    if isinstance(od, str):
        od = DTYPE_NAMES[od]
    p = Problem.make(m, n, k, dtype=dt, out_dtype=od, trans_a=trans_a, trans_b=trans_b, alpha=alpha, beta=beta,
                     lda=lda, ldb=ldb, ldc=ldc, ldd=ldd, kernel=kernel, rounding=rounding, scale_a=scale_a,
                     scale_b=scale_b)
    if D is None:
        tdt = {FP32: torch.float32, FP16: torch.float16, BF16: torch.bfloat16}[od]
        D = torch.empty(p.ldd * n, dtype=tdt, device=A.device)
    (handle or default_handle()).gemm(p, D, C, A, B, solution=solution, stream=stream)
    return D


_MM_PROBLEMS = {}


def _mm_rowmajor(X, W, trans_x=False, trans_w=False):
    """Row-major X(M,K) @ W(K,N) through the column-major kernels (op flags on the stored tensors).
    The problem descriptor is built once per (dtype, layout, shape) and reused: the per-call host cost
    is then the two tensor-map encodings and the launch."""
    import torch
    Xs, Ws = X.contiguous(), W.contiguous()
    M = Xs.shape[1] if trans_x else Xs.shape[0]
    K = Xs.shape[0] if trans_x else Xs.shape[1]
    N = Ws.shape[0] if trans_w else Ws.shape[1]
    key = (X.dtype, trans_x, trans_w, M, N, K)
    p = _MM_PROBLEMS.get(key)
    if p is None:
        # Y (row-major M x N) == column-major N x M:  Y^T = op(W)^T op(X)^T
        p = Problem.make(N, M, K, dtype=torch_dtype_code(X.dtype), trans_a=trans_w, trans_b=trans_x,
                         lda=Ws.shape[1], ldb=Xs.shape[1], ldd=N)
        _MM_PROBLEMS[key] = p
    Y = torch.empty((M, N), dtype=X.dtype, device=X.device)
    default_handle().gemm(p, Y, None, Ws, Xs)
    return Y


class _Matmul:
    pass


def _make_autograd():
    import torch

    class TLMatmul(torch.autograd.Function):
        """Y = X @ W on the library's kernels.
        Forward  Y^T  = W^T X^T       -> NN, (m, n, k) = (N, M, K), A = W, B = X
        dX^T = W dY^T                  -> TN, (m, n, k) = (K, M, N), A = W, B = dY
        dW^T = dY^T X                  -> NT, (m, n, k) = (N, K, M), A = dY, B = X   (column-major view)
        """

        @staticmethod
        def forward(ctx, X, W):
            ctx.save_for_backward(X, W)
            return _mm_rowmajor(X, W)

        @staticmethod
        def backward(ctx, dY):
            X, W = ctx.saved_tensors
            dY = dY.contiguous()
            dX = dW = None
            if ctx.needs_input_grad[0]:
                dX = _mm_rowmajor(dY, W, trans_w=True)       # dY (M,N) @ W^T (N,K)
            if ctx.needs_input_grad[1]:
                dW = _mm_rowmajor(X, dY, trans_x=True)       # X^T (K,M) @ dY (M,N)
            return dX, dW

    return TLMatmul


_TLMatmul = None


def linear(X, W, bias=None, activation="none", amax=None):
    """Inference-only fused Y = act(X @ W + bias) on the tensor-core kernel (row-major X (M, K),
    W (K, N), bias (N,)); `amax`, a one-element float32 CUDA tensor, receives max |Y| (atomically
    maxed into it).  No autograd."""
    import torch
    Xs, Ws = X.contiguous(), W.contiguous()
    M, K = Xs.shape
    N = Ws.shape[1]
    Y = torch.empty((M, N), dtype=X.dtype, device=X.device)
    # Y^T = W^T X^T column-major: m = N (bias index), n = M
    p = Problem.make(N, M, K, dtype=torch_dtype_code(X.dtype), lda=N, ldb=K, ldd=N)
    default_handle().gemm_ex(p, Y, None, Ws, Xs, bias=bias, activation=activation, amax=amax)
    return Y


def matmul(X, W):
    """Differentiable X @ W (2-D, fp16/bf16/fp32) on the tensor-core / CUDA-core kernels."""
    global _TLMatmul
    if _TLMatmul is None:
        _TLMatmul = _make_autograd()
    return _TLMatmul.apply(X, W)
