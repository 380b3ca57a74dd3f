"""bench.py -- GEMM throughput on GB300 through the library's C ABI.

Default workload (the configuration the headline metric is quoted on): bf16 GEMM, M = N = K = 4096,
NN column-major, alpha = 1, beta = 0.5, A, B, C ~ N(0,1) from numpy PCG64 seed 1 (drawn A, B, C),
cast to bf16 (RNE), fp32 accumulation, bf16 output.  One step = one GEMM launch.

  value      device throughput (TFLOP/s, 2*M*N*K per step) with inputs resident in HBM; K steps
             timed with CUDA events on the launching stream, rotating over copies of the inputs
             (together at least twice the 129 MB L2) so no step reads an earlier one's tiles from
             L2.  A step that is one kernel launch is timed from CUDA-graph replay of the same K
             launches (the device time; a Python-level launch costs this host several microseconds),
             with the eager figure beside it.
  e2e        the same GEMM through the public API with host buffers: per step the pinned-host A,
             B, C are copied in (tl_memcpy_h2d), the GEMM runs, D is copied out (tl_memcpy_d2h);
             with the host link's own pinned bandwidth beside it (copy_bound), the rate e2e cannot beat.
  roofline   the tcgen05 kernel against the measured dense bf16 peak (MEASURED_PEAKS.json).
  cpu_baseline  the reference's CPU GEMM loop (src/gemmMfma.cpp:313-346, restated in oracle/) on
             a bounded sample of output columns of the same problem, all host threads, and on one
             thread as the reference runs it; the host's CPU model is named.
  suite      (default run only) the other configurations, measured after the headline: fp16 and the
             other bf16 layouts at 4096^3 (and NN with beta = 0, which runs as the transposed TT
             product), bf16 480x1024x4096, fp8 8192^3, the 256-problem grouped
             launch, forward+backward, bf16x3 / bf16x6 / CUDA-core fp32 at 8192^3 and the CUDA-core
             480x512x512 case -- throughput, roofline fraction and FP64 error of each.

Other workloads (--workload): fp16_4096_nn|nt|tn, bf16_4096_nt|tn|nn_b0, bf16_480x1024x4096, bf16x3_8192,
simt_fp32_8192, fp8_8192, grouped256, fwdbwd.  `--impl reference` times the reference's CPU loop
(the oracle port) on the same workload instead.

One GPU only.  The library is a single-device GEMM (the reference has no multi-device path either),
and its cluster-of-four kernel loads through TMA multicast, which is kept to one-GPU runs.  Launched
with WORLD_SIZE > 1 (torchrun), the GPU arm prints one line saying so on rank 0 and every rank exits
without touching a GPU; the reference arm (host cores only) runs on rank 0 alone.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GEMM TFLOP/s & %peak per dtype; bf16x3 vs plain FP32 at matched FP64 error"
L2_BYTES = 129e6      # GB300 L2


# ----------------------------------------------------------------------------------------------
# workloads
# ----------------------------------------------------------------------------------------------
WORKLOADS = {
    "bf16_4096_nn": dict(dtype="bf16", m=4096, n=4096, k=4096, lay="NN", alpha=1.0, beta=0.5, seed=1, dist="normal"),
    "bf16_4096_nn_b0": dict(dtype="bf16", m=4096, n=4096, k=4096, lay="NN", alpha=1.0, beta=0.0, seed=1, dist="normal",
                            no_profile=True),
    "bf16_4096_nt": dict(dtype="bf16", m=4096, n=4096, k=4096, lay="NT", alpha=1.0, beta=0.5, seed=1, dist="normal"),
    "bf16_4096_tn": dict(dtype="bf16", m=4096, n=4096, k=4096, lay="TN", alpha=1.0, beta=0.5, seed=1, dist="normal"),
    "fp16_4096_nn": dict(dtype="fp16", m=4096, n=4096, k=4096, lay="NN", alpha=1.0, beta=0.5, seed=1, dist="normal"),
    "fp16_4096_nt": dict(dtype="fp16", m=4096, n=4096, k=4096, lay="NT", alpha=1.0, beta=0.5, seed=1, dist="normal"),
    "fp16_4096_tn": dict(dtype="fp16", m=4096, n=4096, k=4096, lay="TN", alpha=1.0, beta=0.5, seed=1, dist="normal"),
    "bf16_480x1024x4096": dict(dtype="bf16", m=480, n=1024, k=4096, lay="NN", alpha=1.0, beta=0.5, seed=1,
                               dist="normal"),
    "bf16x3_8192": dict(dtype="fp32", m=8192, n=8192, k=8192, lay="NN", alpha=1.0, beta=0.0, seed=2,
                        dist="uniform", kernel="bf16x3", steps=300),
    "bf16x6_8192": dict(dtype="fp32", m=8192, n=8192, k=8192, lay="NN", alpha=1.0, beta=0.0, seed=2,
                        dist="uniform", kernel="bf16x6", steps=200),
    "simt_fp32_8192": dict(dtype="fp32", m=8192, n=8192, k=8192, lay="NN", alpha=1.0, beta=0.0, seed=2,
                           dist="uniform", kernel="simt", steps=50),
    "grouped256": dict(kind="grouped", dtype="bf16", count=256, seed=3, lay="NN", alpha=1.0, beta=0.0,
                       steps=1000),
    "fwdbwd": dict(kind="fwdbwd", dtype="bf16", m=4096, k=1024, n=4096, seed=4),
    "fp8_8192": dict(dtype="fp8", m=8192, n=8192, k=8192, lay="TN", alpha=1.0, beta=0.0, seed=2, dist="normal",
                     steps=2000),
    "simt_fp32_480x512x512": dict(dtype="fp32", m=480, n=512, k=512, lay="NN", alpha=1.0, beta=0.0, seed=0,
                                  dist="uniform", kernel="simt"),
}


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "bf16_tflops": float(d["bf16_tflops"]),
                "bf16_tflops_sustained": float(d.get("bf16_tflops_sustained", d["bf16_tflops"])), "source": "measured"}
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "source": "fallback"}


def profile_traffic(kernel_tag):
    """dram bytes per launch recorded from an ncu capture in profiles/ (line 'traffic_bytes_per_launch: N')."""
    d = os.path.join(ROOT, "profiles")
    if not os.path.isdir(d):
        return None
    for name in sorted(os.listdir(d)):
        if kernel_tag in name and name.endswith((".txt", ".md")):
            with open(os.path.join(d, name)) as f:
                m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", f.read())
            if m:
                return float(m.group(1))
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms while active."""

    FIELDS = ("clocks.sm,clocks.max.sm,utilization.gpu,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.rows.append(parts)

    def mark(self):
        return len(self.rows)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)

    def summary(self, start=0, end=None):
        rows = self.rows[start:end] if end is not None else self.rows[start:]
        if not rows:
            rows = self.rows
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        load = [r for r in rows if (num(r[2]) or 0) > 0] or rows
        sm = [num(r[0]) for r in load if num(r[0]) is not None]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for i, nm in enumerate(names):
                if r[4 + i].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": num(rows[0][1]),
                "reasons": sorted(reasons), "samples": len(load),
                "power_w_max": max((num(r[3]) or 0) for r in rows)}


# ----------------------------------------------------------------------------------------------
# input generation (host, numpy PCG64)
# ----------------------------------------------------------------------------------------------
def host_inputs(w):
    g = np.random.default_rng(w["seed"])
    m, n, k = w["m"], w["n"], w["k"]
    ta, tb = w["lay"][0] == "T", w["lay"][1] == "T"
    draw = (lambda c: g.uniform(-1.0, 1.0, c)) if w["dist"] == "uniform" else (lambda c: g.standard_normal(c))
    A = draw(m * k).astype(np.float32)
    B = draw(k * n).astype(np.float32)
    C = draw(m * n).astype(np.float32) if w["beta"] != 0.0 else None
    lda = k if ta else m
    ldb = n if tb else k
    return A, B, C, lda, ldb


def to_device_dtype(x, dtype):
    import torch
    t = torch.from_numpy(x).cuda()
    if dtype == "bf16":
        return t.to(torch.bfloat16)
    if dtype == "fp16":
        return t.to(torch.float16)
    return t


# ----------------------------------------------------------------------------------------------
# CPU baseline: the reference loop (oracle port) on a bounded column sample
# ----------------------------------------------------------------------------------------------
def cpu_sample_setup(w, A, B, dtype, C=None):
    """Packed TN storage (Ap[m][k], Bp[n][k]) of the values the GPU multiplies, and C (column-major
    m x n), all as fp32 (inputs rounded to the GPU dtype, then widened)."""
    import torch
    m, n, k = w["m"], w["n"], w["k"]
    ta, tb = w["lay"][0] == "T", w["lay"][1] == "T"

    def widen(x):
        if x is not None and dtype in ("bf16", "fp16"):
            tt = torch.bfloat16 if dtype == "bf16" else torch.float16
            return torch.from_numpy(x).to(tt).float().numpy()
        return x
    Aw, Bw = widen(A), widen(B)
    Ap = np.ascontiguousarray(Aw.reshape(m, k) if ta else Aw.reshape(k, m).T)          # m x k
    Bp = np.ascontiguousarray(Bw.reshape(k, n).T if tb else Bw.reshape(n, k))          # n x k
    Cw = np.ascontiguousarray(widen(C), np.float32) if C is not None else None
    return Ap.astype(np.float32), Bp.astype(np.float32), Cw


def cpu_run_columns(Ap, Bp, m, n, k, cols, threads, col0=0, alpha=1.0, beta=0.0, C=None):
    """The reference loop (alpha*sum + beta*c per element) over output columns [col0, col0 + cols)."""
    import ctypes
    from oracle import oracle as orc
    L = orc.lib()
    D = np.zeros((cols, m), np.float32)
    f32p = ctypes.POINTER(ctypes.c_float)
    Bsub = np.ascontiguousarray(Bp[col0:col0 + cols])
    use_c = C is not None and beta != 0.0
    Csub = np.ascontiguousarray(C[col0 * m:(col0 + cols) * m]) if use_c else None
    t0 = time.perf_counter()
    L.orc_gemm_ref_f32_packed(m, cols, k, ctypes.c_float(alpha), Ap.ctypes.data_as(f32p), Bsub.ctypes.data_as(f32p),
                              ctypes.c_float(beta if use_c else 0.0), Csub.ctypes.data_as(f32p) if use_c else None, m,
                              D.ctypes.data_as(f32p), m, 0, cols, threads)
    return time.perf_counter() - t0


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu part")):
                    return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def _cpu_rate(Ap, Bp, m, n, k, threads, target_s, alpha, beta, C):
    """(columns, seconds) of the loop on `threads` threads over a sample sized to about target_s."""
    c0 = min(n, max(threads, 1))
    t = cpu_run_columns(Ap, Bp, m, n, k, c0, threads, alpha=alpha, beta=beta, C=C)
    cols = int(min(n, max(c0, c0 / max(t, 1e-6) * target_s)))
    t = cpu_run_columns(Ap, Bp, m, n, k, cols, threads, alpha=alpha, beta=beta, C=C)
    return cols, t


def cpu_baseline(w, A, B, dtype, target_s=10.0, threads=None, C=None):
    """The reference's CPU GEMM loop (cpuCompute, restated) on a bounded column sample of the same
    problem: on all host threads (value) and on one thread, as the reference runs it."""
    from oracle import oracle as orc
    orc.lib()
    threads = threads or os.cpu_count() or 1
    m, n, k = w["m"], w["n"], w["k"]
    alpha, beta = w.get("alpha", 1.0), w.get("beta", 0.0)
    Ap, Bp, Cw = cpu_sample_setup(w, A, B, dtype, C)
    per_col = 2.0 * m * k
    cols, t = _cpu_rate(Ap, Bp, m, n, k, threads, target_s, alpha, beta, Cw)
    cols1, t1 = _cpu_rate(Ap, Bp, m, n, k, 1, target_s / 3.0, alpha, beta, Cw)
    model = cpu_model()
    return {"value": per_col * cols / t / 1e12, "unit": "TFLOP/s", "cores": threads, "kind": "port",
            "cpu_model": model,
            "sample": f"reference CPU loop (src/gemmMfma.cpp:313-346 restated, -O2 -ffp-contract=off: "
                      f"alpha*sum + beta*c) over {cols} of {n} output columns of the {m}x{n}x{k} problem, "
                      f"{t:.1f} s, {threads} threads ({model})",
            "seconds": t,
            "single_thread": {"value": per_col * cols1 / t1 / 1e12, "unit": "TFLOP/s", "cores": 1,
                              "sample": f"{cols1} of {n} columns, {t1:.1f} s, one thread (as the reference "
                                        f"runs cpuCompute)"}}


# ----------------------------------------------------------------------------------------------
# GPU arm (one GPU)
# ----------------------------------------------------------------------------------------------
def launch_env():
    """(world size, rank) of a torchrun launch; (1, 0) for a plain one."""
    return int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0"))


def smi_index():
    """nvidia-smi's index of the GPU this process uses (device 0 of CUDA_VISIBLE_DEVICES)."""
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0].strip()
    return int(vis) if vis.isdigit() else 0


def refusal_line(world, impl):
    return {"metric": METRIC, "impl": impl, "n_gpus": world,
            "unavailable": f"one-GPU library: bench.py runs the GPU arm on one GPU only (asked for {world}); "
                           "the library has no multi-device path and its cluster-of-four kernel uses TMA multicast, "
                           "which is kept to one-GPU runs"}


def run_gpu(args, w, name):
    import torch
    import tensilelite_gb300 as tl

    torch.cuda.set_device(0)
    h = tl.Handle()
    dtype = w["dtype"]
    m, n, k = w["m"], w["n"], w["k"]
    ta, tb = w["lay"][0] == "T", w["lay"][1] == "T"
    kernel = w.get("kernel", "tcgen05" if dtype != "fp32" else "simt")
    A, B, C, lda, ldb = host_inputs(w)
    out_dt = "bf16" if dtype == "fp8" else dtype
    tdt = {"fp32": torch.float32, "fp16": torch.float16, "bf16": torch.bfloat16}[out_dt]
    stream = torch.cuda.Stream()

    scale_a = scale_b = 1.0
    if dtype == "fp8":
        # per-tensor amax scaling on the device (tl_quantize_fp8), dequant factors folded into alpha
        dA32, dB32 = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
        qa = torch.empty(A.size, dtype=torch.uint8, device="cuda")
        qb = torch.empty(B.size, dtype=torch.uint8, device="cuda")
        sa = torch.zeros(1, device="cuda")
        sb = torch.zeros(1, device="cuda")
        h.quantize_fp8(dA32, A.size, qa, scale_out=sa)
        h.quantize_fp8(dB32, B.size, qb, scale_out=sb)
        torch.cuda.synchronize()
        scale_a, scale_b = sa.item(), sb.item()
        base = (qa, qb)
        del dA32, dB32
    else:
        base = (to_device_dtype(A, dtype), to_device_dtype(B, dtype))
    dC = to_device_dtype(C, out_dt) if C is not None else None
    p = tl.Problem.make(m, n, k, dtype=dtype, out_dtype=out_dt, trans_a=ta, trans_b=tb, alpha=w["alpha"],
                        beta=w["beta"], lda=lda, ldb=ldb, kernel=kernel, scale_a=scale_a, scale_b=scale_b)
    sol = h.default_solution(p)
    if args.tune and kernel != "simt":
        Dt = torch.empty(m * n, dtype=tdt, device="cuda")
        sol, _ = h.tune(p, Dt, dC, base[0], base[1], max_candidates=args.tune, reps=5)
        del Dt
    # rotating copies so the working set of consecutive steps exceeds L2: at least twice its 129 MB
    # pass through between two steps that use the same copy (a small problem rotates over many)
    bytes_per_set = sum(x.numel() * x.element_size() for x in base) + (dC.numel() * dC.element_size() if dC is not None
                                                                         else 0) + m * n * tdt.itemsize
    nsets = max(1, int(np.ceil(2 * L2_BYTES / bytes_per_set)))
    sets = []
    for i in range(nsets):
        a = base[0] if i == 0 else base[0].clone()
        b = base[1] if i == 0 else base[1].clone()
        c = dC if (i == 0 or dC is None) else dC.clone()
        d = torch.empty(m * n, dtype=tdt, device="cuda")
        sets.append((a, b, c, d))
    torch.cuda.synchronize()

    flops = 2.0 * m * n * k
    clocks = ClockSampler(smi_index())
    clocks.start()
    with torch.cuda.stream(stream):
        for i in range(args.warmup):
            a, b, c, d = sets[i % nsets]
            h.gemm(p, d, c, a, b, solution=sol, stream=stream)
    stream.synchronize()
    h.device_status(stream)
    time.sleep(0.2)
    torch.cuda.synchronize()
    mark0 = clocks.mark()
    launches0 = h.launch_count()
    # a split-kernel step is pre-pass + GEMM: time the GEMM kernel itself with an event pair per launch
    multi = kernel in ("bf16x3", "bf16x6")
    if multi:
        h.set_kernel_timing(True)
        h.kernel_timing(reset=True)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t_wall = time.perf_counter()
    ev0.record(stream)
    for i in range(args.steps):
        a, b, c, d = sets[i % nsets]
        h.gemm(p, d, c, a, b, solution=sol, stream=stream)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall
    launches = h.launch_count() - launches0
    mark1 = clocks.mark()
    h.device_status(stream)
    ms_total = ev0.elapsed_time(ev1)
    eager_ms_per_step = ms_total / args.steps
    timing = "eager: K calls of the public API back to back, CUDA events on the launching stream"
    if multi:
        kms, kn = h.kernel_timing(reset=True)
        h.set_kernel_timing(False)
        kernel_ms = kms / max(1, kn)
    else:
        # The same K launches captured in CUDA graphs and replayed: the device time of the steps.
        # This host issues a call from Python in several microseconds, so K eager calls of a short
        # GEMM measure the host; the graph keeps every launch (and its inputs) as it was.
        per_step = max(1, launches // max(1, args.steps))
        g_len = min(args.steps, max(64, nsets))   # one replay walks every input copy

        def capture(count, first):
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph, stream=stream):
                for i in range(first, first + count):
                    a, b, c, d = sets[i % nsets]
                    h.gemm(p, d, c, a, b, solution=sol, stream=stream)
            return graph
        full = capture(g_len, 0)
        rest_n = args.steps % g_len
        rest = capture(rest_n, 0) if rest_n else None
        with torch.cuda.stream(stream):
            full.replay()
        torch.cuda.synchronize()
        h.device_status(stream)
        for st in sets:  # all-ones bytes are NaN in every output type: the accuracy check then reads the replay
            st[3].view(torch.uint8).fill_(255)
        torch.cuda.synchronize()
        time.sleep(0.1)
        mark0 = clocks.mark()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):  # replay() launches on the current stream
            e0.record(stream)
            for _ in range(args.steps // g_len):
                full.replay()
            if rest is not None:
                rest.replay()
            e1.record(stream)
        e1.synchronize()
        mark1 = clocks.mark()
        h.device_status(stream)
        ms_total = e0.elapsed_time(e1)
        launches = per_step * args.steps
        timing = (f"CUDA-graph replay of the K launches ({g_len} per graph, inputs rotating as in the eager loop); "
                  f"eager: {eager_ms_per_step:.6f} ms per step")
    value = flops * args.steps / (ms_total / 1e3) / 1e12
    ms_per_step = ms_total / args.steps
    if not multi:
        kernel_ms = ms_per_step

    # accuracy of the benchmarked result against an FP64 host oracle (numpy float64 matmul)
    err = None
    if args.check and m * n * k <= 8192 ** 3:
        a, b, c, d = sets[(args.steps - 1) % nsets]
        try:
            err = fp64_error(h, w, A, B, C, d, out_dt, scale_a, scale_b, base)
        except Exception as e:  # keep the bench line even if the host is short of memory
            err = {"error": str(e)[:200]}

    # e2e through the public API: pinned host buffers in, result out, every step
    e2e = None
    if args.e2e_steps > 0:
        e2e = run_e2e(h, p, sol, base, dC, m, n, tdt, stream, args.e2e_steps)
    clocks.stop()
    clk = clocks.summary(mark0, mark1)
    peaks = load_peaks()
    nterms = {"bf16x3": 3, "bf16x6": 6}.get(kernel, 1)
    # tensor work actually executed: the split paths run nterms bf16 products per output
    achieved = nterms * flops / (kernel_ms / 1e3) / 1e12
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "TFLOP/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 6), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": dtype,
        "data": f"synthetic: numpy PCG64 seed {w['seed']}, {'N(0,1)' if w['dist'] == 'normal' else 'uniform[-1,1)'}",
        "config": {"workload": describe(w, name), "m": m, "n": n, "k": k, "layout": w["lay"], "alpha": w["alpha"],
                   "beta": w["beta"], "kernel": kernel, "solution": sol.as_dict(),
                   "l2": f"rotating {nsets} input sets of {bytes_per_set / 2**20:.0f} MiB (> L2 together)"
                   if nsets > 1 else "inputs larger than L2",
                   "parallelism": "1 GPU"},
        "roofline": {"bound": "tensor" if kernel != "simt" else "fp32-pipe", "achieved": round(achieved, 2),
                     "peak": (peaks["bf16_tflops"] * (2 if dtype == "fp8" else 1)) if kernel != "simt"
                     else round(nominal_fp32_tflops(), 1),
                     "unit": "TFLOP/s", "frac": None, "traffic": None,
                     "peak_source": (peaks["source"] + " bf16 burst" + (" x2 (fp8 dense = 2x bf16)" if dtype == "fp8"
                                                                          else "")) if kernel != "simt"
                     else "nominal FP32 FMA rate: SMs x 128 lanes x 2 x max SM clock",
                     "kernel_ms": round(kernel_ms, 6)},
        "clocks": clk, "gpu_launches": launches, "wall_s_timed": round(t_wall, 4), "timing": timing,
    }
    if line["roofline"]["peak"]:
        line["roofline"]["frac"] = round(achieved / line["roofline"]["peak"], 4)
    if nterms > 1:
        line["roofline"]["note"] = (f"{kernel}: {nterms} bf16 tensor products per output; achieved counts them all "
                                    f"over the GEMM kernel's own event-timed duration; value counts 2*m*n*k once "
                                    f"over the whole step (fp32 split pre-pass + GEMM)")
    tag = {"bf16": "bf16", "fp16": "fp16", "fp8": "fp8", "fp32": kernel}[dtype]
    traffic = profile_traffic(f"tc_gemm_{tag}_{m}") if kernel != "simt" else profile_traffic(f"simt_{m}")
    if w.get("no_profile"):
        traffic = None        # no ncu capture of this configuration in profiles/
    if traffic:
        line["roofline"]["traffic"] = traffic
        line["roofline"]["traffic_vs_algorithmic"] = round(traffic / alg_bytes(w), 3)
    if err is not None:
        line["accuracy_vs_fp64"] = err
    if e2e is not None:
        line["e2e"] = e2e
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(w, A, B, dtype, target_s=args.cpu_seconds, C=C)
    h.close()
    return line


def nominal_fp32_tflops():
    import torch
    prop = torch.cuda.get_device_properties(torch.cuda.current_device())
    max_mhz = 2070.0
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            max_mhz = float(json.load(f).get("sm_max_mhz", max_mhz))
    except Exception:
        pass
    return prop.multi_processor_count * 128 * 2 * max_mhz * 1e6 / 1e12


def alg_bytes(w):
    es = {"fp32": 4, "bf16": 2, "fp16": 2, "fp8": 1}[w["dtype"]]
    od = {"fp32": 4, "bf16": 2, "fp16": 2, "fp8": 2}[w["dtype"]]
    m, n, k = w["m"], w["n"], w["k"]
    return m * k * es + k * n * es + m * n * od + (m * n * od if w["beta"] != 0 else 0)


def describe(w, name):
    return (f"{name}: {w['dtype']} GEMM M={w['m']} N={w['n']} K={w['k']} {w['lay']} column-major, "
            f"alpha={w['alpha']} beta={w['beta']}, fp32 accumulate")


def fp64_error(h, w, A, B, C, d, out_dt, scale_a, scale_b, base):
    """max|d - r| / max|r| with r the FP64 product of the exact operand values the GPU used (torch
    float64 on the device, outside the timed region), reduced on the device by tl_error_norms."""
    import torch
    import tensilelite_gb300 as tl
    m, n, k = w["m"], w["n"], w["k"]
    ta, tb = w["lay"][0] == "T", w["lay"][1] == "T"
    if w["dtype"] == "fp8":
        Av = base[0].view(torch.float8_e4m3fn).double() * scale_a
        Bv = base[1].view(torch.float8_e4m3fn).double() * scale_b
    else:
        Av, Bv = base[0].double(), base[1].double()
    # row-major views of the column-major buffers: X stored R x C (ld R) is the (C, R) tensor X^T
    opA = Av.view(m, k) if ta else Av.view(k, m).T
    opB = Bv.view(k, n) if tb else Bv.view(n, k).T
    R = w["alpha"] * (opA @ opB)
    del Av, Bv, opA, opB
    if C is not None:
        Cv = torch.from_numpy(C).to({"bf16": torch.bfloat16, "fp16": torch.float16, "fp32": torch.float32}[out_dt])
        R += w["beta"] * Cv.cuda().double().view(n, m).T
    Rc = R.T.contiguous()                                             # column-major m x n
    del R
    out = h.error_norms({"fp32": tl.FP32, "bf16": tl.BF16, "fp16": tl.FP16}[out_dt], d, m, Rc, m, m, n)
    return {"normwise": out[0] / out[1] if out[1] else out[0], "max_abs": out[0], "max_ref": out[1],
            "reduction": "on-device FP64 (tl_error_norms); reference = float64 product of the exact operands"}


def run_e2e(h, p, sol, base, dC, m, n, tdt, stream, steps):
    """The GEMM through the public API with host buffers, pipelined over three streams: step i's
    operands go host->device (tl_memcpy_h2d) while step i-1 computes (tl_gemm) and step i-2's result
    goes device->host (tl_memcpy_d2h); device buffers are double-buffered and every hand-over is an
    event, so each step still moves all of its inputs in and its whole result out."""
    import torch
    import tensilelite_gb300 as tl
    hA = torch.empty_like(base[0], device="cpu").pin_memory()
    hB = torch.empty_like(base[1], device="cpu").pin_memory()
    hA.copy_(base[0].cpu())
    hB.copy_(base[1].cpu())
    hC = dC.cpu().pin_memory() if dC is not None else None
    hD = [torch.empty(m * n, dtype=tdt).pin_memory() for _ in range(2)]
    dA = [torch.empty_like(base[0]) for _ in range(2)]
    dB = [torch.empty_like(base[1]) for _ in range(2)]
    dC2 = [torch.empty_like(dC) for _ in range(2)] if dC is not None else [None, None]
    dD = [torch.empty(m * n, dtype=tdt, device="cuda") for _ in range(2)]
    L = tl.lib()
    s_in, s_out = torch.cuda.Stream(), torch.cuda.Stream()
    s_cmp = stream
    ev_in = [torch.cuda.Event() for _ in range(2)]
    ev_cmp = [torch.cuda.Event() for _ in range(2)]
    ev_out = [torch.cuda.Event() for _ in range(2)]
    bi = hA.numel() * hA.element_size() + hB.numel() * hB.element_size() + (hC.numel() * hC.element_size() if hC is not None else 0)
    bo = hD[0].numel() * hD[0].element_size()
    used = [False, False]

    def step(i):
        b = i % 2
        if used[b]:
            s_in.wait_event(ev_cmp[b])        # the GEMM that read this input slot is done
        tl.check(L.tl_memcpy_h2d(dA[b].data_ptr(), hA.data_ptr(), hA.numel() * hA.element_size(), s_in.cuda_stream))
        tl.check(L.tl_memcpy_h2d(dB[b].data_ptr(), hB.data_ptr(), hB.numel() * hB.element_size(), s_in.cuda_stream))
        if hC is not None:
            tl.check(L.tl_memcpy_h2d(dC2[b].data_ptr(), hC.data_ptr(), hC.numel() * hC.element_size(), s_in.cuda_stream))
        ev_in[b].record(s_in)
        s_cmp.wait_event(ev_in[b])
        if used[b]:
            s_cmp.wait_event(ev_out[b])       # the result slot was read back
        h.gemm(p, dD[b], dC2[b], dA[b], dB[b], solution=sol, stream=s_cmp)
        ev_cmp[b].record(s_cmp)
        s_out.wait_event(ev_cmp[b])
        tl.check(L.tl_memcpy_d2h(hD[b].data_ptr(), dD[b].data_ptr(), bo, s_out.cuda_stream))
        ev_out[b].record(s_out)
        used[b] = True

    for i in range(4):
        step(i)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(s_in)
    for i in range(steps):
        step(i)
    s_in.wait_stream(s_out)
    ev1.record(s_in)
    ev1.synchronize()
    ms = ev0.elapsed_time(ev1)
    flops = p.flops() * steps
    bound = copy_bound(hA, dA[0], hD[0], dD[0], s_in, s_out, bi, bo, p.flops())
    return {"value": round(flops / (ms / 1e3) / 1e12, 3), "unit": "TFLOP/s", "h2d_bytes_per_step": int(bi),
            "d2h_bytes_per_step": int(bo), "steps": steps, "ms_per_step": round(ms / steps, 4),
            "path": "pinned host -> tl_memcpy_h2d -> tl_gemm -> tl_memcpy_d2h, three streams pipelined "
                    "(copies of step i+1 and i-1 overlap the GEMM of step i), double-buffered device operands",
            "copy_bound": bound}


def copy_bound(h_in, d_in, h_out, d_out, s_in, s_out, bi, bo, flops_per_step, reps=20):
    """The host link's own pinned bandwidth, one tl_memcpy (cudaMemcpyAsync) per copy as the e2e path
    makes them: host->device alone, device->host alone, and both directions at once (the pipelined e2e
    overlaps them).  An e2e step cannot beat the time its bytes take at these rates."""
    import torch
    import tensilelite_gb300 as tl
    L = tl.lib()
    nb_in = h_in.numel() * h_in.element_size()
    nb_out = h_out.numel() * h_out.element_size()

    def timed(fn, stream):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    h2d = lambda: tl.check(L.tl_memcpy_h2d(d_in.data_ptr(), h_in.data_ptr(), nb_in, s_in.cuda_stream))
    d2h = lambda: tl.check(L.tl_memcpy_d2h(h_out.data_ptr(), d_out.data_ptr(), nb_out, s_out.cuda_stream))
    ms_in = timed(h2d, s_in)
    ms_out = timed(d2h, s_out)
    # both directions at once: the two streams side by side, timed on s_in after joining s_out
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s_in)
    s_out.wait_event(e0)
    for _ in range(reps):
        h2d()
        d2h()
    s_in.wait_stream(s_out)
    e1.record(s_in)
    e1.synchronize()
    ms_both = e0.elapsed_time(e1) / reps
    gbs_in, gbs_out = nb_in / ms_in / 1e6, nb_out / ms_out / 1e6
    # per step: each direction at its own rate, and both together at the rate they reach side by side
    alone_ms = max(bi / (gbs_in * 1e6), bo / (gbs_out * 1e6))
    duplex_ms = (bi + bo) * ms_both / (nb_in + nb_out)
    step_ms = max(alone_ms, duplex_ms)
    return {"h2d_gbs": round(gbs_in, 1), "d2h_gbs": round(gbs_out, 1),
            "both_directions_gbs": round((nb_in + nb_out) / ms_both / 1e6, 1),
            "step_ms_at_link_rate": round(step_ms, 4),
            "tflops_at_link_rate": round(flops_per_step / (step_ms / 1e3) / 1e12, 2),
            "measured": f"{reps} copies of {nb_in >> 20} MiB host->device and {nb_out >> 20} MiB device->host from "
                        f"pinned memory, one cudaMemcpyAsync each; alone and both directions together"}


def grouped_sizes(seed, count):
    """M = 16*U{4..128} for all problems, then N likewise, then K = 64*U{1..64} (numpy PCG64)."""
    g = np.random.default_rng(seed)
    M = 16 * g.integers(4, 129, count)
    N = 16 * g.integers(4, 129, count)
    K = 64 * g.integers(1, 65, count)
    return [(int(m), int(n), int(k)) for m, n, k in zip(M, N, K)]


def run_grouped(args, w, name):
    """256 independent bf16 GEMMs in one persistent launch (tile picked by tl_tune_grouped), replayed from a
    CUDA graph; one step = one replay.  Entries N(0,1) from torch's generator seeded 3 on the device."""
    import torch
    import tensilelite_gb300 as tl
    torch.cuda.set_device(0)
    h = tl.Handle()
    sizes = grouped_sizes(w["seed"], w["count"])
    gen = torch.Generator(device="cuda").manual_seed(w["seed"])
    probs, A, B, D = [], [], [], []
    for (m, n, k) in sizes:
        A.append(torch.randn(m * k, device="cuda", generator=gen).to(torch.bfloat16))
        B.append(torch.randn(k * n, device="cuda", generator=gen).to(torch.bfloat16))
        D.append(torch.empty(m * n, device="cuda", dtype=torch.bfloat16))
        probs.append(tl.Problem.make(m, n, k, dtype="bf16", alpha=w["alpha"], beta=w["beta"], kernel="tcgen05"))
    flops = sum(2.0 * m * n * k for m, n, k in sizes)
    if args.no_tune_grouped:
        sol, tuned_ms = None, 0.0            # the plan's heuristic tile (profiling runs)
    else:
        sol, tuned_ms = h.tune_grouped(probs, D, None, A, B, reps=3)
    plan = h.grouped_plan(probs, D, None, A, B, solution=sol)
    stream = torch.cuda.Stream()
    graph = plan.capture(stream)
    clocks = ClockSampler(smi_index())
    clocks.start()
    for _ in range(args.warmup):
        graph.launch(stream)
    stream.synchronize()
    h.device_status(stream)
    mark0 = clocks.mark()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = h.launch_count()
    ev0.record(stream)
    for _ in range(args.steps):
        graph.launch(stream)
    ev1.record(stream)
    ev1.synchronize()
    mark1 = clocks.mark()
    h.device_status(stream)
    ms = ev0.elapsed_time(ev1)
    value = flops * args.steps / (ms / 1e3) / 1e12
    # e2e: host operands in, results out, through the public API (plan launch), every step
    e2e = None
    if args.e2e_steps > 0:
        hA = [a.cpu().pin_memory() for a in A]
        hB = [b.cpu().pin_memory() for b in B]
        hD = [torch.empty(d.numel(), dtype=torch.bfloat16).pin_memory() for d in D]
        L = tl.lib()
        sp = stream.cuda_stream
        bi = sum(x.numel() * 2 for x in hA + hB)
        bo = sum(x.numel() * 2 for x in hD)

        def step():
            for ha, da in zip(hA, A):
                tl.check(L.tl_memcpy_h2d(da.data_ptr(), ha.data_ptr(), ha.numel() * 2, sp))
            for hb, db in zip(hB, B):
                tl.check(L.tl_memcpy_h2d(db.data_ptr(), hb.data_ptr(), hb.numel() * 2, sp))
            plan.launch(stream)
            for hd, dd in zip(hD, D):
                tl.check(L.tl_memcpy_d2h(hd.data_ptr(), dd.data_ptr(), hd.numel() * 2, sp))
        step()
        stream.synchronize()
        # every step moves ~2 GB over the host link: a few steps are enough
        esteps = max(1, min(args.e2e_steps, 10))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(esteps):
            step()
        e1.record(stream)
        e1.synchronize()
        ems = e0.elapsed_time(e1)
        e2e = {"value": round(flops * esteps / (ems / 1e3) / 1e12, 3),
               "unit": "TFLOP/s", "h2d_bytes_per_step": int(bi), "d2h_bytes_per_step": int(bo),
               "steps": esteps, "path": "pinned host -> tl_memcpy_h2d x512 -> tl_grouped_plan_launch -> "
                                                 "tl_memcpy_d2h x256, one stream"}
    clocks.stop()
    peaks = load_peaks()
    fl, tiles, psol = plan.info()
    kernel_ms = ms / args.steps
    line = {"metric": METRIC, "value": round(value, 3), "unit": "TFLOP/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(kernel_ms, 6), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16",
            "data": f"synthetic: sizes numpy PCG64 seed {w['seed']}; entries N(0,1) torch CUDA generator seed {w['seed']}",
            "config": {"workload": f"{name}: {w['count']} bf16 NN GEMMs, M,N in 16*[4,128], K in 64*[1,64], "
                                   f"one persistent launch replayed from a CUDA graph",
                       "problems": w["count"], "total_flop": flops, "tiles": tiles, "solution": psol.as_dict(),
                       "tuned_ms": round(tuned_ms, 4), "l2": f"operands {sum(a.numel() + b.numel() for a, b in zip(A, B)) * 2 / 2**30:.1f} GiB > L2",
                       "parallelism": "1 GPU"},
            "roofline": {"bound": "tensor", "achieved": round(value, 2), "peak": peaks["bf16_tflops"],
                         "unit": "TFLOP/s", "frac": round(value / peaks["bf16_tflops"], 4),
                         "traffic": None, "peak_source": peaks["source"] + " bf16 burst", "kernel_ms": round(kernel_ms, 6)},
            "clocks": clocks.summary(mark0, mark1), "gpu_launches": h.launch_count() - l0 or args.steps}
    traffic = profile_traffic(f"tc_gemm_bf16_{name}")
    if traffic:
        alg = sum((m * k + k * n + m * n) * 2 for m, n, k in sizes)     # bf16 A, B and D (beta 0)
        line["roofline"]["traffic"] = traffic
        line["roofline"]["traffic_vs_algorithmic"] = round(traffic / alg, 3)
    if e2e:
        line["e2e"] = e2e
    if not args.no_cpu:
        m, n, k = sizes[0]
        wl = dict(dtype="bf16", m=m, n=n, k=k, lay="NN", alpha=1.0, beta=0.0, seed=w["seed"], dist="normal")
        Ah = A[0].float().cpu().numpy()
        Bh = B[0].float().cpu().numpy()
        cb = cpu_baseline(wl, Ah, Bh, "fp32", target_s=args.cpu_seconds)
        cb["sample"] = "problem 0 of the group: " + cb["sample"]
        line["cpu_baseline"] = cb
    plan.close()
    graph.close()
    h.close()
    return line


def run_fwdbwd(args, w, name):
    """Y = X W forward and dX = dY W^T, dW = X^T dY backward through tensilelite_gb300.matmul (autograd);
    one step = forward + backward (3 GEMM launches).  value: the step captured once in a CUDA graph
    (torch.cuda.graph around the autograd calls) and replayed; eager: the same step called from Python."""
    import torch
    import tensilelite_gb300 as tl
    torch.cuda.set_device(0)
    M, K, N = w["m"], w["k"], w["n"]
    g = np.random.default_rng(w["seed"])
    Xh = (g.standard_normal(M * K) * 0.02).astype(np.float32).reshape(M, K)
    Wh = (g.standard_normal(K * N) * 0.02).astype(np.float32).reshape(K, N)
    dYh = g.standard_normal(M * N).astype(np.float32).reshape(M, N)
    X = torch.from_numpy(Xh).cuda().to(torch.bfloat16).requires_grad_()
    W = torch.from_numpy(Wh).cuda().to(torch.bfloat16).requires_grad_()
    dY = torch.from_numpy(dYh).cuda().to(torch.bfloat16)
    h = tl.default_handle()
    flops = 3 * 2.0 * M * N * K

    def step():
        X.grad = None
        W.grad = None
        Y = tl.matmul(X, W)
        Y.backward(dY)
        return Y

    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(args.warmup):
            step()
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    h.device_status()

    # eager: Python + autograd per step; kernel time from an event pair around each GEMM launch
    eager_steps = min(args.steps, 2000)
    h.set_kernel_timing(True)
    h.kernel_timing(reset=True)
    l0 = h.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(eager_steps):
        step()
    ev1.record()
    ev1.synchronize()
    eager_ms = ev0.elapsed_time(ev1) / eager_steps
    eager_launches = (h.launch_count() - l0) / eager_steps
    kms, kn = h.kernel_timing(reset=True)
    h.set_kernel_timing(False)
    kernel_ms_per_step = kms / max(1, kn) * eager_launches

    # graph: the step captured once per copy of the operands; the copies (X, W, dY and the three
    # results each) together exceed twice the L2, so a replayed step reads none of its operands
    # from the previous steps' L2 lines
    set_bytes = 2 * (2 * M * K + 2 * K * N + 2 * M * N)
    nsets = max(1, int(np.ceil(2 * L2_BYTES / set_bytes)))
    Xs = [X] + [X.detach().clone().requires_grad_() for _ in range(nsets - 1)]
    Ws = [W] + [W.detach().clone().requires_grad_() for _ in range(nsets - 1)]
    dYs = [dY] + [dY.clone() for _ in range(nsets - 1)]

    def capture(count):
        gr = torch.cuda.CUDAGraph()
        outs = []
        with torch.cuda.graph(gr):
            for i in range(count):
                Xs[i].grad = None
                Ws[i].grad = None
                Yi = tl.matmul(Xs[i], Ws[i])
                Yi.backward(dYs[i])
                outs.append(Yi)
        return gr, outs
    graph, youts = capture(nsets)
    Yg = youts[0]
    rest_n = args.steps % nsets
    rest = capture(rest_n)[0] if rest_n else None
    graph.replay()
    torch.cuda.synchronize()
    h.device_status()
    clocks = ClockSampler(smi_index())
    clocks.start()
    for _ in range(max(1, args.warmup // nsets)):
        graph.replay()
    torch.cuda.synchronize()
    mark0 = clocks.mark()
    ev0.record()
    for _ in range(args.steps // nsets):
        graph.replay()
    if rest is not None:
        rest.replay()
    ev1.record()
    ev1.synchronize()
    mark1 = clocks.mark()
    h.device_status()
    ms = ev0.elapsed_time(ev1)
    value = flops * args.steps / (ms / 1e3) / 1e12
    # FP64 reference gradients at full size
    Xd, Wd, dYd = X.detach().double(), W.detach().double(), dY.double()
    err = {}
    for nm, got, ref in (("Y", Yg, Xd @ Wd), ("dX", X.grad, dYd @ Wd.T), ("dW", W.grad, Xd.T @ dYd)):
        err[nm] = float((got.detach().double() - ref).abs().max() / ref.abs().max())
    e2e = None
    if args.e2e_steps > 0:
        hX = torch.from_numpy(Xh).to(torch.bfloat16).pin_memory()
        hW = torch.from_numpy(Wh).to(torch.bfloat16).pin_memory()
        hdY = torch.from_numpy(dYh).to(torch.bfloat16).pin_memory()
        hdX = torch.empty(M, K, dtype=torch.bfloat16).pin_memory()
        hdW = torch.empty(K, N, dtype=torch.bfloat16).pin_memory()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.e2e_steps):
            with torch.no_grad():
                X.copy_(hX, non_blocking=True)
                W.copy_(hW, non_blocking=True)
                dY.copy_(hdY, non_blocking=True)
            step()
            hdX.copy_(X.grad, non_blocking=True)
            hdW.copy_(W.grad, non_blocking=True)
        e1.record()
        e1.synchronize()
        ems = e0.elapsed_time(e1)
        e2e = {"value": round(flops * args.e2e_steps / (ems / 1e3) / 1e12, 3),
               "unit": "TFLOP/s", "h2d_bytes_per_step": 2 * (M * K + K * N + M * N),
               "d2h_bytes_per_step": 2 * (M * K + K * N), "steps": args.e2e_steps,
               "path": "pinned host -> copy -> tensilelite_gb300.matmul fwd+bwd (eager) -> grads to pinned host"}
    clocks.stop()
    peaks = load_peaks()
    # the replayed graph is the three GEMM kernels back to back: its time is their summed duration
    achieved = value
    line = {"metric": METRIC, "value": round(value, 3), "unit": "TFLOP/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 6), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16",
            "data": f"synthetic: numpy PCG64 seed {w['seed']}: X, W ~ N(0,1)*0.02, dY ~ N(0,1)",
            "config": {"workload": f"{name}: Y = X W, X {M}x{K}, W {K}x{N}, forward NN + backward TN (dX) and NT (dW)",
                       "step": f"CUDA graph replay of the captured forward+backward (3 GEMM launches), {nsets} steps "
                               "per graph, one per operand copy",
                       "eager": {"value": round(flops / (eager_ms / 1e3) / 1e12, 3), "ms_per_step": round(eager_ms, 6),
                                 "steps": eager_steps},
                       "l2": f"rotating {nsets} copies of the operands and results, {set_bytes / 2**20:.0f} MiB each "
                             "(> L2 together)",
                       "parallelism": "1 GPU"},
            "roofline": {"bound": "tensor", "achieved": round(achieved, 2), "peak": peaks["bf16_tflops"],
                         "unit": "TFLOP/s", "frac": round(achieved / peaks["bf16_tflops"], 4),
                         "traffic": None, "peak_source": peaks["source"] + " bf16 burst",
                         "kernel_ms": round(ms / args.steps, 6),
                         "eager_kernel_ms_per_step": round(kernel_ms_per_step, 6),
                         "note": "achieved over the graph replay (the three GEMM kernels back to back); the eager "
                                 "per-launch event pairs also time the host's launch gaps"},
            "accuracy_vs_fp64": err, "clocks": clocks.summary(mark0, mark1),
            "gpu_launches": int(round(eager_launches * args.steps))}
    if e2e:
        line["e2e"] = e2e
    if not args.no_cpu:
        wl = dict(dtype="bf16", m=N, n=M, k=K, lay="NN", alpha=1.0, beta=0.0, seed=w["seed"], dist="normal")
        # Y^T = W^T X^T column-major: A = W's storage (N x K), B = X's storage (K x M)
        line["cpu_baseline"] = cpu_baseline(wl, W.detach().float().cpu().numpy().reshape(-1),
                                            X.detach().float().cpu().numpy().reshape(-1), "fp32",
                                            target_s=args.cpu_seconds)
    return line


# ----------------------------------------------------------------------------------------------
# reference arm: the reference's CPU GEMM loop (oracle port), all host threads
# ----------------------------------------------------------------------------------------------
def run_reference(args, w, name):
    world, _ = launch_env()
    from oracle import oracle as orc
    orc.lib()
    threads = os.cpu_count() or 1
    A, B, C, lda, ldb = host_inputs(w)
    dtype = w["dtype"]
    if dtype == "fp8":
        dtype = "fp32"
    Ap, Bp, Cw = cpu_sample_setup(w, A, B, dtype, C)
    m, n, k = w["m"], w["n"], w["k"]
    alpha, beta = w.get("alpha", 1.0), w.get("beta", 0.0)
    per_col = 2.0 * m * k
    c0 = min(n, threads)
    t = cpu_run_columns(Ap, Bp, m, n, k, c0, threads, alpha=alpha, beta=beta, C=Cw)
    rate = c0 / max(t, 1e-6)
    budget = min(2.0, 150.0 / max(1, args.steps + args.warmup))      # seconds per step
    cols = int(min(n, max(1, rate * budget)))
    for i in range(args.warmup):
        cpu_run_columns(Ap, Bp, m, n, k, cols, threads, col0=(i * cols) % max(1, n - cols + 1), alpha=alpha,
                        beta=beta, C=Cw)
    times = []
    for i in range(args.steps):
        times.append(cpu_run_columns(Ap, Bp, m, n, k, cols, threads, col0=(i * cols) % max(1, n - cols + 1),
                                     alpha=alpha, beta=beta, C=Cw))
    tot = sum(times)
    value = per_col * cols * args.steps / tot / 1e12
    model = cpu_model()
    sample = (f"reference CPU loop (src/gemmMfma.cpp:313-346 restated in oracle/tl_oracle.c: alpha*sum + beta*c) "
              f"over {cols} of {n} output columns per step of the {m}x{n}x{k} problem, {threads} threads ({model}); "
              f"every column costs the same, so the sample's throughput stands for the whole problem")
    return {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tot / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": w["dtype"], "data": "synthetic (same seeds as the GPU arm)",
            "config": {"workload": describe(w, name), "m": m, "n": n, "k": k, "layout": w["lay"], "alpha": alpha,
                       "beta": beta},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": threads, "kind": "port", "sample": sample,
                             "cpu_model": model},
            "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# The other benchmark configurations, measured after the headline in the same run and reported in
# its line under "suite" (device throughput, roofline fraction, FP64 error; no e2e or CPU legs):
# (workload, timed steps, warm-up steps)
SUITE = [
    ("fp16_4096_nn", 100, 10), ("bf16_4096_nn_b0", 100, 10), ("bf16_4096_tn", 100, 10), ("bf16_4096_nt", 100, 10),
    ("bf16_480x1024x4096", 2000, 20), ("fp8_8192", 50, 5), ("grouped256", 100, 5), ("fwdbwd", 200, 10),
    ("bf16x3_8192", 20, 3), ("bf16x6_8192", 20, 3), ("simt_fp32_8192", 4, 3), ("simt_fp32_480x512x512", 2000, 20),
]


def compact(line):
    """The fields of a workload's line the suite keeps."""
    keep = {k: line.get(k) for k in ("value", "unit", "ms_per_step", "steps", "dtype", "gpu_launches")}
    keep["workload"] = line["config"].get("workload")
    rf = line.get("roofline", {})
    keep["roofline"] = {k: rf.get(k) for k in ("bound", "achieved", "peak", "frac", "peak_source", "kernel_ms",
                                               "traffic_vs_algorithmic", "note") if k in rf}
    if "solution" in line["config"]:
        keep["solution"] = line["config"]["solution"]
    acc = line.get("accuracy_vs_fp64")
    if isinstance(acc, dict) and "normwise" in acc:
        keep["accuracy_vs_fp64"] = acc["normwise"]
    elif acc is not None:
        keep["accuracy_vs_fp64"] = acc
    clk = line.get("clocks", {})
    keep["clocks"] = {k: clk.get(k) for k in ("sm_mhz", "reasons")}
    return keep


def run_suite(args):
    import torch
    out = {}
    for name, steps, warmup in SUITE:
        sub = argparse.Namespace(**vars(args))
        sub.steps, sub.warmup, sub.e2e_steps, sub.no_cpu, sub.tune = steps, warmup, 0, True, 0
        sub.no_tune_grouped = False
        w = WORKLOADS[name]
        kind = w.get("kind", "gemm")
        try:
            line = (run_grouped if kind == "grouped" else run_fwdbwd if kind == "fwdbwd" else run_gpu)(sub, w, name)
            out[name] = compact(line)
        except Exception as e:                # one failing configuration does not drop the others
            out[name] = {"error": f"{type(e).__name__}: {str(e)[:300]}"}
        torch.cuda.empty_cache()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: about one second of GPU work for the workload)")
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="tensilelite_gb300", choices=["tensilelite_gb300", "reference"])
    ap.add_argument("--workload", default="bf16_4096_nn", choices=sorted(WORKLOADS))
    ap.add_argument("--tune", type=int, default=0, help="autotune over this many candidates first")
    ap.add_argument("--e2e-steps", type=int, default=200)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-check", dest="check", action="store_false")
    ap.add_argument("--no-tune-grouped", action="store_true",
                    help="grouped256: use the plan's heuristic tile instead of tl_tune_grouped")
    ap.add_argument("--suite", dest="suite", action="store_true", default=None,
                    help="also measure the other configurations (default: on for the default workload)")
    ap.add_argument("--no-suite", dest="suite", action="store_false")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    w = WORKLOADS[args.workload]
    if args.steps is None:
        args.steps = w.get("steps", 10000)
    kind = w.get("kind", "gemm")
    world, rank = launch_env()
    if world > 1:
        # the GPU arm is a one-GPU deliverable; the reference arm uses host cores on rank 0 only
        if rank != 0:
            return
        if args.impl != "reference":
            print(json.dumps(refusal_line(world, args.impl)), flush=True)
            return
    if args.impl == "reference":
        if kind == "grouped":
            m, n, k = grouped_sizes(w["seed"], w["count"])[0]
            w = dict(dtype="bf16", m=m, n=n, k=k, lay="NN", alpha=1.0, beta=0.0, seed=w["seed"], dist="normal")
        elif kind == "fwdbwd":
            w = dict(dtype="bf16", m=w["n"], n=w["m"], k=w["k"], lay="NN", alpha=1.0, beta=0.0, seed=w["seed"],
                     dist="normal")
        line = run_reference(args, w, args.workload)
    elif kind == "grouped":
        line = run_grouped(args, w, args.workload)
    elif kind == "fwdbwd":
        line = run_fwdbwd(args, w, args.workload)
    else:
        line = run_gpu(args, w, args.workload)
    if line is not None and args.impl != "reference" and (args.suite or (args.suite is None and
                                                                         args.workload == "bf16_4096_nn")):
        line["suite"] = run_suite(args)
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
