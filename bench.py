"""bench.py -- GEMM throughput on GB300 through the library's C ABI.

Default workload (the configuration the headline metric is quoted on): bf16 GEMM, M = N = K = 4096,
NN column-major, alpha = 1, beta = 0.5, A, B, C ~ N(0,1) from numpy PCG64 seed 1 (drawn A, B, C),
cast to bf16 (RNE), fp32 accumulation, bf16 output.  One step = one GEMM launch.

  value      device throughput (TFLOP/s, 2*M*N*K per step) with inputs resident in HBM; K steps
             timed back to back with CUDA events on the launching stream, rotating over 4 copies
             of the inputs (4 x 128 MiB > the 129 MB L2) so no step reads the previous one's tiles
             from L2.
  e2e        the same GEMM through the public API with host buffers: per step the pinned-host A,
             B, C are copied in (tl_memcpy_h2d), the GEMM runs, D is copied out (tl_memcpy_d2h).
  roofline   the tcgen05 kernel against the measured dense bf16 peak (MEASURED_PEAKS.json).
  cpu_baseline  the reference's CPU GEMM loop (src/gemmMfma.cpp:313-346, restated in oracle/) on
             a bounded sample of output columns of the same problem, all host threads.

Other workloads (--workload): fp16_4096_nn|nt|tn, bf16_4096_nt|tn, bf16_480x1024x4096, bf16x3_8192,
simt_fp32_8192, fp8_8192, grouped256, fwdbwd.  `--impl reference` times the reference's CPU loop
(the oracle port) on the same workload instead.  Multi-GPU (torchrun): every rank runs its own
replica of the workload; value sums the ranks' FLOPs over the slowest rank's time.
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


# ----------------------------------------------------------------------------------------------
# workloads
# ----------------------------------------------------------------------------------------------
WORKLOADS = {
    "bf16_4096_nn": dict(dtype="bf16", m=4096, n=4096, k=4096, lay="NN", alpha=1.0, beta=0.5, seed=1, dist="normal"),
    "bf16_4096_nt": dict(dtype="bf16", m=4096, n=4096, k=4096, lay="NT", alpha=1.0, beta=0.5, seed=1, dist="normal"),
    "bf16_4096_tn": dict(dtype="bf16", m=4096, n=4096, k=4096, lay="TN", alpha=1.0, beta=0.5, seed=1, dist="normal"),
    "fp16_4096_nn": dict(dtype="fp16", m=4096, n=4096, k=4096, lay="NN", alpha=1.0, beta=0.5, seed=1, dist="normal"),
    "fp16_4096_nt": dict(dtype="fp16", m=4096, n=4096, k=4096, lay="NT", alpha=1.0, beta=0.5, seed=1, dist="normal"),
    "fp16_4096_tn": dict(dtype="fp16", m=4096, n=4096, k=4096, lay="TN", alpha=1.0, beta=0.5, seed=1, dist="normal"),
    "bf16_480x1024x4096": dict(dtype="bf16", m=480, n=1024, k=4096, lay="NN", alpha=1.0, beta=0.5, seed=1,
                               dist="normal"),
    "bf16x3_8192": dict(dtype="fp32", m=8192, n=8192, k=8192, lay="NN", alpha=1.0, beta=0.0, seed=2,
                        dist="uniform", kernel="bf16x3"),
    "simt_fp32_8192": dict(dtype="fp32", m=8192, n=8192, k=8192, lay="NN", alpha=1.0, beta=0.0, seed=2,
                           dist="uniform", kernel="simt"),
    "fp8_8192": dict(dtype="fp8", m=8192, n=8192, k=8192, lay="TN", alpha=1.0, beta=0.0, seed=2, dist="normal"),
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
def cpu_sample_setup(w, A, B, dtype):
    """Packed TN storage (Ap[m][k], Bp[n][k]) of the values the GPU multiplies (fp32 widened)."""
    import torch
    m, n, k = w["m"], w["n"], w["k"]
    ta, tb = w["lay"][0] == "T", w["lay"][1] == "T"

    def widen(x):
        if dtype in ("bf16", "fp16"):
            tt = torch.bfloat16 if dtype == "bf16" else torch.float16
            return torch.from_numpy(x).to(tt).float().numpy()
        return x
    Aw, Bw = widen(A), widen(B)
    Ap = np.ascontiguousarray(Aw.reshape(m, k) if ta else Aw.reshape(k, m).T)          # m x k
    Bp = np.ascontiguousarray(Bw.reshape(k, n).T if tb else Bw.reshape(n, k))          # n x k
    return Ap.astype(np.float32), Bp.astype(np.float32)


def cpu_run_columns(Ap, Bp, m, n, k, cols, threads, col0=0):
    import ctypes
    from oracle import oracle as orc
    L = orc.lib()
    D = np.zeros((cols, m), np.float32)
    f32p = ctypes.POINTER(ctypes.c_float)
    Bsub = np.ascontiguousarray(Bp[col0:col0 + cols])
    t0 = time.perf_counter()
    L.orc_gemm_ref_f32_packed(m, cols, k, ctypes.c_float(1.0), Ap.ctypes.data_as(f32p), Bsub.ctypes.data_as(f32p),
                              D.ctypes.data_as(f32p), m, 0, cols, threads)
    return time.perf_counter() - t0


def cpu_baseline(w, A, B, dtype, target_s=10.0, threads=None):
    from oracle import oracle as orc
    orc.lib()
    threads = threads or os.cpu_count() or 1
    m, n, k = w["m"], w["n"], w["k"]
    Ap, Bp = cpu_sample_setup(w, A, B, dtype)
    per_col = 2.0 * m * k
    # calibrate on a few columns, then size the sample to ~target_s
    c0 = min(n, max(threads, 1))
    t = cpu_run_columns(Ap, Bp, m, n, k, c0, threads)
    rate = c0 / max(t, 1e-6)
    cols = int(min(n, max(c0, rate * target_s)))
    t = cpu_run_columns(Ap, Bp, m, n, k, cols, threads)
    tflops = per_col * cols / t / 1e12
    return {"value": tflops, "unit": "TFLOP/s", "cores": threads, "kind": "port",
            "sample": f"reference CPU loop (src/gemmMfma.cpp:313-346 restated, -O2 -ffp-contract=off) over {cols} of "
                      f"{n} output columns of the {m}x{n}x{k} problem, {t:.1f} s, {threads} threads",
            "seconds": t}


# ----------------------------------------------------------------------------------------------
# GPU arm
# ----------------------------------------------------------------------------------------------
def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def run_gpu(args, w, name):
    import torch
    import tensilelite_gb300 as tl

    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
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
    # rotating copies so the working set of consecutive steps exceeds L2
    bytes_per_set = sum(x.numel() * x.element_size() for x in base) + (dC.numel() * dC.element_size() if dC is not None
                                                                         else 0) + m * n * tdt.itemsize
    nsets = max(1, min(4, int(np.ceil(2 * 129e6 / bytes_per_set)) if bytes_per_set < 2 * 129e6 else 1))
    if bytes_per_set * nsets < 129e6:
        nsets = 4
    sets = []
    for i in range(nsets):
        a = base[0] if i == 0 else base[0].clone()
        b = base[1] if i == 0 else base[1].clone()
        c = dC if (i == 0 or dC is None) else dC.clone()
        d = torch.empty(m * n, dtype=tdt, device="cuda")
        sets.append((a, b, c, d))
    torch.cuda.synchronize()

    flops = 2.0 * m * n * k
    clocks = ClockSampler(local)
    clocks.start()
    with torch.cuda.stream(stream):
        for i in range(args.warmup):
            a, b, c, d = sets[i % nsets]
            h.gemm(p, d, c, a, b, solution=sol, stream=stream)
    stream.synchronize()
    h.device_status(stream)
    time.sleep(0.2)
    barrier(world)
    torch.cuda.synchronize()
    mark0 = clocks.mark()
    launches0 = h.launch_count()
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
    barrier(world)
    h.device_status(stream)
    ms_total = ev0.elapsed_time(ev1)
    ms_max = max_over_ranks(ms_total, world)
    total_flops = sum_over_ranks(flops * args.steps, world)
    value = total_flops / (ms_max / 1e3) / 1e12
    ms_per_step = ms_max / args.steps
    kernel_ms = ms_total / args.steps / max(1, launches // max(1, args.steps))

    # accuracy of the benchmarked result against an FP64 host oracle (numpy float64 matmul)
    err = None
    if args.check and m * n * k <= 8192 ** 3 and rank == 0:
        a, b, c, d = sets[(args.steps - 1) % nsets]
        try:
            err = fp64_error(h, w, A, B, C, d, out_dt, scale_a, scale_b, base)
        except Exception as e:  # keep the bench line even if the host is short of memory
            err = {"error": str(e)[:200]}

    # e2e through the public API: pinned host buffers in, result out, every step
    e2e = None
    if args.e2e_steps > 0:
        e2e = run_e2e(h, p, sol, base, dC, m, n, tdt, stream, args.e2e_steps, world)
    clocks.stop()
    clk = clocks.summary(mark0, mark1)
    peaks = load_peaks()
    achieved = flops / (kernel_ms / 1e3) / 1e12
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 6), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": dtype,
        "data": f"synthetic: numpy PCG64 seed {w['seed']}, {'N(0,1)' if w['dist'] == 'normal' else 'uniform[-1,1)'}",
        "config": {"workload": describe(w, name), "m": m, "n": n, "k": k, "layout": w["lay"], "alpha": w["alpha"],
                   "beta": w["beta"], "kernel": kernel, "solution": sol.as_dict(),
                   "l2": f"rotating {nsets} input sets of {bytes_per_set / 2**20:.0f} MiB (> L2 together)"
                   if nsets > 1 else "inputs larger than L2",
                   "parallelism": "replicas" if world > 1 else "1 GPU"},
        "roofline": {"bound": "tensor" if kernel != "simt" else "fp32-pipe", "achieved": round(achieved, 2),
                     "peak": peaks["bf16_tflops"] * (2 if dtype == "fp8" else 1) if kernel != "simt" else None,
                     "unit": "TFLOP/s", "frac": None, "traffic": None,
                     "peak_source": peaks["source"] + (" bf16 burst" + (" x2 (fp8 dense = 2x bf16)" if dtype == "fp8"
                                                                         else "")),
                     "kernel_ms": round(kernel_ms, 6)},
        "clocks": clk, "gpu_launches": launches, "wall_s_timed": round(t_wall, 4),
    }
    if line["roofline"]["peak"]:
        line["roofline"]["frac"] = round(achieved / line["roofline"]["peak"], 4)
    tag = {"bf16": "bf16", "fp16": "fp16", "fp8": "fp8", "fp32": kernel}[dtype]
    traffic = profile_traffic(f"tc_gemm_{tag}_{m}") if kernel != "simt" else profile_traffic(f"simt_{m}")
    if traffic:
        line["roofline"]["traffic"] = traffic
        line["roofline"]["traffic_vs_algorithmic"] = round(traffic / alg_bytes(w), 3)
    if err is not None:
        line["accuracy_vs_fp64"] = err
    if e2e is not None:
        line["e2e"] = e2e
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(w, A, B, dtype, target_s=args.cpu_seconds)
    h.close()
    return line if rank == 0 else None


def alg_bytes(w):
    es = {"fp32": 4, "bf16": 2, "fp16": 2, "fp8": 1}[w["dtype"]]
    od = {"fp32": 4, "bf16": 2, "fp16": 2, "fp8": 2}[w["dtype"]]
    m, n, k = w["m"], w["n"], w["k"]
    return m * k * es + k * n * es + m * n * od + (m * n * od if w["beta"] != 0 else 0)


def describe(w, name):
    return (f"{name}: {w['dtype']} GEMM M={w['m']} N={w['n']} K={w['k']} {w['lay']} column-major, "
            f"alpha={w['alpha']} beta={w['beta']}, fp32 accumulate")


def fp64_error(h, w, A, B, C, d, out_dt, scale_a, scale_b, base):
    """max|d - r| / max|r| with r the FP64 product of the exact operand values the GPU used."""
    import torch
    import tensilelite_gb300 as tl
    m, n, k = w["m"], w["n"], w["k"]
    ta, tb = w["lay"][0] == "T", w["lay"][1] == "T"
    if w["dtype"] == "fp8":
        def deq(q, s):
            return q.view(torch.float8_e4m3fn).float().double().cpu().numpy() * s
        Av, Bv = deq(base[0], scale_a), deq(base[1], scale_b)
    else:
        Av = base[0].double().cpu().numpy()
        Bv = base[1].double().cpu().numpy()
    opA = Av.reshape(m, k) if ta else Av.reshape(k, m).T
    opB = Bv.reshape(k, n) if tb else Bv.reshape(n, k).T
    R = w["alpha"] * (opA @ opB)
    if C is not None:
        Cv = torch.from_numpy(C).to({"bf16": torch.bfloat16, "fp16": torch.float16, "fp32": torch.float32}[out_dt])
        R = R + w["beta"] * Cv.double().numpy().reshape(n, m).T
    Rc = torch.from_numpy(np.ascontiguousarray(R.T)).cuda()        # column-major m x n
    out = h.error_norms({"fp32": tl.FP32, "bf16": tl.BF16, "fp16": tl.FP16}[out_dt], d, m, Rc, m, m, n)
    return {"normwise": out[0] / out[1] if out[1] else out[0], "max_abs": out[0], "max_ref": out[1],
            "reduction": "on-device FP64 (tl_error_norms); reference = numpy float64 matmul of the exact operands"}


def run_e2e(h, p, sol, base, dC, m, n, tdt, stream, steps, world):
    import torch
    import tensilelite_gb300 as tl
    hA = torch.empty_like(base[0], device="cpu").pin_memory()
    hB = torch.empty_like(base[1], device="cpu").pin_memory()
    hA.copy_(base[0].cpu())
    hB.copy_(base[1].cpu())
    hC = dC.cpu().pin_memory() if dC is not None else None
    hD = torch.empty(m * n, dtype=tdt).pin_memory()
    dA, dB = torch.empty_like(base[0]), torch.empty_like(base[1])
    dC2 = torch.empty_like(dC) if dC is not None else None
    dD = torch.empty(m * n, dtype=tdt, device="cuda")
    L = tl.lib()
    sp = stream.cuda_stream
    bi = hA.numel() * hA.element_size() + hB.numel() * hB.element_size() + (hC.numel() * hC.element_size() if hC is not None else 0)
    bo = hD.numel() * hD.element_size()

    def step():
        tl.check(L.tl_memcpy_h2d(dA.data_ptr(), hA.data_ptr(), hA.numel() * hA.element_size(), sp))
        tl.check(L.tl_memcpy_h2d(dB.data_ptr(), hB.data_ptr(), hB.numel() * hB.element_size(), sp))
        if hC is not None:
            tl.check(L.tl_memcpy_h2d(dC2.data_ptr(), hC.data_ptr(), hC.numel() * hC.element_size(), sp))
        h.gemm(p, dD, dC2, dA, dB, solution=sol, stream=stream)
        tl.check(L.tl_memcpy_d2h(hD.data_ptr(), dD.data_ptr(), bo, sp))

    for _ in range(3):
        step()
    stream.synchronize()
    barrier(world)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(steps):
        step()
    ev1.record(stream)
    ev1.synchronize()
    ms = max_over_ranks(ev0.elapsed_time(ev1), world)
    flops = sum_over_ranks(p.flops() * steps, world)
    return {"value": round(flops / (ms / 1e3) / 1e12, 3), "unit": "TFLOP/s", "h2d_bytes_per_step": int(bi),
            "d2h_bytes_per_step": int(bo), "steps": steps, "ms_per_step": round(ms / steps, 4),
            "path": "pinned host -> tl_memcpy_h2d -> tl_gemm -> tl_memcpy_d2h, one stream"}


# ----------------------------------------------------------------------------------------------
# reference arm: the reference's CPU GEMM loop (oracle port), all host threads
# ----------------------------------------------------------------------------------------------
def run_reference(args, w, name):
    world, rank, _ = dist_setup(args)
    if rank != 0:
        return None
    from oracle import oracle as orc
    orc.lib()
    threads = os.cpu_count() or 1
    A, B, C, lda, ldb = host_inputs(w)
    dtype = w["dtype"]
    if dtype == "fp8":
        dtype = "fp32"
    Ap, Bp = cpu_sample_setup(w, A, B, dtype)
    m, n, k = w["m"], w["n"], w["k"]
    per_col = 2.0 * m * k
    c0 = min(n, threads)
    t = cpu_run_columns(Ap, Bp, m, n, k, c0, threads)
    rate = c0 / max(t, 1e-6)
    budget = min(2.0, 150.0 / max(1, args.steps + args.warmup))      # seconds per step
    cols = int(min(n, max(1, rate * budget)))
    for i in range(args.warmup):
        cpu_run_columns(Ap, Bp, m, n, k, cols, threads, col0=(i * cols) % max(1, n - cols + 1))
    times = []
    for i in range(args.steps):
        times.append(cpu_run_columns(Ap, Bp, m, n, k, cols, threads, col0=(i * cols) % max(1, n - cols + 1)))
    tot = sum(times)
    value = per_col * cols * args.steps / tot / 1e12
    sample = (f"reference CPU loop (src/gemmMfma.cpp:313-346 restated in oracle/tl_oracle.c) over {cols} of {n} "
              f"output columns per step of the {m}x{n}x{k} problem")
    return {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tot / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": w["dtype"], "data": "synthetic (same seeds as the GPU arm)",
            "config": {"workload": describe(w, name), "m": m, "n": n, "k": k, "layout": w["lay"]},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "TFLOP/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="tensilelite_gb300", choices=["tensilelite_gb300", "reference"])
    ap.add_argument("--workload", default="bf16_4096_nn", choices=sorted(WORKLOADS))
    ap.add_argument("--tune", type=int, default=0, help="autotune over this many candidates first")
    ap.add_argument("--e2e-steps", type=int, default=200)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-check", dest="check", action="store_false")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        line = run_reference(args, w, args.workload)
    else:
        line = run_gpu(args, w, args.workload)
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
