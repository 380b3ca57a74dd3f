"""Builds libtensilelite_gb300.so in place with nvcc for sm_103a (and the CLI binary).

Every translation unit compiles in parallel to tensilelite_gb300/_build/, then one shared library
is linked next to this file.  Only symbols marked TL_API are exported.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libtensilelite_gb300.so")
CLI = os.path.join(HERE, "tensilelite")

SOURCES = ["gemm_tc.cu", "gemm_simt.cu", "aux_kernels.cu", "tl_api.cpp", "noalloc.cu"]
# The tcgen05 kernel template is instantiated in generated units, one per operand kind (0 fp16/bf16,
# 1 fp8), cluster size and epilogue variant, so they compile in parallel.  Plain kernels write fp32,
# fp16 or bf16; the fused-epilogue kernels also fp8 (E4M3).
INSTANCES = [(k, e, cl) for k in (0, 1) for e in (False, True) for cl in (1, 2, 4)]
OUT_TYPES = ("float", "__half", "__nv_bfloat16")
EPI_OUT_TYPES = OUT_TYPES + ("__nv_fp8_e4m3",)


def _instance_sources():
    gen = os.path.join(BUILD, "gen")
    os.makedirs(gen, exist_ok=True)
    paths = []
    for k, e, cl in INSTANCES:
        lines = ['#include "tensilelite_gb300/csrc/gemm_tc_kernel.cuh"', "namespace tl {", "namespace tc {"]
        for td in (EPI_OUT_TYPES if e else OUT_TYPES):
            lines.append(f"template tl_status launch_kernel<{k}, {td}, {cl}, {'true' if e else 'false'}>("
                         "const TcKernelParams&, int, size_t, cudaStream_t);")
            if not e:
                lines.append(f"template int max_clusters<{k}, {td}, {cl}>(size_t);")
        lines += ["}  // namespace tc", "}  // namespace tl", ""]
        text = "\n".join(lines)
        path = os.path.join(gen, f"tc_k{k}_e{int(e)}_c{cl}.cu")
        if not os.path.exists(path) or open(path).read() != text:
            with open(path, "w") as f:
                f.write(text)
        paths.append(path)
    return paths
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden", "-I" + ROOT]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "tensilelite.h"))
    nv = nvcc()
    jobs = []
    objs = []
    for path in [os.path.join(CSRC, src) for src in SOURCES] + _instance_sources():
        src = os.path.basename(path)
        obj = os.path.join(BUILD, src + ".o")
        objs.append(obj)
        if force or _stale(obj, [path] + headers):
            cmd = [nv] + ARCH + COMMON + ["-c", path, "-o", obj]
            if src.endswith(".cpp"):
                cmd = [nv] + COMMON + ["-x", "cu"] + ARCH + ["-c", path, "-o", obj]
            jobs.append(cmd)
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    if force or jobs or _stale(LIB, objs):
        _run([nv] + ARCH + ["-shared", "-o", LIB] + objs + ["-Xcompiler", "-fvisibility=hidden"])
    cli_src = os.path.join(CSRC, "tl_cli.cpp")
    if os.path.exists(cli_src) and (force or _stale(CLI, [cli_src, LIB] + headers)):
        _run([nv, "-O2", "-std=c++17", "-I" + ROOT, "-x", "cu"] + ARCH +
             [cli_src, "-o", CLI, "-L" + HERE, "-ltensilelite_gb300", "-Xlinker", "-rpath=$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
