"""bench.py under a multi-process launch, on CPU.

The library is a one-GPU deliverable (its cluster-of-four kernel uses TMA multicast, kept to one-GPU
runs), so bench.py launched with WORLD_SIZE > 1 must not run the GPU arm at all: rank 0 prints one
line saying so and every rank exits 0 before touching CUDA.  The reference arm uses host cores only
and runs on rank 0 alone; the other ranks exit without output."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench(rank, *args):
    # CUDA_VISIBLE_DEVICES="" makes any attempt to use a GPU fail loudly, even on a GPU host
    env = dict(os.environ, WORLD_SIZE="2", RANK=str(rank), LOCAL_RANK=str(rank), CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([sys.executable, "bench.py", *args], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    return [l for l in r.stdout.splitlines() if l.startswith("{")]


@pytest.mark.parametrize("rank", [0, 1])
def test_gpu_arm_refuses_world_size_2(rank):
    lines = _bench(rank, "--steps", "2", "--warmup", "3")
    if rank == 1:
        assert lines == []
    else:
        assert len(lines) == 1
        line = json.loads(lines[0])
        assert line["n_gpus"] == 2 and line["impl"] == "tensilelite_gb300"
        assert "one GPU only" in line["unavailable"] and "value" not in line


def test_gpu_arm_refusal_imports_no_cuda_library():
    """The refusal happens before torch or the library is imported."""
    code = ("import os, sys, runpy; os.environ.update(WORLD_SIZE='2', RANK='0'); sys.argv=['bench.py'];"
            "runpy.run_path('bench.py', run_name='__main__');"
            "print('LOADED', sorted(m for m in ('torch', 'tensilelite_gb300') if m in sys.modules))")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert "LOADED []" in r.stdout


@pytest.mark.parametrize("rank", [0, 1])
def test_reference_arm_rank0_only(rank):
    lines = _bench(rank, "--impl", "reference", "--workload", "simt_fp32_480x512x512", "--steps", "2",
                   "--warmup", "3")
    if rank == 1:
        assert lines == []
    else:
        line = json.loads(lines[-1])
        assert line["impl"] == "reference" and line["unit"] == "TFLOP/s" and line["value"] > 0
        assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0


def test_reference_arm_line_carries_the_contract_keys():
    """One process (no WORLD_SIZE): the reference arm's line has every key of the bench contract,
    on the workload and metric of the GPU arm's headline."""
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    env["CUDA_VISIBLE_DEVICES"] = ""
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3"], cwd=ROOT,
                       env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr
    line = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["n_gpus"] == 1 and line["steps"] == 1 and line["warmup"] >= 3
    assert line["higher_is_better"] is True and line["unit"] == "TFLOP/s" and line["value"] > 0
    assert line["config"]["workload"].startswith("bf16_4096_nn")
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["e2e"]["d2h_bytes_per_step"] == 0
