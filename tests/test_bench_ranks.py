"""bench.py's multi-process plumbing on CPU: two gloo ranks aggregate the way the bench reports a
whole-job number (the slowest rank's time, the summed work), and the reference arm runs on rank 0
only while the other ranks exit without output."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    bench.barrier(world)
    t = bench.max_over_ranks(1.0 + rank, world)          # rank times 1.0 and 2.0
    w = bench.sum_over_ranks(10.0 * (rank + 1), world)   # work 10 and 20
    q.put((rank, t, w))
    dist.destroy_process_group()


def test_rank_aggregation_gloo():
    import multiprocessing as mp
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [2.0, 2.0]      # max over ranks
    assert [o[2] for o in out] == [30.0, 30.0]    # sum over ranks


@pytest.mark.parametrize("rank", [0, 1])
def test_reference_arm_rank0_only(rank):
    env = dict(os.environ, WORLD_SIZE="2", RANK=str(rank), LOCAL_RANK=str(rank))
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "simt_fp32_480x512x512",
                        "--steps", "2", "--warmup", "3"], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    if rank == 1:
        assert lines == []
    else:
        line = json.loads(lines[-1])
        assert line["impl"] == "reference" and line["unit"] == "TFLOP/s" and line["value"] > 0
        assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
