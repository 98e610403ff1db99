"""The N > 1 path of bench.py on CPU: world-size-2 gloo ranks render
independent replicas (disjoint seeds), the job time is the max over ranks,
the value is the whole-job rate, and the reference arm runs on rank 0 only."""
import json
import os
import socket
import subprocess
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        ms = 10.0 + 7.5 * rank  # a slower second rank
        t = bench.max_over_ranks(ms)
        res = {"seed": bench.replica_seed(rank), "max_ms": t,
               "rate": bench.whole_job_rate(world, 1000, 4, t)}
        with open(os.path.join(out, f"r{rank}.json"), "w") as f:
            json.dump(res, f)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_aggregate_like_the_bench(tmp_path):
    port = _free_port()
    mp.start_processes(_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    r = [json.load(open(tmp_path / f"r{i}.json")) for i in range(2)]
    assert r[0]["seed"] != r[1]["seed"]  # independent replicas
    assert r[0]["max_ms"] == r[1]["max_ms"] == 17.5  # the slowest rank times the job
    assert r[0]["rate"] == r[1]["rate"] == 2 * 1000 * 4 / 17.5e-3 / 1e6


def test_single_process_needs_no_group():
    assert bench.max_over_ranks(3.25) == 3.25
    assert bench.whole_job_rate(1, 2_073_600, 10, 36.0) == 2_073_600 * 10 / 0.036 / 1e6


def test_reference_arm_prints_only_on_rank_zero():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    res = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "3"], capture_output=True, text=True, env=env, timeout=120)
    assert res.returncode == 0 and res.stdout.strip() == ""
