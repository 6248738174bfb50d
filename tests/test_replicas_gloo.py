"""The N > 1 path of bench.py on CPU: two ranks over gloo (127.0.0.1).  The build does not shard
(one index is built on one GPU), so N ranks run independent replicas and the
only cross-rank operations are the barrier and the max of the per-rank times."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(world)
    q.put((rank, bench.allmax(float(10 + rank), world)))
    dist.destroy_process_group()


def test_allmax_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == {0: 11.0, 1: 11.0}


def test_reference_arm_under_torchrun_prints_once():
    port = 30500 + os.getpid() % 1000
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl",
           "reference", "--gpus", "2", "--points", "1500", "--dim", "32", "--steps", "1", "--warmup", "0",
           "--cpu-seconds", "2"]
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="", OMP_NUM_THREADS="2")
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["ms_per_step"] is not None and line["ms_per_step"] > 0  # the whole build fit


def test_metric_names():
    """The default workload's metric string, and the batched form naming its sub-indexes."""
    sys.path.insert(0, ROOT)
    import argparse
    import bench
    a = argparse.Namespace(n=1_000_000, d=200, degree=32, beam=64, cosine=False, batched=0)
    assert bench.metric_name(a) == ("distance_evals_per_s (build, 1Mx200 IP, M=32, L=64, "
                                    "screened vs FP32, identical edges)")
    a = argparse.Namespace(n=1_000_000, d=512, degree=32, beam=64, cosine=False, batched=64)
    assert "64 sub-indexes, 9769080x512" in bench.metric_name(a, 9769080)
