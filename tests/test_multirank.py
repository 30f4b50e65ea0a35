"""The N > 1 path of bench.py on CPU ranks (gloo, world size 2): replicas
with max-over-ranks time and summed throughput, and the reference arm where
only rank 0 works."""
import json
import os
import socket
import subprocess
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.dist_init("gloo")
    t = bench.reduce_max(1.0 + rank, d)          # per-rank step time
    v = bench.reduce_sum(10.0 * (rank + 1), d)    # per-rank throughput
    bench.barrier(d)
    out[rank] = (t, v)
    dist.destroy_process_group()


def test_replica_aggregation_two_ranks():
    ws = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_worker, args=(ws, _free_port(), out), nprocs=ws, start_method="spawn")
    assert out[0] == out[1] == (2.0, 30.0)


def test_reference_arm_under_torchrun_rank0_only():
    env = dict(os.environ, OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr=127.0.0.1", f"--master-port={_free_port()}", os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "3", "--mesh", "6"]
    r = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    j = json.loads(lines[0])
    assert j["impl"] == "reference" and j["value"] > 0 and j["n_gpus"] == 2
    assert j["cpu_baseline"]["kind"] in ("reference", "port")
    assert j["e2e"]["h2d_bytes_per_step"] == 0
    # the same workload description as the GPU arm's line
    assert j["config"]["workload"].startswith("BLU-SGS 5x5 face Jacobians") and j["config"]["colors"] > 1
