"""The N > 1 path of bench.py on the CPU with the gloo backend (world size 2): rank
0 alone prints the reference arm's JSON line, and the timing helpers take the
maximum over ranks. The GPU arm runs independent replicas (no data-path
collective), so these are its only collective calls."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_reference_arm_under_torchrun_prints_one_line():
    env = dict(os.environ, EIF_BENCH_BACKEND="gloo", OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--workload", "couette_circle"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0


def _worker(rank, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=2)
    import bench
    bench.barrier(dist)
    out[rank] = bench.max_over_ranks(dist, 1.5 + rank, None)
    dist.destroy_process_group()


def test_max_over_ranks_with_gloo():
    import torch.multiprocessing as mp
    mgr = mp.get_context("spawn").Manager()   # no fork of a threaded process
    out = mgr.dict()
    mp.spawn(_worker, args=(_free_port(), out), nprocs=2, join=True)
    assert out[0] == 2.5 and out[1] == 2.5
