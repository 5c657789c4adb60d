"""CPU, world size 2 over gloo: the bench's replica plumbing. Scenes are independent, so ranks exchange no data on
the path; they only meet at a barrier and combine their timings (max) and particle counts (sum). The reference
arm under torchrun runs on rank 0 alone and prints one line."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench

    w, r = bench.dist_setup()
    bench.barrier(w)
    mx = bench.allreduce_max(w, 10.0 * (r + 1))
    sm = bench.allreduce_sum(w, 1000 + r)
    import torch.distributed as td

    td.destroy_process_group()
    q.put((r, w, mx, sm, os.environ.get("CUDA_VISIBLE_DEVICES")))


def test_two_ranks_meet_and_combine():
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[0] for o in out] == [0, 1]
    for r, w, mx, sm, vis in out:
        assert w == 2 and mx == 20.0 and sm == 2001  # max of per-rank times, sum of per-rank particles
        assert vis == str(r)  # one GPU per rank: the local rank's device


def test_reference_arm_under_torchrun_prints_once():
    port = free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr", "127.0.0.1",
           "--master-port", str(port), "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
