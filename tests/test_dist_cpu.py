"""The benchmark's multi-process path on CPU (gloo, world size 2): the path
does not shard, so N GPUs run N replicas; what is shared is the barrier, the
max-over-ranks timing and rank 0's single output line."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank), SBP_BENCH_BACKEND="gloo")
    sys.path.insert(0, str(ROOT))
    import bench
    d = bench.Dist(world)
    d.barrier()
    q.put((rank, d.max(1.5 * (rank + 1)), d.rank, d.world))
    d.barrier()
    d.close()


def test_dist_barrier_and_max_over_ranks():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(o[0] for o in out) == [0, 1]
    assert all(o[1] == 3.0 and o[3] == 2 and o[2] == o[0] for o in out)


def test_reference_arm_under_torchrun_two_ranks():
    # rank 0 alone runs the CPU baseline and prints the one JSON line; the
    # other rank exits 0 without work
    env = dict(os.environ, SBP_BENCH_BACKEND="gloo", OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py",
           "--impl", "reference", "--gpus", "2", "--grid", "129", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["config"]["n"] == 129
    assert d["cpu_baseline"]["kind"] == "port" and d["value"] > 0
