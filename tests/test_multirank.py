"""The N-GPU path of bench.py, on CPU: replicas (one rank per GPU) with no
exchange inside a step; each rank integrates its own seeded batch and the job
time is the largest over the ranks. Two gloo ranks here."""
import json
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        m = bench.max_over_ranks(10.0 * (rank + 1), ws, "cpu")
        mech, state, dt = bench.workload_inputs(16, rank, "53")
        out.put((rank, m, state.sum(), dt.sum(), mech.n_species))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_share_the_slowest_time_and_get_distinct_batches():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, m0, s0, d0, n0), (r1, m1, s1, d1, n1) = res
    assert m0 == m1 == 20.0                  # max over ranks on both
    assert n0 == n1 == 53                    # the same mechanism
    assert s0 != s1 and d0 != d1             # each rank its own seeded states (weak scaling)


def test_reference_arm_under_torchrun_prints_one_line():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--points", "16",
           "--mech", "53", "--cpu-seconds", "0.2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "points/s"
