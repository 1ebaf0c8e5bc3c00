"""Replicas on several ranks: `bench.py --gpus N` runs one process per GPU,
each stepping its own galaxy with no data-path collective.  The host side of
that path runs here on CPU with the gloo backend at world size 2: every rank
seeds a different galaxy, the timing is the slowest rank's, the value counts
all ranks' body-steps over that time, and the reference arm's extra ranks
exit without work."""
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        w = bench.WORKLOADS["direct4096"]
        pm, _ = bench.seed_workload(w, bench.replica_seed(rank))
        own_ms = 10.0 + 5.0 * rank          # this rank's timed region
        slowest = bench.max_over_ranks(own_ms)
        out.put((rank, float(np.abs(pm[:, :3]).sum()), slowest,
                 bench.replicas_value(world, w["n"], 5, slowest)))
    finally:
        dist.destroy_process_group()


def test_two_replicas_gloo():
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
    (r0, sum0, max0, val0), (r1, sum1, max1, val1) = res
    assert (r0, r1) == (0, 1)
    assert sum0 != sum1                          # each replica steps its own galaxy
    assert max0 == max1 == 15.0                  # timed by the slowest rank
    assert val0 == val1 == pytest.approx(2 * 4096 * 5 / 15e-3)


def test_single_process_needs_no_group():
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.replicas_value(1, 1000, 10, 2.0) == pytest.approx(5.0e6)
    assert bench.replica_seed(0) != bench.replica_seed(1)


def test_reference_arm_extra_rank_exits_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                        "direct4096", "--steps", "1", "--warmup", "3"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
