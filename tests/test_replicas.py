"""Replica scaling of bench.py on CPU (no GPU): the max-over-ranks reduction
and the whole-job rate over a world-size-2 gloo process group, and the
reference arm under two ranks (rank 0 alone prints, rank 1 exits 0 without
work)."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    seconds = [2.0, 3.0][rank]
    slowest = bench.max_over_ranks(seconds, dist, device="cpu")
    rate = bench.aggregate_rate(world, 1000, 50, 10, slowest)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, slowest, rate))


def test_max_over_ranks_and_rate_with_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, slowest, rate in got:
        assert slowest == 3.0                     # every rank sees the slowest rank's time
        assert rate == 2 * 1000 * 50 * 10 / 3.0   # both replicas' work over that time


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(1.5, None) == 1.5
    assert bench.aggregate_rate(1, 10, 50, 2, 1.0) == 1000.0


def test_reference_arm_under_two_ranks():
    port = _free_port()
    outs = []
    for rank in range(2):
        env = dict(os.environ, WORLD_SIZE="2", RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), OMP_NUM_THREADS="2")
        outs.append(subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                                    "--workload", "c0", "--steps", "1", "--warmup", "3"],
                                   env=env, capture_output=True, text=True, timeout=600))
    assert outs[0].returncode == 0, outs[0].stderr[-2000:]
    assert outs[1].returncode == 0, outs[1].stderr[-2000:]
    assert outs[1].stdout.strip() == ""
    line = json.loads([l for l in outs[0].stdout.splitlines() if l.startswith("{")][-1])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["e2e"]["value"] == line["value"] and line["cpu_baseline"]["kind"] == "port"
