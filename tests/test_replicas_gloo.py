"""The N > 1 path of bench.py on CPU: world-size-2 gloo process groups.

The batched path shards by replica: every rank integrates its own
independent ensemble (seeded by rank), with no collective on the data path;
the ranks meet only at the barriers around the timed region and in the
max-over-ranks reduction of the timed duration.  The reference arm runs on
rank 0 alone; the other ranks exit without work.
"""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        bench.barrier(world)
        slowest = bench.max_over_ranks(10.0 * (rank + 1), world)
        ens = bench.make_workload("ensemble8", 4, rank)
        sig = torch.tensor([float(np.sum(ens["body_f64"][:, :, 5:8]))], dtype=torch.float64)
        sigs = [torch.zeros(1, dtype=torch.float64) for _ in range(world)]
        dist.all_gather(sigs, sig)
        bench.barrier(world)
        out.put((rank, slowest, [float(x.item()) for x in sigs], ens["n_sys"]))
    finally:
        dist.destroy_process_group()


def test_two_replicas_meet_only_at_barriers_and_the_max():
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
    for rank, slowest, sigs, n_sys in res:
        assert slowest == 20.0            # the slower rank's time
        assert n_sys == 4
        assert sigs[0] != sigs[1]          # each rank integrates its own ensemble
    import bench
    # whole-job throughput: both replicas' systems over the slowest rank's time
    assert bench.replica_value(2, 4096, 100, 20.0) == 2 * 4096 * 100 / 0.02


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    args = type("A", (), {"workload": "ensemble8", "n_systems": 4, "steps": 1, "warmup": 1})()
    buf = io.StringIO()
    with redirect_stdout(buf):
        bench.run_reference(args)
    assert buf.getvalue() == ""
