"""Multi-GPU host logic (replicas only) on CPU with two gloo ranks: every
rank runs its own replica (distinct noise replica id and initial state), the
reported time is the slowest rank's, and no data moves between ranks."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        w = bench.WORKLOADS["cfg1"]
        cfg, (x, p) = bench.rank_workload(w, "fp64", rank)
        t = bench.max_over_ranks(0.5 + rank, dist, device="cpu")
        # the per-rank inputs, gathered only to check them here
        xs = [torch.zeros(x.size, dtype=torch.float64) for _ in range(world)]
        dist.all_gather(xs, torch.from_numpy(np.ascontiguousarray(x).ravel()))
        out[rank] = (cfg.replica, t, [float(torch.abs(xs[0] - xs[k]).max()) for k in range(world)])
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_run_independent_replicas():
    pytest.importorskip("torch.distributed")
    world = 2
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    assert sorted(out.keys()) == [0, 1]
    for rank in range(world):
        replica, t, diffs = out[rank]
        assert replica == rank            # distinct noise streams
        assert t == 0.5 + (world - 1)     # the slowest rank's time
        assert diffs[0] == 0.0 and diffs[1] > 0.0  # distinct initial states
