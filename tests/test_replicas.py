"""Multi-rank logic on CPU: two gloo ranks split a batch, time, and sum a gradient.

The GPU path shards by batch column with no collective; only a batch-split gradient needs one sum of
dJ/dp.  Here each rank computes the oracle's exact gradient of its own columns (complex128, CPU), the
ranks sum them with ``allreduce_grad``, and the sum must equal the full-batch gradient.
"""
import os
import socket
import tempfile

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from meshes_gb300.replicas import allreduce_grad, max_over_ranks, shard_range
from oracle import meshes_oracle as O


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out_dir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rng = np.random.default_rng(5)
        om = O.random_mesh(rng, 16, "clements", "mzi", 0.02)
        B = 37
        x = O.unit_columns(rng, 16, B)
        t = O.unit_columns(rng, 16, B)
        b0, b1 = shard_range(B, rank, world)
        y = O.propagate(om, x[b0:b1])
        G, _, _ = O.vjp_unitary(om, y, 2 * (y - t[b0:b1]))
        dp_local = torch.tensor(O.contract_dp(om, G), dtype=torch.float32)
        dp = allreduce_grad(dp_local)
        t_max = max_over_ranks(0.5 + rank)
        np.save(os.path.join(out_dir, "dp%d.npy" % rank), dp.numpy())
        np.save(os.path.join(out_dir, "t%d.npy" % rank), np.array([t_max, b0, b1]))
    finally:
        dist.destroy_process_group()


def test_shard_range_covers_the_batch():
    for B in (0, 1, 5, 37, 4096):
        for world in (1, 2, 3, 8):
            spans = [shard_range(B, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == B
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            assert max(b - a for a, b in spans) - min(b - a for a, b in spans) <= 1
    with pytest.raises(ValueError):
        shard_range(4, 2, 2)


def test_two_gloo_ranks_split_batch_and_sum_gradient():
    world = 2
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_worker, args=(world, _free_port(), d), nprocs=world, join=True, start_method="spawn")
        dps = [np.load(os.path.join(d, "dp%d.npy" % r)) for r in range(world)]
        ts = [np.load(os.path.join(d, "t%d.npy" % r)) for r in range(world)]
    assert np.array_equal(dps[0], dps[1])                      # every rank holds the same sum
    assert all(t[0] == 1.5 for t in ts)                        # the slowest rank's time
    assert ts[0][1] == 0 and ts[0][2] == ts[1][1] and ts[1][2] == 37
    rng = np.random.default_rng(5)
    om = O.random_mesh(rng, 16, "clements", "mzi", 0.02)
    x = O.unit_columns(rng, 16, 37)
    t = O.unit_columns(rng, 16, 37)
    y = O.propagate(om, x)
    G, _, _ = O.vjp_unitary(om, y, 2 * (y - t))
    full = O.contract_dp(om, G)
    assert O.rel_err(dps[0], full) < 1e-6                       # float32 sum of the two halves
