"""Multi-rank batch sharding (host logic of the N-GPU path), world_size 2 over
gloo on CPU: every path lands on exactly one rank, the work is balanced, and
the per-rank results (CPU oracle standing in for each rank's GPU) assemble to
the single-rank result."""
import importlib
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, queue):
    import sys

    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    sharding = importlib.import_module("rough-path-primitives_gb300.sharding")
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rng = np.random.default_rng(7)
    W, D = 3, 3
    lengths = rng.integers(0, 40, 57)
    offsets = np.concatenate([[0], np.cumsum(lengths)]).astype(np.int64)
    incr = rng.normal(0, 0.3, (offsets[-1], W))
    b0, b1, local = sharding.shard_offsets(offsets, world, rank)
    sig, _ = O.Oracle().signature(W, D, incr[offsets[b0]:offsets[b1]], local)
    gathered = [None] * world
    dist.all_gather_object(gathered, (b0, b1, int(local[-1]), sig))
    if rank == 0:
        full, _ = O.Oracle().signature(W, D, incr, offsets)
        queue.put((gathered, full, int(offsets[-1])))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sharding_covers_batch_and_balances_work():
    world = 2
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, queue)) for r in range(world)]
    for p in procs:
        p.start()
    gathered, full, total = queue.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    bounds = [(g[0], g[1]) for g in gathered]
    assert bounds[0][0] == 0 and bounds[-1][1] == full.shape[0]
    assert all(bounds[i][1] == bounds[i + 1][0] for i in range(world - 1))
    steps = [g[2] for g in gathered]
    assert sum(steps) == total and max(steps) - min(steps) <= 40
    assembled = np.concatenate([g[3] for g in gathered])
    assert np.array_equal(assembled, full)


def test_shard_bounds_edge_cases():
    sharding = importlib.import_module("rough-path-primitives_gb300.sharding")
    assert sharding.shard_bounds([0], 4, 2) == (0, 0)
    offs = np.array([0, 0, 0, 10])
    assert [sharding.shard_bounds(offs, 2, r) for r in range(2)] == [(0, 3), (3, 3)]
    offs = np.array([0, 4, 8, 12, 16])
    assert [sharding.shard_bounds(offs, 2, r) for r in range(2)] == [(0, 2), (2, 4)]
    with pytest.raises(ValueError):
        sharding.shard_bounds(offs, 2, 2)
