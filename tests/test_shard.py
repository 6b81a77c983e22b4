"""Replica sharding: the split is deterministic and balanced, and the
cross-rank combination (sum of work, slowest time) holds under two gloo ranks
on the CPU."""
import os
import socket

import pytest

from halmd_gb300.shard import combine, partition


def test_partition_is_balanced_and_complete():
    w = [500 + (k * 7919) % 31500 for k in range(256)]      # ensemble-like sizes
    for nparts in (1, 2, 3, 4, 8):
        parts = partition(w, nparts)
        flat = sorted(k for p in parts for k in p)
        assert flat == list(range(len(w)))
        loads = [sum(w[k] for k in p) for p in parts]
        assert max(loads) - min(loads) <= max(w)              # LPT bound
        assert partition(w, nparts) == parts                  # every rank computes the same split


def test_partition_edge_cases():
    assert partition([], 2) == [[], []]
    assert partition([5], 3) == [[0], [], []]
    assert partition([1, 1, 1, 1], 2) == [[0, 2], [1, 3]]
    with pytest.raises(ValueError):
        partition([1], 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        work, ms = combine(1000.0 * (rank + 1), 10.0 + rank, device="cpu")
        q.put((rank, work, ms))
    finally:
        dist.destroy_process_group()


def test_combine_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    out = sorted(q.get(timeout=10) for _ in range(2))
    for _, work, ms in out:
        assert work == 3000.0 and ms == 11.0


def test_combine_without_process_group():
    assert combine(5.0, 2.0) == (5.0, 2.0)
