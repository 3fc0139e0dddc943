"""Multi-rank path on CPU: two gloo ranks shard a request by event range.

Each rank computes its own events with the oracle (standing in for its GPU); Generate shards
concatenate to the single-process result bit for bit, and the one AverageOn exchange (a 24-byte
StatsPHSP per rank, merged in rank order) gives every rank the same result as the in-process merge
of the same shards.
"""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from conftest import REPO

MASSES = [0.493677, 0.13957, 0.13957, 0.13957, 0.13957]


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, n, out_dir):
    import sys
    sys.path.insert(0, str(REPO))
    import torch.distributed as dist
    from hydra_gb300 import shard
    from oracle import oracle as O
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ch = O.make_channel(MASSES, 1.86484, 0x3039, O.ENGINE_PHILOX)
    fn = O.make_functor(2, 0, 1, 0.8955, 0.0473)
    first, count = shard.event_range(rank, world, n)
    four, w = O.generate(ch, first, count, nthreads=1)
    np.save(os.path.join(out_dir, f"four_{rank}.npy"), four)
    res = shard.average_on_sharded(n, 0, lambda f, m: O.average_on(ch, fn, f, m, nthreads=1))
    np.save(os.path.join(out_dir, f"avg_{rank}.npy"), np.array(res))
    dist.barrier()
    dist.destroy_process_group()


def test_event_range_partitions():
    from hydra_gb300 import shard
    for world in (1, 2, 3, 7):
        spans = [shard.event_range(r, world, 1000, 50) for r in range(world)]
        assert spans[0][0] == 50 and sum(c for _, c in spans) == 1000
        for (f0, c0), (f1, _) in zip(spans, spans[1:]):
            assert f0 + c0 == f1
    with pytest.raises(ValueError):
        shard.event_range(2, 2, 10)


def test_two_gloo_ranks(oracle, tmp_path):
    n, world = 20_001, 2
    mp.start_processes(_rank, args=(world, free_port(), n, str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    from hydra_gb300 import shard
    ch = oracle.make_channel(MASSES, 1.86484, 0x3039, oracle.ENGINE_PHILOX)
    fn = oracle.make_functor(2, 0, 1, 0.8955, 0.0473)
    four, _ = oracle.generate(ch, 0, n, nthreads=1)
    parts = [np.load(tmp_path / f"four_{r}.npy") for r in range(world)]
    assert np.array_equal(np.concatenate(parts, axis=1), four)
    a0, a1 = (np.load(tmp_path / f"avg_{r}.npy") for r in range(world))
    assert np.array_equal(a0, a1)                                   # every rank agrees
    local = shard.merge_in_order([oracle.average_on(ch, fn, f, m, nthreads=1)
                                  for f, m in (shard.event_range(r, world, n) for r in range(world))])
    assert tuple(a0) == local
    seq = oracle.average_on(ch, fn, 0, n, nthreads=1)
    assert abs(a0[0] - seq[0]) <= 1e-12 * abs(seq[0]) and abs(a0[2] - seq[2]) <= 1e-12 * seq[2]
