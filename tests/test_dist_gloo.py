"""Multi-rank logic on the CPU: two gloo ranks shard a batch of sources and
reduce their timings (the path bench.py takes under torchrun)."""

import os
import socket

import numpy as np
import pytest

from fastlisaresponse_gb300.dist import max_over_ranks, shard_by_samples


def test_shards_partition_and_balance():
    rng = np.random.default_rng(0)
    lengths = np.exp(rng.uniform(np.log(2**15), np.log(2**22), 2048)).astype(int)
    for world in (1, 2, 4, 8):
        shards = [shard_by_samples(lengths, r, world) for r in range(world)]
        flat = sorted(i for s in shards for i in s)
        assert flat == list(range(len(lengths)))
        loads = [int(lengths[s].sum()) for s in shards]
        assert max(loads) - min(loads) <= int(lengths.max())
    with pytest.raises(ValueError):
        shard_by_samples([1, 2], 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, lengths, q):
    import torch.distributed as td

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    td.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = shard_by_samples(lengths, rank, world)
        work = float(sum(lengths[i] for i in mine))
        reduced = max_over_ranks([work, float(rank)])
        q.put((rank, mine, work, reduced))
    finally:
        td.destroy_process_group()


def test_two_gloo_ranks_shard_and_reduce():
    import torch.multiprocessing as mp

    lengths = [int(x) for x in np.random.default_rng(1).integers(1000, 100000, 37)]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, lengths, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, s0, w0, red0), (r1, s1, w1, red1) = results
    assert sorted(s0 + s1) == list(range(len(lengths)))
    assert red0 == red1 == [max(w0, w1), 1.0]


def test_time_shards_partition_the_output():
    """One source's output range cut into tile-aligned shards: contiguous,
    in rank order, covering [ts, n - ts) exactly, balanced to one tile."""
    from fastlisaresponse_gb300.dist import input_range, shard_time

    for n, ts, tile in ((6311629, 2000, 512), (50000, 1000, 256), (5000, 1000, 512)):
        tiles = -(-(n - 2 * ts) // tile)
        for world in (1, 2, 3, 4, 8, 64):
            rngs = [shard_time(n, ts, tile, r, world) for r in range(world)]
            got = [r for r in rngs if r is not None]
            assert got[0][0] == ts and got[-1][1] == n - ts
            for (a0, b0), (a1, b1) in zip(got, got[1:]):
                assert b0 == a1 and (a1 - ts) % tile == 0
            sizes = [-(-(b - a) // tile) for a, b in got]
            assert sum(sizes) == tiles and max(sizes) - min(sizes) <= 1
            assert len(got) == min(world, tiles)
            for a, b in got:
                lo, hi = input_range((a, b), n, 100)
                assert lo == max(0, a - 100) and hi == min(n, b + 100)
    with pytest.raises(ValueError):
        shard_time(100, 60, 16, 0, 1)


def _time_worker(rank, world, port, n, ts, tile, q):
    import torch
    import torch.distributed as td

    from fastlisaresponse_gb300.dist import shard_time

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    td.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r = shard_time(n, ts, tile, rank, world)
        mine = torch.tensor(list(r) if r else [-1, -1], dtype=torch.int64)
        allr = [torch.zeros(2, dtype=torch.int64) for _ in range(world)]
        td.all_gather(allr, mine)
        q.put((rank, [tuple(x.tolist()) for x in allr]))
    finally:
        td.destroy_process_group()


def test_two_gloo_ranks_time_shard_one_source():
    """Each rank computes its own range; gathered, they are the same on both
    ranks and tile the output."""
    import torch.multiprocessing as mp

    n, ts, tile = 6311629, 2000, 512
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_time_worker, args=(r, 2, port, n, ts, tile, q))
             for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (_, a), (_, b) = results
    assert a == b and a[0][0] == ts and a[0][1] == a[1][0] and a[1][1] == n - ts
