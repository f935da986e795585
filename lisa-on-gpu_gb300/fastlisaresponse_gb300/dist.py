"""Sharding sources across GPUs (one process per GPU).

Sources are independent, so a batch shards by source with no collective on
the data path: each rank evaluates its share on its own GPU.  The only
collective is the reduction of timings (the job time is the slowest rank's).
"""

from __future__ import annotations

import heapq
from typing import List, Sequence


def shard_by_samples(lengths: Sequence[int], rank: int, world: int) -> List[int]:
    """Indices of the sources rank `rank` of `world` evaluates: longest first,
    each to the rank with the fewest samples so far (LPT), so ranks get nearly
    equal work.  The shards partition range(len(lengths)) and each is in
    ascending order."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    heap = [(0, r) for r in range(world)]
    owner = [0] * len(lengths)
    for i in sorted(range(len(lengths)), key=lambda i: (-int(lengths[i]), i)):
        load, r = heapq.heappop(heap)
        owner[i] = r
        heapq.heappush(heap, (load + int(lengths[i]), r))
    return [i for i in range(len(lengths)) if owner[i] == rank]


def max_over_ranks(values: Sequence[float], device=None) -> List[float]:
    """Element-wise maximum over the ranks of the default process group (the
    values unchanged when torch.distributed is not initialised)."""
    import torch
    import torch.distributed as td

    if not (td.is_available() and td.is_initialized()) or td.get_world_size() == 1:
        return [float(v) for v in values]
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]
