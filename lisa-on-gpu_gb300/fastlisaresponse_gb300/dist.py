"""Sharding across GPUs (one process per GPU).

Sources are independent, so a batch shards by source with no collective on
the data path: each rank evaluates its share on its own GPU.  One long source
shards by time: each rank computes a tile-aligned range of its output samples
from the slice of the input its delays reach (the reference's kernels stride
over samples the same way inside one GPU, LISAResponse.cu:293-302, 526-535);
the ranges partition the output, no exchange is needed.  The only collective
is the reduction of timings (the job time is the slowest rank's).
"""

from __future__ import annotations

import heapq
from typing import List, Optional, Sequence, Tuple


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


def shard_time(n: int, tdi_start: int, tile: int, rank: int,
               world: int) -> Optional[Tuple[int, int]]:
    """Output range [begin, end) of rank `rank` of `world` for one source of n
    samples whose outputs are [tdi_start, n - tdi_start), cut at multiples of
    the tile from tdi_start (the batched kernel's work items), the tiles
    spread as evenly as possible; None when the rank has no tile.  The ranges
    of all ranks partition the output range in rank order."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    if tile < 1 or 2 * tdi_start >= n:
        raise ValueError("need tile >= 1 and 2 * tdi_start < n")
    tiles = -(-(n - 2 * tdi_start) // tile)
    first, last = rank * tiles // world, (rank + 1) * tiles // world
    if first == last:
        return None
    return tdi_start + first * tile, min(tdi_start + last * tile, n - tdi_start)


def input_range(out_range: Tuple[int, int], n: int, reach: int) -> Tuple[int, int]:
    """Input samples [lo, hi) an output range reads: the range widened by the
    reach of its delays, link-stream halo and taps on each side."""
    a, b = out_range
    return max(0, a - reach), min(n, b + reach)
