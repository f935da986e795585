"""Tile-length autotuner for the batched response + TDI kernel.

A work item of the persistent kernel is one tile of T output samples of one
source.  Per item the kernel stages an input window, computes the six link
streams over the tile plus a halo on each side (the largest TDI delay in
samples plus the Lagrange half-width), then the TDI channels of the tile.
Short tiles spend more of their time on halos and per-item set-up; long tiles
leave SMs idle when a batch has few tiles, and the latency of one item (a CTA
works through its tile serially) grows with T.  The best T depends on the
Lagrange order (halo and taps), the TDI generation (delay depth: halo), the
arithmetic (registers and shared memory, hence CTAs per SM) and the batch
size, so it is measured.

:func:`best_tile` times each candidate tile on a synthetic batch of
galactic-binary sources generated on the device (lengths as given, by default
a mid-sized batch), with CUDA events on the current stream, and returns the
fastest.  Results are cached in memory and in a JSON file (``FLR_TUNE_CACHE``,
default ``~/.cache/fastlisaresponse_gb300/tiles.json``) under a key made of
the GPU name, precision, Lagrange order, TDI sets, output channels, orbit kind
(equal arms or not), sampling frequency and the batch's size class (log2 of
its output samples).  ``BatchedResponseTDI(tile="auto")`` calls it.
"""

from __future__ import annotations

import json
import math
import os
import threading
from typing import Dict, Optional, Sequence

import numpy as np

TILE_CANDIDATES = (128, 256, 512, 768, 1024, 2048)
DEFAULT_TUNE_LENGTHS = (2**18,) * 32

_memo: Dict[str, dict] = {}
_lock = threading.Lock()


def cache_path() -> str:
    return os.environ.get("FLR_TUNE_CACHE") or os.path.join(
        os.path.expanduser("~"), ".cache", "fastlisaresponse_gb300", "tiles.json")


def _load() -> dict:
    try:
        with open(cache_path()) as fh:
            data = json.load(fh)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def _store(key: str, entry: dict) -> None:
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        data = _load()
        data[key] = entry
        tmp = f"{path}.{os.getpid()}.tmp"
        with open(tmp, "w") as fh:
            json.dump(data, fh, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass  # a read-only home: the in-memory cache still applies


def equal_arms(orbits) -> bool:
    """True when all six light travel times agree at every knot."""
    ltt = np.asarray(orbits.pycppdetector_args[3], dtype=np.float64).reshape(-1, 6)
    return bool(np.all(ltt == ltt[:, :1]))


def size_class(lengths: Sequence[int], tdi_start: int) -> int:
    total = sum(max(int(n) - 2 * tdi_start, 0) for n in lengths)
    return int(math.floor(math.log2(max(total, 1))))


def tune_key(device_name: str, precision: str, order: int, tdi_sets: list, tdi_chan: str,
             equal: bool, sampling_frequency: float, cls: int) -> str:
    sets = ";".join(f"{t['num_units']}:{len(t['tdi_link_combinations'])}" for t in tdi_sets)
    return (f"{device_name}|{precision}|order{order}|tdi[{sets}]|{tdi_chan}|"
            f"{'equal' if equal else 'flex'}|fs{sampling_frequency!r}|2^{cls}")


def measure(make_plan, lengths: Sequence[int], candidates: Sequence[int], device,
            reps: int = 3, seed: int = 0) -> Dict[int, float]:
    """Seconds per batch for each candidate tile (median of `reps` timed runs
    after one warm-up, device time only); make_plan(tile) returns a
    BatchedResponseTDI."""
    import torch

    from ._lib import FLRError
    from .waveforms import draw_gb_parameters

    rng = np.random.default_rng(seed)
    p = draw_gb_parameters(rng, len(lengths))
    prm = np.stack([p[k] for k in ("A", "f", "fdot", "iota", "phi0", "psi")], axis=1)
    timings = {}
    hs = None
    for tile in candidates:
        try:
            plan = make_plan(int(tile))
        except (FLRError, ValueError):  # e.g. the window does not fit in shared memory
            continue
        if hs is None:  # the same waveforms for every candidate
            _, hs = plan.run_gb(prm, lengths, p["lam"], p["beta"])
        plan(hs, p["lam"], p["beta"])
        stream = torch.cuda.current_stream(device)
        times = []
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            # hold the stream ~1 ms so the host has queued the run when e0 fires
            torch.cuda._sleep(2_000_000)
            e0.record(stream)
            plan(hs, p["lam"], p["beta"])
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) * 1e-3)
        if plan.status() != 0:
            raise RuntimeError(f"tile {tile}: kernel status {plan.status():#x}")
        timings[int(tile)] = float(np.median(times))
        del plan
    return timings


def best_tile(sampling_frequency, order, tdi, orbits, precision, tdi_chan="XYZ",
              t_buffer=10000.0, force_backend=None, lengths: Optional[Sequence[int]] = None,
              candidates: Sequence[int] = TILE_CANDIDATES, use_cache: bool = True) -> dict:
    """Fastest tile for this configuration: {"tile", "key", "timings"
    (seconds per candidate), "lengths", "cached"}."""
    import torch

    from .batch import BatchedResponseTDI, _combinations
    from .response import _orbit_instance, _resolve_device, tdi_unit_tables

    device = _resolve_device(force_backend)
    orbits = _orbit_instance(orbits)
    lengths = [int(n) for n in (lengths if lengths is not None else DEFAULT_TUNE_LENGTHS)]
    specs = tdi if (isinstance(tdi, (list, tuple)) and tdi and
                    not isinstance(tdi[0], dict)) else [tdi]
    sets = [tdi_unit_tables(_combinations(s)) for s in specs]
    tdi_start = int(t_buffer * sampling_frequency)
    key = tune_key(torch.cuda.get_device_name(device), precision, order, sets, tdi_chan,
                   equal_arms(orbits), sampling_frequency, size_class(lengths, tdi_start))
    if use_cache:
        with _lock:
            hit = _memo.get(key) or _load().get(key)
        if hit and int(hit.get("tile", 0)) in set(int(c) for c in candidates):
            _memo[key] = hit
            return dict(hit, key=key, cached=True)

    def make_plan(tile):
        return BatchedResponseTDI(sampling_frequency, order=order, tdi=tdi, orbits=orbits,
                                  tdi_chan=tdi_chan, precision=precision, t_buffer=t_buffer,
                                  tile=tile, force_backend=device)

    timings = measure(make_plan, lengths, candidates, device)
    if not timings:
        raise RuntimeError("no candidate tile fits this configuration")
    best = min(timings, key=timings.get)
    entry = {"tile": best, "timings": {str(k): v for k, v in timings.items()},
             "lengths": [min(lengths), max(lengths), len(lengths)]}
    with _lock:
        _memo[key] = entry
        if use_cache:
            _store(key, entry)
    return dict(entry, key=key, cached=False)
