"""Continuous-batching service for response + TDI requests.

Many likelihood samplers submit single evaluations -- a galactic-binary
source (7 waveform/sky parameters), a length and a TDI generation -- at any
time.  :class:`ResponseServer` keeps the orbit and Lagrange tables resident on
the GPU, admits requests against an HBM budget (each request needs its three
output channels, 24 bytes per sample: its waveform is generated inside the
kernel, straight into the staged input window), and packs the admitted
requests into one persistent fused response + TDI launch per batch
(:meth:`BatchedResponseTDI.run_gb` with ``keep_waveforms=False``), replayed
from the CUDA graph of the batch's size bucket (sources rounded up to a power
of two; lengths are free).
Batches go to ``num_streams`` CUDA
streams, so a batch formed from requests that arrived while others were
running starts right away and overlaps with them on the device; memory
returns to the budget when a batch completes.

The scheduling loop runs on the host (one thread); no kernel waits on
another or on the host, so a stalled client can never hang the GPU.  Each
result is independent of what it was batched with (every output sample is
computed by one thread from its own source's data in a fixed order), which
``tests/test_gpu_serve.py`` checks bit for bit.

The scheduling logic talks to an *executor* (launch a batch, ask whether it
finished); :class:`GpuExecutor` drives the CUDA kernels, and the tests drive
the same loop with a fake executor on the CPU.
"""

from __future__ import annotations

import collections
import queue
import threading
import time
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

BYTES_PER_SAMPLE = 24  # three float64 channels (waveforms are generated in the kernel)


@dataclass
class Request:
    """One response + TDI evaluation.  ``params`` = (A, f, fdot, iota, phi0,
    psi, lam, beta); ``n`` samples; ``tdi_set`` indexes the server's TDI sets."""

    params: Sequence[float]
    n: int
    tdi_set: int = 0
    t0: float = 0.0
    t_submit: float = 0.0
    t_launch: float = 0.0
    t_done: float = 0.0
    result_value: object = None
    error: Optional[BaseException] = None
    _done: threading.Event = field(default_factory=threading.Event, repr=False)

    @property
    def footprint(self) -> int:
        return int(self.n) * BYTES_PER_SAMPLE

    @property
    def latency(self) -> float:
        return self.t_done - self.t_submit

    def done(self) -> bool:
        return self._done.is_set()

    def result(self, timeout: Optional[float] = None):
        """The (3, n) output channels (a CUDA tensor for the GPU executor)."""
        if not self._done.wait(timeout):
            raise TimeoutError("request not finished")
        if self.error is not None:
            raise self.error
        return self.result_value


def admit(waiting: "collections.deque", used: int, budget: int, max_batch_samples: int,
          max_batch_sources: int) -> List[Request]:
    """Take requests from the front of `waiting` (FIFO) while their memory fits
    the budget and the batch stays under its size limits.  A request larger
    than the whole budget is rejected by the server before it gets here."""
    batch: List[Request] = []
    samples = 0
    while waiting and len(batch) < max_batch_sources:
        r = waiting[0]
        if used + r.footprint > budget:
            break
        if batch and samples + r.n > max_batch_samples:
            break
        waiting.popleft()
        batch.append(r)
        used += r.footprint
        samples += r.n
    return batch


class GpuExecutor:
    """Runs batches with one BatchedResponseTDI plan and stream per lane."""

    def __init__(self, sampling_frequency, orbits, order, tdi_sets, tdi_chan, precision,
                 t_buffer, num_streams, device, use_graphs=True):
        import torch

        from .batch import BatchedResponseTDI

        self.torch = torch
        self.device = device
        self.plans = [BatchedResponseTDI(sampling_frequency, order=order, tdi=list(tdi_sets),
                                         orbits=orbits, tdi_chan=tdi_chan, precision=precision,
                                         t_buffer=t_buffer, force_backend=device)
                      for _ in range(num_streams)]
        self.streams = [torch.cuda.Stream(device=device) for _ in range(num_streams)]
        self.lanes = num_streams
        self.use_graphs = use_graphs

    def launch(self, lane: int, batch: List[Request]):
        torch = self.torch
        params = np.asarray([r.params[:6] for r in batch], dtype=np.float64)
        lam = [r.params[6] for r in batch]
        beta = [r.params[7] for r in batch]
        s = self.streams[lane]
        with torch.cuda.device(self.device), torch.cuda.stream(s):
            outs = [torch.empty((3, r.n), dtype=torch.float64, device=self.device)
                    for r in batch]
            # waveforms generated inside the fused kernel: only the channels
            # reach memory
            self.plans[lane].run_gb(params, [r.n for r in batch], lam, beta,
                                    t0=[r.t0 for r in batch], tdi_set=[r.tdi_set for r in batch],
                                    out=outs, stream=s, use_graph=self.use_graphs,
                                    keep_waveforms=False)
            ev = torch.cuda.Event()
            ev.record(s)
        return (ev, outs)

    def finished(self, handle) -> bool:
        return handle[0].query()

    def results(self, handle):
        return handle[1]


class ResponseServer:
    """Continuous-batching response + TDI service.

    Args:
        sampling_frequency: sample rate [Hz].
        orbits: orbit class or instance.
        order: Lagrange order.
        tdi_sets: TDI combinations requests can choose from (index = tdi_set).
        tdi_chan: "XYZ", "AET" or "AE".
        precision: "mixed" (default) or "fp64".
        memory_budget: bytes of HBM that admitted requests may hold.
        num_streams: concurrent batches on the device.
        max_batch_samples / max_batch_sources: batch size limits.  2^23
            samples (~12k tiles, ~10 ms of GPU work) still fill the GPU while
            bounding how long a small request waits behind a batch: at 0.8 of
            saturation p99 24 ms against 150 ms with 2^26, at 94 % instead of
            95 % of the batched throughput.
        executor: override (tests); default drives the GPU.
        keep_results: False drops each result once its request is done (only
            the timings stay; ``result()`` then returns None): for load
            tests whose clients do not read the channels.
    """

    def __init__(self, sampling_frequency, orbits=None, order=25,
                 tdi_sets=("1st generation", "2nd generation"), tdi_chan="XYZ",
                 precision="mixed", t_buffer=10000.0, memory_budget=160e9, num_streams=2,
                 max_batch_samples=2**23, max_batch_sources=512, force_backend=None,
                 executor=None, keep_results=True):
        self.tdi_start_ind = int(t_buffer * sampling_frequency)
        self.budget = int(memory_budget)
        self.max_batch_samples = int(max_batch_samples)
        self.max_batch_sources = int(max_batch_sources)
        self.num_sets = len(tdi_sets)
        if executor is None:
            from .orbits import EqualArmlengthOrbits
            from .response import _orbit_instance, _resolve_device

            device = _resolve_device(force_backend)
            executor = GpuExecutor(sampling_frequency, _orbit_instance(
                orbits if orbits is not None else EqualArmlengthOrbits), order, tdi_sets,
                tdi_chan, precision, t_buffer, num_streams, device)
        self.executor = executor
        self.keep_results = bool(keep_results)
        self._inbox: "queue.SimpleQueue[Request]" = queue.SimpleQueue()
        self._wake = threading.Event()
        self._stop = False
        self.completed: List[Request] = []
        self.used = 0
        self.peak_used = 0
        self.batches = 0
        self._thread = threading.Thread(target=self._loop, name="flr-serve", daemon=True)
        self._thread.start()

    # -- client side --------------------------------------------------------------
    def submit(self, params, n, tdi_set=0, t0=0.0) -> Request:
        """Queue one evaluation; returns its Request (``result()`` blocks)."""
        r = Request(params=tuple(float(x) for x in params), n=int(n), tdi_set=int(tdi_set),
                    t0=float(t0))
        if len(r.params) != 8:
            raise ValueError("params must be (A, f, fdot, iota, phi0, psi, lam, beta)")
        if not 0 <= r.tdi_set < self.num_sets:
            raise ValueError(f"tdi_set must be in [0, {self.num_sets})")
        if r.n <= 2 * self.tdi_start_ind:
            raise ValueError(f"n must exceed twice the garbage margin ({2 * self.tdi_start_ind})")
        if r.footprint > self.budget:
            raise ValueError("request larger than the whole memory budget")
        r.t_submit = time.perf_counter()
        self._inbox.put(r)
        self._wake.set()
        return r

    def close(self, timeout: Optional[float] = None) -> None:
        """Finish the queued work and stop the scheduling thread."""
        self._stop = True
        self._wake.set()
        self._thread.join(timeout)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- scheduling loop ------------------------------------------------------------
    def _loop(self) -> None:
        waiting: "collections.deque[Request]" = collections.deque()
        in_flight = {}  # lane -> (handle, batch)
        lanes = self.executor.lanes
        while True:
            while True:
                try:
                    waiting.append(self._inbox.get_nowait())
                except queue.Empty:
                    break
            now = time.perf_counter()
            for lane in list(in_flight):
                handle, batch = in_flight[lane]
                if self.executor.finished(handle):
                    outs = self.executor.results(handle)
                    done = time.perf_counter()
                    for r, o in zip(batch, outs):
                        r.result_value = o if self.keep_results else None
                        r.t_done = done
                        self.used -= r.footprint
                        self.completed.append(r)
                        r._done.set()
                    del in_flight[lane]
            free = [lane for lane in range(lanes) if lane not in in_flight]
            if free and waiting:
                batch = admit(waiting, self.used, self.budget, self.max_batch_samples,
                              self.max_batch_sources)
                if batch:
                    lane = free[0]
                    for r in batch:
                        r.t_launch = now
                    try:
                        handle = self.executor.launch(lane, batch)
                    except BaseException as e:  # the batch fails; the service goes on
                        done = time.perf_counter()
                        for r in batch:
                            r.error = e
                            r.t_done = done
                            r._done.set()
                    else:
                        self.used += sum(r.footprint for r in batch)
                        self.peak_used = max(self.peak_used, self.used)
                        self.batches += 1
                        in_flight[lane] = (handle, batch)
                    continue
            if self._stop and not waiting and not in_flight and self._inbox.empty():
                return
            if in_flight:
                time.sleep(20e-6)
            else:
                self._wake.wait(0.01)
                self._wake.clear()

    # -- reporting --------------------------------------------------------------------
    def stats(self) -> dict:
        done = [r for r in self.completed if r.error is None]
        if not done:
            return {"requests": 0}
        lat = np.asarray([r.latency for r in done])
        t_first = min(r.t_submit for r in done)
        t_last = max(r.t_done for r in done)
        samples = sum(r.n - 2 * self.tdi_start_ind for r in done)
        return {"requests": len(done), "batches": self.batches,
                "p50_ms": 1e3 * float(np.percentile(lat, 50)),
                "p99_ms": 1e3 * float(np.percentile(lat, 99)),
                "mean_ms": 1e3 * float(lat.mean()),
                "throughput_samples_per_s": samples / (t_last - t_first),
                "throughput_requests_per_s": len(done) / (t_last - t_first),
                "peak_memory_bytes": self.peak_used}
