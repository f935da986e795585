"""Device-resident serving: requests appended to a source list that a
persistent launch of the fused kernel works through as they arrive.

:class:`DeviceLoopServer` keeps the orbit, Lagrange and TDI tables of one
mixed-precision plan on the GPU, and a list of up to ``capacity`` sources in
page-locked host memory mapped into the device (``flr_server_*`` in
``include/flr_gb300.h``).  ``submit`` writes a request's descriptor and
galactic-binary parameters there and publishes its tiles; the running kernel
(one CTA per resident slot, the plan's persistent grid) claims published
tiles with an atomic counter, generates each tile's waveform window in
shared memory, and the CTA that writes a request's last tile sets the
request's done flag in host memory.  So a request submitted while others are
on the GPU needs no launch, no copy and no host synchronisation: it is
admitted the moment its tiles are published and runs as soon as a CTA is
free.  The kernel leaves after ``idle_seconds`` without work (every wait is
bounded); ``submit`` and ``result`` relaunch it when requests are pending and
none is running.

Results are bit-identical to ``BatchedResponseTDI.run_gb(...,
keep_waveforms=False)`` on the same requests (the same kernel code computes
every tile).  The request loop of :class:`serve.ResponseServer` (host-side
batching into graph launches) is the alternative for callers that want
admission against a memory budget; this one trades that for launch-free
admission.
"""

from __future__ import annotations

import ctypes
import time
from typing import Optional, Sequence

import numpy as np

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None

from . import _lib
from .batch import CHANNELS, GB_DTYPE, GB_MODELS, SOURCE_DTYPE, BatchedResponseTDI
from .response import sky_basis


def _server_fns():
    lib = _lib.lib()
    p, i, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    lib.flr_server_create.argtypes = [p, i, i, d, ctypes.POINTER(p)]
    lib.flr_server_create.restype = i
    lib.flr_server_submit.argtypes = [p, p, p, ctypes.POINTER(i)]
    lib.flr_server_submit.restype = i
    lib.flr_server_pump.argtypes = [p, p]
    lib.flr_server_pump.restype = i
    lib.flr_server_info.argtypes = [p, ctypes.POINTER(ctypes.c_longlong), i]
    lib.flr_server_info.restype = i
    lib.flr_server_done_flags.argtypes = [p]
    lib.flr_server_done_flags.restype = p
    lib.flr_server_stop.argtypes = [p]
    lib.flr_server_stop.restype = i
    lib.flr_server_destroy.argtypes = [p]
    lib.flr_server_destroy.restype = i
    return lib


class DeviceTicket:
    """A submitted request: ``done()``, ``result(timeout)`` (the (3, n)
    channels, a CUDA tensor), ``latency`` once done (seconds from submit to
    the first ``done()`` that saw it finished)."""

    def __init__(self, server: "DeviceLoopServer", slot: int, out):
        self._server = server
        self.slot = slot
        self.out = out
        self.t_submit = time.perf_counter()
        self.t_done = None

    def done(self) -> bool:
        if self.t_done is None and self._server._is_done(self.slot):
            self.t_done = time.perf_counter()
        return self.t_done is not None

    @property
    def latency(self) -> Optional[float]:
        return None if self.t_done is None else self.t_done - self.t_submit

    def result(self, timeout: Optional[float] = None):
        end = None if timeout is None else time.perf_counter() + timeout
        while not self.done():
            self._server.pump()
            if end is not None and time.perf_counter() > end:
                raise TimeoutError(f"request {self.slot} not finished")
            time.sleep(2e-5)
        return self.out


class DeviceLoopServer:
    """Device-resident continuous serving of galactic-binary requests.

    Args:
        sampling_frequency: sample rate [Hz].
        orbits: orbit class or instance (default equal-arm).
        order: Lagrange order.
        tdi_sets: TDI combinations requests can choose from (index = tdi_set).
        tdi_chan: "XYZ", "AET" or "AE".
        t_buffer: garbage time at each end [s].
        capacity: requests per server (its source list does not wrap).
        idle_seconds: the kernel leaves after this long without work.
        tile: output samples per work item (0: the library default).
        force_backend: device.
    """

    def __init__(self, sampling_frequency, orbits=None, order: int = 25,
                 tdi_sets: Sequence = ("1st generation", "2nd generation"),
                 tdi_chan: str = "XYZ", t_buffer: float = 10000.0, capacity: int = 65536,
                 idle_seconds: float = 0.02, tile: int = 0, force_backend=None):
        self.plan = BatchedResponseTDI(sampling_frequency, order=order, tdi=list(tdi_sets),
                                       orbits=orbits, tdi_chan=tdi_chan, precision="mixed",
                                       t_buffer=t_buffer, tile=tile,
                                       force_backend=force_backend)
        self.device = self.plan.device
        self.capacity = int(capacity)
        lib = _server_fns()
        self._lib = lib
        srv = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(lib.flr_server_create(self.plan._plan, self.capacity, CHANNELS[tdi_chan],
                                             float(idle_seconds), ctypes.byref(srv)))
        self._srv = srv
        flags = lib.flr_server_done_flags(srv)
        self._done = np.frombuffer((ctypes.c_uint32 * self.capacity).from_address(flags),
                                   dtype=np.uint32)
        self.stream = torch.cuda.Stream(device=self.device)
        self._pending = {}  # slot -> (output, stored waveform), kept alive until written

    # -- requests --------------------------------------------------------------
    def submit(self, params, n: int, tdi_set: int = 0, t0: float = 0.0, model: str = "config",
               out=None, h=None) -> DeviceTicket:
        """Submit one request: ``params`` = (A, f, fdot, iota, phi0, psi, lam,
        beta), ``n`` samples from ``t0``; the waveform is generated inside the
        kernel from the first six.  With ``h`` (a contiguous complex128 CUDA
        tensor of n samples on this device, kept alive until the request is
        done) the stored waveform is used instead and only lam, beta are read
        from ``params``.  ``out`` (optional) receives the (3, n) float64
        channels on this server's device.  The running kernel reads ``h`` and
        writes ``out`` as soon as the request is published, outside any
        stream order, so when either is given ``submit`` first waits for the
        work queued on the current stream (which may still write ``h`` or
        read ``out``)."""
        n = int(n)
        if h is not None and (tuple(h.shape) != (n,) or h.dtype != torch.complex128
                              or not h.is_cuda or not h.is_contiguous()):
            raise ValueError(f"h must be a contiguous ({n},) complex128 CUDA tensor")
        caller_out = out is not None
        if out is None:
            with torch.cuda.device(self.device), torch.cuda.stream(self.stream):
                out = torch.empty((3, n), dtype=torch.float64, device=self.device)
        elif (tuple(out.shape) != (3, n) or out.dtype != torch.float64 or not out.is_cuda
              or not out.is_contiguous()):
            raise ValueError(f"out must be a contiguous (3, {n}) float64 CUDA tensor")
        src = np.zeros(1, dtype=SOURCE_DTYPE)
        src["h"] = 0 if h is None else h.data_ptr()
        src["out"] = out.data_ptr()
        src["n"] = n
        src["projections_start"] = self.plan.projections_start_ind
        src["tdi_start"] = self.plan.tdi_start_ind
        src["t0"] = float(t0)
        src["k"][0], src["u"][0], src["v"][0] = sky_basis(float(params[6]), float(params[7]))
        src["tdi_set"] = int(tdi_set)
        if h is not None or caller_out:
            ev = torch.cuda.Event()
            ev.record(torch.cuda.current_stream(self.device))
            ev.synchronize()
        gb_ptr = None
        if h is None:
            gb = np.zeros(1, dtype=GB_DTYPE)
            for j, key in enumerate(("A", "f", "fdot", "iota", "phi0", "psi")):
                gb[key] = float(params[j])
            gb["model"] = GB_MODELS[model]
            gb_ptr = gb.ctypes.data
        slot = ctypes.c_int()
        with torch.cuda.device(self.device):
            _lib.check(self._lib.flr_server_submit(self._srv, src.ctypes.data, gb_ptr,
                                                   ctypes.byref(slot)))
        self._pending[slot.value] = (out, h)
        self.pump()
        return DeviceTicket(self, slot.value, out)

    def pump(self) -> None:
        """Launch the serving kernel if requests are pending and none runs."""
        with torch.cuda.device(self.device):
            _lib.check(self._lib.flr_server_pump(self._srv, self.stream.cuda_stream))

    def _is_done(self, slot: int) -> bool:
        if self._done[slot] == 0:
            return False
        self._pending.pop(slot, None)
        return True

    def info(self) -> dict:
        buf = (ctypes.c_longlong * 5)()
        _lib.check(self._lib.flr_server_info(self._srv, buf, 5))
        return dict(zip(("submitted", "tiles", "first_open", "launches", "running"),
                        list(buf)))

    def status(self, reset: bool = False) -> int:
        """The plan's sticky kernel status bits (0 = no problem)."""
        return self.plan.status(reset)

    def close(self) -> None:
        """Let the kernel finish what is published, then release the server."""
        if getattr(self, "_srv", None) is not None:
            self._lib.flr_server_stop(self._srv)
            self._lib.flr_server_destroy(self._srv)
            self._srv = None
            self._done = None
            self._pending.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
