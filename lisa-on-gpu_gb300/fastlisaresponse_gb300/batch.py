"""Many sources per launch: the batched, fused response + TDI.

``BatchedResponseTDI`` evaluates a list of sources -- each its own complex
waveform (any length), sky position and start time -- in one persistent
kernel launch over a flattened (source, tile) work list.  The six link streams
stay in on-chip memory; outputs are the TDI channels (XYZ, AET or AE), as
``pyResponseTDI.get_tdi_delays`` returns them.

``precision="fp64"`` reproduces the plain path bit for bit (and so the
reference's CPU arithmetic); ``precision="mixed"`` keeps the delay path in FP64
(integer indices bit-exact) and evaluates the Lagrange taps in double-float
arithmetic on the FP32 pipe, ~1e-9 relative to the FP64 result for typical
sources (see the tests for the bound that is checked).

There is no counterpart in the reference, which evaluates one source per
call (response.py:455-673).
"""

from __future__ import annotations

import collections
import ctypes
from typing import Optional, Sequence

import numpy as np

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None

from . import _lib
from .binding import OrbitsWrap
from .orbits import EqualArmlengthOrbits
from .response import (TDI_FIRST_GENERATION, TDI_SECOND_GENERATION_EXTRA, _as_device,
                       _orbit_instance, _resolve_device, lagrange_tables, sky_basis,
                       tdi_unit_tables)

C_inv = 3.3356409519815204e-09

PRECISION = {"fp64": 0, "mixed": 1}
CHANNELS = {"XYZ": 0, "AET": 1, "AE": 2}


class _TdiUnits(ctypes.Structure):
    _fields_ = [("num_units", ctypes.c_int),
                ("unit_starts", ctypes.c_void_p),
                ("unit_lengths", ctypes.c_void_p),
                ("tdi_base_link", ctypes.c_void_p),
                ("tdi_link_combinations", ctypes.c_void_p),
                ("tdi_signs", ctypes.c_void_p),
                ("channels", ctypes.c_void_p),
                ("num_combos", ctypes.c_int)]


class _GbParams(ctypes.Structure):
    _fields_ = [("A", ctypes.c_double), ("f", ctypes.c_double), ("fdot", ctypes.c_double),
                ("iota", ctypes.c_double), ("phi0", ctypes.c_double), ("psi", ctypes.c_double),
                ("model", ctypes.c_int), ("reserved", ctypes.c_int)]


# waveform models of the device generator (include/flr_gb300.h)
GB_MODELS = {"config": 0, "gbwave": 1}


class _Source(ctypes.Structure):
    _fields_ = [("h", ctypes.c_void_p),
                ("out", ctypes.c_void_p),
                ("n", ctypes.c_longlong),
                ("projections_start", ctypes.c_int),
                ("tdi_start", ctypes.c_int),
                ("t0", ctypes.c_double),
                ("k", ctypes.c_double * 3),
                ("u", ctypes.c_double * 3),
                ("v", ctypes.c_double * 3),
                ("tdi_set", ctypes.c_int),
                ("reserved", ctypes.c_int),
                ("y_out", ctypes.c_void_p),
                ("d_rec_out", ctypes.c_void_p),
                ("d_em_out", ctypes.c_void_p),
                ("d_tdi_out", ctypes.c_void_p),
                ("data", ctypes.c_void_p),
                ("inner", ctypes.c_void_p),
                ("out_begin", ctypes.c_longlong),
                ("out_end", ctypes.c_longlong)]


def _combinations(spec):
    if spec == "1st generation":
        return list(TDI_FIRST_GENERATION)
    if spec == "2nd generation":
        return list(TDI_FIRST_GENERATION) + list(TDI_SECOND_GENERATION_EXTRA)
    if isinstance(spec, list) and (not spec or isinstance(spec[0], dict)):
        return spec
    raise ValueError("tdi must be '1st generation', '2nd generation' or a list of "
                     "combination dicts (or a list of those for several sets)")


def _plan_fns():
    lib = _lib.lib()
    p, i, d = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    lib.flr_batch_plan_create.argtypes = [p, i, p, d, i, p, d, ctypes.POINTER(_TdiUnits), i, i,
                                          i, ctypes.POINTER(p)]
    lib.flr_batch_plan_create.restype = i
    lib.flr_batch_plan_destroy.argtypes = [p]
    lib.flr_batch_plan_destroy.restype = i
    lib.flr_batch_plan_info.argtypes = [p, ctypes.POINTER(ctypes.c_int), i]
    lib.flr_batch_plan_info.restype = i
    lib.flr_batch_run.argtypes = [p, ctypes.POINTER(_Source), i, i, p]
    lib.flr_batch_run.restype = i
    lib.flr_batch_run_gb.argtypes = [p, ctypes.POINTER(_Source), ctypes.POINTER(_GbParams), i, i,
                                     p]
    lib.flr_batch_run_gb.restype = i
    lib.flr_batch_graph_create.argtypes = [p, i, i, i, ctypes.POINTER(p)]
    lib.flr_batch_graph_create.restype = i
    lib.flr_batch_graph_launch.argtypes = [p, ctypes.POINTER(_Source), ctypes.POINTER(_GbParams),
                                           i, p]
    lib.flr_batch_graph_launch.restype = i
    lib.flr_batch_graph_destroy.argtypes = [p]
    lib.flr_batch_graph_destroy.restype = i
    lib.flr_batch_plan_set_wait_limit.argtypes = [p, ctypes.c_longlong]
    lib.flr_batch_plan_set_wait_limit.restype = i
    return lib


SOURCE_DTYPE = np.dtype(_Source)
GB_DTYPE = np.dtype(_GbParams)
GRAPH_WAVEFORMS = 0x1
GRAPH_DIAGNOSTICS = 0x2


def _contiguous_runs(tensors):
    """Runs of consecutive contiguous tensors that follow each other in one
    storage: (first index, end index, one flat tensor over the run), so that
    a run is copied with one cudaMemcpyAsync instead of one per tensor."""
    runs, k = [], 0
    while k < len(tensors):
        first = tensors[k]
        end = first.data_ptr() + first.numel() * first.element_size()
        base = first.untyped_storage().data_ptr()
        count, j = first.numel(), k + 1
        while j < len(tensors):
            x = tensors[j]
            if (x.data_ptr() != end or x.dtype != first.dtype
                    or x.untyped_storage().data_ptr() != base):
                break
            end += x.numel() * x.element_size()
            count += x.numel()
            j += 1
        span = first.reshape(-1) if j == k + 1 else \
            first.as_strided((count,), (1,), first.storage_offset())
        runs.append((k, j, span))
        k = j
    return runs


def _waveform_buffers(h, lengths, device, keep_waveforms):
    """Waveform buffers of a run with generated waveforms: the caller's, new
    ones, or (keep_waveforms False) None for each source: generated inside
    the fused kernel."""
    if not keep_waveforms:
        return [None] * len(lengths)
    hs = list(h) if h is not None else [
        torch.empty(n, dtype=torch.complex128, device=device) for n in lengths]
    for i, n in enumerate(lengths):
        if hs[i].numel() != n or hs[i].dtype != torch.complex128 or not hs[i].is_cuda:
            raise ValueError(f"h[{i}] must be a complex128 CUDA buffer of {n} samples")
    return hs


class BatchedResponseTDI:
    """Response + TDI of many sources per launch.

    Args:
        sampling_frequency: sample rate [Hz] shared by the batch.
        order: Lagrange order (default 25; up to 79).
        tdi: "1st generation", "2nd generation", a combination list, or a
            list of these (one TDI set each; sources pick one by index).
        orbits: orbit class or instance (default :class:`EqualArmlengthOrbits`).
        tdi_chan: "XYZ", "AET" or "AE".
        precision: "fp64" (bit-identical to the plain path) or "mixed".
        t_buffer: garbage time removed at each end [s] (as in get_projections).
        tile: output samples per work item (0 = library default, 512), or
            "auto": the fastest of the autotuner's candidates for this
            configuration, measured on first use and cached
            (:mod:`fastlisaresponse_gb300.autotune`).
        tune_lengths: source lengths of the batch the autotuner times
            (default 32 x 2^18).
    """

    def __init__(self, sampling_frequency, order=25, tdi="1st generation",
                 orbits=EqualArmlengthOrbits, tdi_chan="XYZ", precision="fp64",
                 t_buffer=10000.0, tile=0, force_backend=None, tune_lengths=None):
        if precision not in PRECISION:
            raise ValueError("precision must be 'fp64' or 'mixed'")
        if tdi_chan not in CHANNELS:
            raise ValueError("tdi_chan must be 'XYZ', 'AET' or 'AE'.")
        self.sampling_frequency = sampling_frequency
        self.dt = 1 / sampling_frequency
        self.order = order
        self.precision = precision
        self.tdi_chan = tdi_chan
        self.t_buffer = t_buffer
        self.device = _resolve_device(force_backend)
        orbits = _orbit_instance(orbits)
        if not getattr(orbits, "configured", True):
            orbits.configure(linear_interp_setup=True)
        self.orbits = orbits
        x_base = np.asarray(orbits.x_base, dtype=np.float64)
        max_sc = float((np.sum(x_base * x_base, axis=-1) ** (1 / 2)).max())
        self.tdi_start_ind = int(t_buffer / self.dt)
        check = int(100.0 * sampling_frequency) + 4 * order
        self.projections_start_ind = self.tdi_start_ind - 2 * check
        if self.projections_start_ind < int(max_sc * C_inv) + 4 * order:
            raise ValueError("Need to increase t_buffer. The initial buffer is not large enough.")

        specs = tdi if (isinstance(tdi, (list, tuple)) and tdi and
                        not isinstance(tdi[0], dict)) else [tdi]
        self.tdi_sets = [tdi_unit_tables(_combinations(s)) for s in specs]

        A, E, deps = lagrange_tables(order)
        self._A = torch.as_tensor(A, device=self.device)
        self._E = torch.as_tensor(E, device=self.device)
        self.deps = deps
        with torch.cuda.device(self.device):
            self.cpp_orbits = OrbitsWrap(*orbits.pycppdetector_args)
        units = (_TdiUnits * len(self.tdi_sets))()
        self._keep = []
        for i, tb in enumerate(self.tdi_sets):
            arrs = [np.ascontiguousarray(tb[k]) for k in ("unit_starts", "unit_lengths",
                                                           "tdi_base_links",
                                                           "tdi_link_combinations",
                                                           "tdi_signs", "channels")]
            self._keep.append(arrs)
            units[i] = _TdiUnits(tb["num_units"], *[a.ctypes.data for a in arrs],
                                 len(tb["tdi_link_combinations"]))
        self.tune = None
        if isinstance(tile, str):
            if tile != "auto":
                raise ValueError("tile must be an integer or 'auto'")
            from .autotune import best_tile

            self.tune = best_tile(sampling_frequency, order, tdi, orbits, precision, tdi_chan,
                                  t_buffer, self.device, lengths=tune_lengths)
            tile = self.tune["tile"]
        lib = _plan_fns()
        plan = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            rc = lib.flr_batch_plan_create(self.cpp_orbits.handle, order, self._A.data_ptr(),
                                           deps, len(A), self._E.data_ptr(), sampling_frequency,
                                           units, len(self.tdi_sets), PRECISION[precision],
                                           int(tile), ctypes.byref(plan))
        _lib.check(rc)
        self._plan = plan
        self._graphs = {}
        info = (ctypes.c_int * 12)()
        lib.flr_batch_plan_info(plan, info, 12)
        self.plan_info = dict(zip(("tile", "y_halo", "win_max", "y_max", "smem_bytes",
                                   "grid", "precision", "grouped", "fp32_tap_from",
                                   "tdi_second_differences", "threads", "staging_depth"),
                                  list(info)))
        if self.tune is not None:  # the knobs the plan runs with, tuned or fixed
            self.tune = dict(self.tune, threads=self.plan_info["threads"],
                             staging_depth=self.plan_info["staging_depth"])
        self._ctor = dict(sampling_frequency=sampling_frequency, order=order, tdi=tdi,
                          orbits=orbits, tdi_chan=tdi_chan, precision=precision,
                          t_buffer=t_buffer, force_backend=self.device)
        # input samples a tile's computation can read beyond its outputs: the
        # link-stream halo plus the largest delay either way (light travel
        # time and the spacecraft's distance from the Sun along k) and the taps
        lmax = float(np.abs(np.asarray(orbits.pycppdetector_args[3], dtype=np.float64)).max())
        self._reach = (self.plan_info["y_halo"]
                       + int(np.ceil((lmax + max_sc * C_inv) * sampling_frequency))
                       + (order + 1) // 2 + 16)

    def __del__(self):
        try:
            for g in getattr(self, "_graphs", {}).values():
                g.close()
            if getattr(self, "_plan", None) is not None:
                _lib.lib().flr_batch_plan_destroy(self._plan)
                self._plan = None
        except Exception:
            pass

    def __call__(self, h: Sequence, lam, beta, t0=0.0, tdi_set=0, out: Optional[Sequence] = None,
                 stream=None, diagnostics: bool = False, use_graph: bool = False,
                 chunks: int = 1, group_samples: Optional[int] = None):
        """Evaluate the batch.

        Args:
            h: sequence of complex waveforms h+ + i hx (torch/numpy/CAI), one
                per source; lengths may differ.
            lam, beta: ecliptic longitude / latitude per source (scalars
                broadcast).
            t0: start time per source (scalar broadcasts).
            tdi_set: TDI set index per source (scalar broadcasts).
            out: optional list of contiguous (3, n) float64 CUDA tensors to
                write into (every sample is written); allocated when omitted.
            diagnostics: also return, per source, the link streams and the
                integer delays the kernel used (for the output samples).
            use_graph: run through the CUDA graph of this batch's size bucket
                (captured on first use; see :meth:`graph`).
            chunks: split each source's outputs into this many tile-aligned
                launches alternating over two streams (and two plans), so that
                one launch's last wave overlaps the next one's start; the same
                bits as one launch.  For few, long sources.
            group_samples: with many sources, launches of about this many
                samples over runs of consecutive sources (longer sources are
                split into ``chunks`` pieces), alternating over the two
                streams as with ``chunks``; the same bits as one launch.
        Returns:
            list of (3, n) tensors: rows X, Y, Z (or A, E, T / A, E and a
            zero third row); samples within t_buffer of either end are zero.
            With diagnostics, (outs, diags) where diags[i] is a dict of
            "y" (6, n), "d_rec" / "d_em" (6, n) and "d_tdi" (units, n).
        """
        dev = self.device
        hs = [_as_device(x, dev, torch.complex128) for x in h]
        lengths = [len(x) for x in hs]
        if (chunks > 1 or group_samples) and not (diagnostics or use_graph):
            outs = list(out) if out is not None else [
                torch.empty((3, n), dtype=torch.float64, device=dev) for n in lengths]
            self._pipeline(hs, None, outs, None, lam, beta, t0, tdi_set, chunks, stream,
                           group_samples=group_samples)
            return outs
        return self._run(hs, None, lengths, lam, beta, t0, tdi_set, out, stream, diagnostics,
                         self._bucket(len(hs), False, diagnostics) if use_graph else None)

    def run_gb(self, params, lengths, lam, beta, t0=0.0, tdi_set=0, h=None, out=None,
               stream=None, use_graph: bool = False, model: str = "config",
               keep_waveforms: bool = True):
        """Generate galactic-binary waveforms on the device and evaluate them.

        Args:
            params: (num_sources, 6) array of (A, f, fdot, iota, phi0, psi).
            lengths: samples per source.
            lam, beta, t0, tdi_set: as for __call__ (scalars broadcast).
            h: optional list of complex128 CUDA buffers of the given lengths
                that receive the waveforms (allocated when omitted).
            out: optional list of (3, n) float64 CUDA tensors.
            use_graph: as for __call__.
            model: "config" (the configurations' binary, waveforms.gb_waveform)
                or "gbwave" (the reference test-suite's generator,
                waveforms.GBWave).
            keep_waveforms: False generates each waveform inside the fused
                kernel, straight into its staged input window, so the
                waveforms never reach memory (24 B of HBM per output sample:
                the channels); ``h`` is then ignored and None returned for it.
        Returns:
            (outs, hs): the TDI channels and the generated waveforms.
        """
        params = np.asarray(params, dtype=np.float64).reshape(-1, 6)
        ns = len(params)
        lengths = [int(n) for n in np.broadcast_to(np.asarray(lengths, dtype=np.int64), (ns,))]
        hs = _waveform_buffers(h, lengths, self.device, keep_waveforms)
        outs = self._run(hs, params, lengths, lam, beta, t0, tdi_set, out, stream, False,
                         self._bucket(ns, True, False) if use_graph else None, model=model)
        return outs, (hs if keep_waveforms else None)

    def inner_products(self, h: Sequence, lam, beta, data: Sequence, t0=0.0, tdi_set=0,
                       stream=None, write_out: bool = False):
        """Channel inner products of each source's response with data, formed
        inside the kernel: the channels need not be written to memory.

        Args:
            h, lam, beta, t0, tdi_set: as for __call__.
            data: per source a (3, n) float64 CUDA tensor in the layout of the
                output channels (X, Y, Z or A, E, T / A, E).
            write_out: also return the channels (else they are never stored).
        Returns:
            (ns, 2, 3) float64 tensor: [i, 0, c] = <h_c|d_c>, [i, 1, c] =
            <h_c|h_c>, sums over the computed samples [tdi_start, n - tdi_start)
            in a fixed order (run to run identical); with write_out, (inner,
            outs).  The white-noise log-likelihood follows as
            -0.5 sum_c (<d|d> - 2 <h|d> + <h|h>) / sigma_c^2.
        """
        dev = self.device
        hs = [_as_device(x, dev, torch.complex128) for x in h]
        lengths = [len(x) for x in hs]
        ds = self._check_data(data, lengths)
        inner = torch.empty((len(hs), 6), dtype=torch.float64, device=dev)
        outs = self._run(hs, None, lengths, lam, beta, t0, tdi_set, None, stream, False, None,
                         data=ds, inner=inner, write_out=write_out)
        inner = inner.view(len(hs), 2, 3)
        return (inner, outs) if write_out else inner

    def inner_products_gb(self, params, lengths, lam, beta, data: Sequence, t0=0.0, tdi_set=0,
                          h=None, stream=None, model: str = "config",
                          keep_waveforms: bool = True):
        """inner_products() of galactic binaries whose waveforms are generated
        on the device (run_gb's parameters, model and keep_waveforms); the
        channels are not stored.  Returns ((ns, 2, 3) inner products,
        waveforms or None)."""
        params = np.asarray(params, dtype=np.float64).reshape(-1, 6)
        ns = len(params)
        lengths = [int(n) for n in np.broadcast_to(np.asarray(lengths, dtype=np.int64), (ns,))]
        hs = _waveform_buffers(h, lengths, self.device, keep_waveforms)
        ds = self._check_data(data, lengths)
        inner = torch.empty((ns, 6), dtype=torch.float64, device=self.device)
        self._run(hs, params, lengths, lam, beta, t0, tdi_set, None, stream, False, None,
                  data=ds, inner=inner, write_out=False, model=model)
        return inner.view(ns, 2, 3), (hs if keep_waveforms else None)

    def run_host(self, h: Sequence, lam, beta, t0=0.0, tdi_set=0, out: Optional[Sequence] = None,
                 chunks: int = 4, group_samples: Optional[int] = None):
        """Evaluate sources whose waveforms are in host memory, overlapping the
        host-device copies with the computation.

        The work is cut into launches: with ``group_samples`` set, runs of
        consecutive sources shorter than it are launched together, about
        ``group_samples`` samples per launch; every other source's output
        range is split into ``chunks`` tile-aligned pieces.  A copy stream
        moves each launch's input (a chunk's with the halo its delays can
        reach), two compute streams with a plan each run the launches (one
        launch's tail overlaps the next one's start) and a second copy stream
        returns each launch's channels as soon as it is done.  A launch of
        whole sources takes one device buffer for its inputs and one for its
        channels, and sources adjacent in host memory (consecutive views of
        one HostArray) move with one copy per run each way.  Results are
        bit-identical to ``__call__`` on device copies of the inputs (sample i
        is at t0 + i dt in every chunk and group).

        Args:
            h: host complex128 waveforms (pinned or registered memory for
                asynchronous copies).
            lam, beta, t0, tdi_set: as for __call__.
            out: optional host (3, n) float64 tensors (pinned); allocated
                pinned when omitted.
            chunks: pieces per source launched alone.
            group_samples: samples per launch of grouped short sources
                (None: every source is launched alone, in ``chunks`` pieces).
        Returns:
            the list of host output tensors; the current CUDA stream is made to
            wait for them (synchronise it before reading them on the host).
        """
        ns = len(h)
        lam = np.broadcast_to(np.asarray(lam, dtype=np.float64), (ns,))
        beta = np.broadcast_to(np.asarray(beta, dtype=np.float64), (ns,))
        t0 = np.broadcast_to(np.asarray(t0, dtype=np.float64), (ns,))
        sets = np.broadcast_to(np.asarray(tdi_set, dtype=np.int64), (ns,))
        hh = [torch.as_tensor(x) for x in h]
        for i, x in enumerate(hh):
            if x.device.type != "cpu" or x.dtype != torch.complex128 or x.ndim != 1 \
                    or not x.is_contiguous():
                raise ValueError(f"h[{i}] must be a contiguous 1-D complex128 host array")
        outs = list(out) if out is not None else [
            torch.empty((3, len(x)), dtype=torch.float64, pin_memory=True) for x in hh]
        for i, (o, x) in enumerate(zip(outs, hh)):
            if (tuple(o.shape) != (3, len(x)) or o.dtype != torch.float64
                    or o.device.type != "cpu" or not o.is_contiguous()):
                raise ValueError(f"out[{i}] must be a contiguous (3, {len(x)}) float64 host tensor")
        self._pipeline(None, hh, None, outs, lam, beta, t0, sets, chunks, None,
                       group_samples=group_samples)
        return outs

    def run_time_shard(self, h, lam, beta, rank: int, world: int, t0=0.0, tdi_set=0,
                       stream=None):
        """One long source sharded by time over `world` ranks (one GPU each):
        this rank's tile-aligned share of the output samples
        (:func:`fastlisaresponse_gb300.dist.shard_time`), computed from the
        slice of the input its delays reach (:func:`dist.input_range`).

        Args:
            h: the whole complex128 waveform (host or device); only the
                rank's input slice is read and copied to this GPU (the rest of
                the device buffer holds NaN, so a read outside the slice would
                show in the output).
            lam, beta, t0, tdi_set: as for __call__ (one source).
            rank, world: this rank and the number of ranks.
        Returns:
            (out, out_range, in_range): a (3, n) float64 device tensor whose
            samples [out_range) are this rank's channels (the first rank's
            also the zeros before tdi_start, the last rank's those after
            n - tdi_start; other samples NaN), the output range (None: no
            tile for this rank) and the input slice read.  The ranks' output
            ranges partition the output, each sample computed as in a
            single run (the same bits).
        """
        from .dist import input_range, shard_time

        dev = self.device
        x = torch.as_tensor(h)
        if x.dtype != torch.complex128 or x.ndim != 1:
            raise ValueError("h must be a 1-D complex128 array")
        n = len(x)
        ts = self.tdi_start_ind
        out = torch.full((3, n), float("nan"), dtype=torch.float64, device=dev)
        rng = shard_time(n, ts, self.plan_info["tile"], rank, world)
        if rng is None:
            return out, None, None
        lo, hi = input_range(rng, n, self._reach)
        d_h = torch.full((n,), complex(float("nan"), float("nan")), dtype=torch.complex128,
                         device=dev)
        d_h[lo:hi].copy_(x[lo:hi], non_blocking=x.device.type == "cpu" and x.is_pinned())
        self._run([d_h], None, [n], lam, beta, t0, tdi_set, [out], stream, False, None,
                  out_range=rng)
        return out, rng, (lo, hi)

    def _launch_units(self, lengths, chunks, group_samples):
        """The launches of a pipelined run: lists of (source, output range or
        None = the whole source).  Consecutive sources shorter than
        group_samples share launches of about that many samples; the others
        are launched alone in `chunks` tile-aligned pieces."""
        tile, ts = self.plan_info["tile"], self.tdi_start_ind
        units, cur, cur_n = [], [], 0
        for i, n in enumerate(lengths):
            if group_samples is not None and n < group_samples:
                cur.append((i, None))
                cur_n += n
                if cur_n >= group_samples:
                    units.append(cur)
                    cur, cur_n = [], 0
                continue
            if cur:
                units.append(cur)
                cur, cur_n = [], 0
            tiles = -(-(n - 2 * ts) // tile)
            per = -(-tiles // max(1, min(int(chunks), tiles)))
            for a in range(0, tiles, per):
                units.append([(i, (ts + a * tile, min(ts + (a + per) * tile, n - ts)))])
        if cur:
            units.append(cur)
        return units

    def _pipeline(self, d_hs, host_hs, d_outs, host_outs, lam, beta, t0, tdi_set, chunks,
                  stream, group_samples=None):
        """Pipelined execution over two compute streams (see run_host): the
        launches of _launch_units alternate between this plan and its twin;
        with host inputs/outputs, a copy stream brings each launch's input
        (with the reach of a chunk's delays) and another returns its
        channels.  The calling stream waits for the result."""
        dev = self.device
        host = host_hs is not None
        ns = len(host_hs if host else d_hs)
        lam = np.broadcast_to(np.asarray(lam, dtype=np.float64), (ns,))
        beta = np.broadcast_to(np.asarray(beta, dtype=np.float64), (ns,))
        t0 = np.broadcast_to(np.asarray(t0, dtype=np.float64), (ns,))
        sets = np.broadcast_to(np.asarray(tdi_set, dtype=np.int64), (ns,))
        plans = [self, self._twin()]
        cur = stream if stream is not None else torch.cuda.current_stream(dev)
        if not hasattr(self, "_side_streams"):
            self._side_streams = [torch.cuda.Stream(device=dev) for _ in range(4)]
        s_in, s_k0, s_k1, s_out = self._side_streams
        s_comp = [s_k0, s_k1]
        start = torch.cuda.Event()
        start.record(cur)
        for s_ in self._side_streams:
            s_.wait_event(start)
        lengths = [len(x) for x in (host_hs if host else d_hs)]
        if not host:
            for i, (d_o, n) in enumerate(zip(d_outs, lengths)):
                if (tuple(d_o.shape) != (3, n) or d_o.dtype != torch.float64 or not d_o.is_cuda
                        or not d_o.is_contiguous()):
                    raise ValueError(f"out[{i}] must be a contiguous (3, {n}) float64 CUDA tensor")
        reach = self._reach
        d_h, d_o, done_in = {}, {}, {}
        in_flight = collections.deque()  # completion events of the launches' returns
        units = self._launch_units(lengths, chunks, group_samples)
        # launches of whole sources take their device buffers from a ring of
        # four slots, allocated once on the calling stream (every side stream's
        # work is joined back into it before they are freed): at most three
        # launches are in flight, so a slot's previous launch has completed
        # when it is reused, and the loop makes no allocation (an allocation
        # that cannot reuse a cached block calls cudaMalloc, which waits for
        # the whole device)
        whole = [all(r is None for _, r in u) for u in units]
        ring_n = max([sum(lengths[i] for i, _ in u) for u, w in zip(units, whole) if w],
                     default=0)
        if host and ring_n:
            with torch.cuda.stream(cur):
                ring_h = [torch.empty(ring_n, dtype=torch.complex128, device=dev)
                          for _ in range(4)]
                ring_o = [torch.empty(3 * ring_n, dtype=torch.float64, device=dev)
                          for _ in range(4)]
        for k, unit in enumerate(units):
            comp = s_comp[k % 2]
            idx = [i for i, _ in unit]
            if host and whole[k]:
                # whole sources: one slot for the launch's inputs and one for its
                # channels, one copy per run of sources adjacent in host memory
                # (e.g. views of one HostArray) each way
                ns_u = [lengths[i] for i in idx]
                offs = np.concatenate([[0], np.cumsum(ns_u)]).astype(np.int64)
                buf_h = ring_h[k % 4][:int(offs[-1])]
                buf_o = ring_o[k % 4][:3 * int(offs[-1])]
                hs_u = [buf_h[offs[j]:offs[j + 1]] for j in range(len(idx))]
                outs_u = [buf_o[3 * offs[j]:3 * offs[j + 1]].view(3, ns_u[j])
                          for j in range(len(idx))]
                ev_in = torch.cuda.Event()
                with torch.cuda.stream(s_in):
                    for a, b, span in _contiguous_runs([host_hs[i] for i in idx]):
                        buf_h[offs[a]:offs[b]].copy_(span, non_blocking=True)
                    ev_in.record(s_in)
                comp.wait_event(ev_in)
                plans[k % 2]._run(hs_u, None, ns_u, lam[idx], beta[idx], t0[idx], sets[idx],
                                  outs_u, comp, False, None)
                ev_k = torch.cuda.Event()
                ev_k.record(comp)
                s_out.wait_event(ev_k)
                with torch.cuda.stream(s_out):
                    for a, b, span in _contiguous_runs([host_outs[i] for i in idx]):
                        span.copy_(buf_o[3 * offs[a]:3 * offs[b]], non_blocking=True)
                    ev_back = torch.cuda.Event()
                    ev_back.record(s_out)
                del buf_h, buf_o, hs_u, outs_u
                in_flight.append(ev_back)
                if len(in_flight) > 3:
                    in_flight.popleft().synchronize()
                continue
            if host:
                ev_in = torch.cuda.Event()
                with torch.cuda.stream(s_in):
                    for i, rng in unit:
                        n = lengths[i]
                        if i not in d_h:  # device buffers of a source, made when first needed
                            d_h[i] = torch.empty(n, dtype=torch.complex128, device=dev)
                            d_o[i] = torch.empty((3, n), dtype=torch.float64, device=dev)
                            for s_ in self._side_streams:
                                d_h[i].record_stream(s_)
                                d_o[i].record_stream(s_)
                            done_in[i] = 0
                        last = rng is None or rng[1] == n - self.tdi_start_ind
                        need = n if last else min(n, rng[1] + reach)
                        if need > done_in[i]:
                            d_h[i][done_in[i]:need].copy_(host_hs[i][done_in[i]:need],
                                                          non_blocking=True)
                            done_in[i] = need
                    ev_in.record(s_in)
                comp.wait_event(ev_in)
                hs_u, outs_u = [d_h[i] for i in idx], [d_o[i] for i in idx]
            else:
                hs_u, outs_u = [d_hs[i] for i in idx], [d_outs[i] for i in idx]
            rng = unit[0][1] if len(unit) == 1 else None
            plans[k % 2]._run(hs_u, None, [lengths[i] for i in idx], lam[idx], beta[idx], t0[idx],
                              sets[idx], outs_u, comp, False, None, out_range=rng)
            if host:
                ev_k = torch.cuda.Event()
                ev_k.record(comp)
                s_out.wait_event(ev_k)
                with torch.cuda.stream(s_out):
                    for i, r in unit:
                        n = lengths[i]
                        if r is None:
                            host_outs[i].copy_(d_o[i], non_blocking=True)
                            continue
                        lo = 0 if r[0] == self.tdi_start_ind else r[0]
                        hi = n if r[1] == n - self.tdi_start_ind else r[1]
                        for c in range(3):
                            host_outs[i][c, lo:hi].copy_(d_o[i][c, lo:hi], non_blocking=True)
                    ev_back = torch.cuda.Event()
                    ev_back.record(s_out)
                # a source's device buffers go back to the allocator once its last
                # output is on its way (reused after the copy, by record_stream);
                # at most three launches' buffers are held at a time
                for i, r in unit:
                    if r is None or r[1] == lengths[i] - self.tdi_start_ind:
                        del d_h[i], d_o[i]
                in_flight.append(ev_back)
                if len(in_flight) > 3:
                    in_flight.popleft().synchronize()
        for s_ in (s_out,) if host else tuple(s_comp):
            end = torch.cuda.Event()
            end.record(s_)
            cur.wait_event(end)

    def _twin(self) -> "BatchedResponseTDI":
        """A second plan with this one's configuration (own staging buffers),
        for a second compute stream."""
        if getattr(self, "_twin_plan", None) is None:
            kw = dict(self._ctor)
            kw["tile"] = self.plan_info["tile"]
            self._twin_plan = BatchedResponseTDI(**kw)
        return self._twin_plan

    def _check_data(self, data, lengths):
        ds = list(data)
        if len(ds) != len(lengths):
            raise ValueError("need one data array per source")
        for i, (x, n) in enumerate(zip(ds, lengths)):
            if (not isinstance(x, torch.Tensor) or tuple(x.shape) != (3, n)
                    or x.dtype != torch.float64 or not x.is_cuda or not x.is_contiguous()
                    or x.device != self.device):
                raise ValueError(f"data[{i}] must be a contiguous (3, {n}) float64 tensor on "
                                 f"{self.device}")
        return ds

    # -- internals ----------------------------------------------------------------
    def _run(self, hs, params, lengths, lam, beta, t0, tdi_set, out, stream, diagnostics, graph,
             data=None, inner=None, write_out=True, out_range=None, model="config"):
        ns = len(hs)
        dev = self.device
        lam = np.broadcast_to(np.asarray(lam, dtype=np.float64), (ns,))
        beta = np.broadcast_to(np.asarray(beta, dtype=np.float64), (ns,))
        t0 = np.broadcast_to(np.asarray(t0, dtype=np.float64), (ns,))
        sets = np.broadcast_to(np.asarray(tdi_set, dtype=np.int64), (ns,))
        if out is not None:
            outs = list(out)
            if len(outs) != ns:
                raise ValueError("need one output per source")
            for i, o in enumerate(outs):
                n = lengths[i]
                if (tuple(o.shape) != (3, n) or o.dtype != torch.float64 or not o.is_cuda
                        or not o.is_contiguous()):
                    raise ValueError(f"out[{i}] must be a contiguous (3, {n}) float64 CUDA tensor")
        elif write_out:
            outs = [torch.empty((3, n), dtype=torch.float64, device=dev) for n in lengths]
        else:
            outs = None
        srcs = np.zeros(ns, dtype=SOURCE_DTYPE)
        srcs["h"] = [0 if x is None else x.data_ptr() for x in hs]
        if outs is not None:
            srcs["out"] = [o.data_ptr() for o in outs]
        if out_range is not None:
            srcs["out_begin"], srcs["out_end"] = out_range
        if data is not None:
            srcs["data"] = [x.data_ptr() for x in data]
            srcs["inner"] = [inner.data_ptr() + 48 * i for i in range(ns)]
        srcs["n"] = lengths
        srcs["projections_start"] = self.projections_start_ind
        srcs["tdi_start"] = self.tdi_start_ind
        srcs["t0"] = t0
        srcs["tdi_set"] = sets
        for i in range(ns):
            srcs["k"][i], srcs["u"][i], srcs["v"][i] = sky_basis(float(lam[i]), float(beta[i]))
        diags = []
        if diagnostics:
            for i in range(ns):
                n, nu = lengths[i], self.tdi_sets[int(sets[i])]["num_units"]
                dg = {"y": torch.zeros((6, n), dtype=torch.float64, device=dev),
                      "d_rec": torch.zeros((6, n), dtype=torch.int32, device=dev),
                      "d_em": torch.zeros((6, n), dtype=torch.int32, device=dev),
                      "d_tdi": torch.zeros((nu, n), dtype=torch.int32, device=dev)}
                diags.append(dg)
                srcs["y_out"][i] = dg["y"].data_ptr()
                srcs["d_rec_out"][i] = dg["d_rec"].data_ptr()
                srcs["d_em_out"][i] = dg["d_em"].data_ptr()
                srcs["d_tdi_out"][i] = dg["d_tdi"].data_ptr()
        gbs = None
        if params is not None:
            prm = np.ascontiguousarray(params, dtype=np.float64).reshape(ns, 6)
            gbs = np.zeros(ns, dtype=GB_DTYPE)
            for k, name in enumerate(("A", "f", "fdot", "iota", "phi0", "psi")):
                gbs[name] = prm[:, k]
            if model not in GB_MODELS:
                raise ValueError(f"model must be one of {sorted(GB_MODELS)}")
            gbs["model"] = GB_MODELS[model]
        if stream is None:
            stream = torch.cuda.current_stream(dev)
        lib = _plan_fns()
        src_p = srcs.ctypes.data_as(ctypes.POINTER(_Source))
        gb_p = gbs.ctypes.data_as(ctypes.POINTER(_GbParams)) if gbs is not None else None
        st = ctypes.c_void_p(stream.cuda_stream)
        with torch.cuda.device(dev), _lib.nvtx_range(f"flr.batch[{ns}]"):
            if graph is not None:
                rc = lib.flr_batch_graph_launch(graph._graph, src_p, gb_p, ns, st)
            elif gbs is not None:
                rc = lib.flr_batch_run_gb(self._plan, src_p, gb_p, ns, CHANNELS[self.tdi_chan], st)
            else:
                rc = lib.flr_batch_run(self._plan, src_p, ns, CHANNELS[self.tdi_chan], st)
        _lib.check(rc)
        self._last_inputs = (hs, data)  # keep the inputs alive until the next call
        return (outs, diags) if diagnostics else outs

    def _bucket(self, ns: int, waveforms: bool, diagnostics: bool) -> "BatchGraph":
        cap = max(8, 1 << max(0, int(ns) - 1).bit_length())
        key = (cap, waveforms, diagnostics)
        g = self._graphs.get(key)
        if g is None:
            g = self._graphs[key] = self.graph(cap, waveforms=waveforms, diagnostics=diagnostics)
        return g

    def graph(self, max_sources: int, waveforms: bool = False,
              diagnostics: bool = False) -> "BatchGraph":
        """A CUDA graph of this plan's staging copy and kernel launch(es) for
        up to ``max_sources`` sources of any lengths (flr_batch_graph_create).
        ``waveforms``: the graph also generates galactic-binary waveforms
        (use its :meth:`BatchGraph.run_gb`)."""
        return BatchGraph(self, max_sources, waveforms, diagnostics)

    def status(self, reset: bool = False) -> int:
        """Kernel status bits (see include/flr_gb300.h; 0x10 = a work item's
        staging copy completed late and its outputs are NaN, 0x20 = a copy
        never completed and the batch's outputs are to be discarded);
        synchronises."""
        return self.cpp_orbits.status(reset=reset)

    def _set_wait_limit(self, polls: int) -> None:
        """Test hook: bound of each work item's first wait for its staging
        copy in later runs (< 0: the default); see
        flr_batch_plan_set_wait_limit."""
        _lib.check(_plan_fns().flr_batch_plan_set_wait_limit(self._plan, int(polls)))


class BatchGraph:
    """A captured batch launch of a :class:`BatchedResponseTDI` plan for up to
    ``max_sources`` sources of any lengths.  Calls take the same arguments as
    the plan's ``__call__`` / ``run_gb`` and give bit-identical results; each
    replays the graph after staging the sources (two staging buffers
    alternate, so a call can be prepared while the previous one runs)."""

    def __init__(self, owner: BatchedResponseTDI, max_sources: int, waveforms: bool,
                 diagnostics: bool):
        self.owner = owner
        self.max_sources = int(max_sources)
        self.waveforms = bool(waveforms)
        self.diagnostics = bool(diagnostics)
        flags = (GRAPH_WAVEFORMS if waveforms else 0) | (GRAPH_DIAGNOSTICS if diagnostics else 0)
        lib = _plan_fns()
        g = ctypes.c_void_p()
        with torch.cuda.device(owner.device):
            rc = lib.flr_batch_graph_create(owner._plan, self.max_sources, flags,
                                            CHANNELS[owner.tdi_chan], ctypes.byref(g))
        _lib.check(rc)
        self._graph = g

    def __call__(self, h: Sequence, lam, beta, t0=0.0, tdi_set=0, out=None, stream=None,
                 diagnostics: bool = False):
        if self.waveforms:
            raise ValueError("this graph generates waveforms: use run_gb")
        o = self.owner
        hs = [_as_device(x, o.device, torch.complex128) for x in h]
        self._check(len(hs))
        return o._run(hs, None, [len(x) for x in hs], lam, beta, t0, tdi_set, out, stream,
                      diagnostics, self)

    def run_gb(self, params, lengths, lam, beta, t0=0.0, tdi_set=0, h=None, out=None,
               stream=None, model: str = "config", keep_waveforms: bool = True):
        if not self.waveforms:
            raise ValueError("this graph was created without waveforms")
        o = self.owner
        params = np.asarray(params, dtype=np.float64).reshape(-1, 6)
        ns = len(params)
        self._check(ns)
        lengths = [int(n) for n in np.broadcast_to(np.asarray(lengths, dtype=np.int64), (ns,))]
        hs = _waveform_buffers(h, lengths, o.device, keep_waveforms)
        outs = o._run(hs, params, lengths, lam, beta, t0, tdi_set, out, stream, False, self,
                      model=model)
        return outs, (hs if keep_waveforms else None)

    def _check(self, ns):
        if ns > self.max_sources:
            raise ValueError(f"{ns} sources: this graph takes at most {self.max_sources}")

    def close(self):
        if getattr(self, "_graph", None) is not None:
            _lib.lib().flr_batch_graph_destroy(self._graph)
            self._graph = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
