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
                ("iota", ctypes.c_double), ("phi0", ctypes.c_double), ("psi", ctypes.c_double)]


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
                ("d_tdi_out", ctypes.c_void_p)]


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
    return lib


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
        tile: output samples per work item (0 = library default).
    """

    def __init__(self, sampling_frequency, order=25, tdi="1st generation",
                 orbits=EqualArmlengthOrbits, tdi_chan="XYZ", precision="fp64",
                 t_buffer=10000.0, tile=0, force_backend=None):
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
        lib = _plan_fns()
        plan = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            rc = lib.flr_batch_plan_create(self.cpp_orbits.handle, order, self._A.data_ptr(),
                                           deps, len(A), self._E.data_ptr(), sampling_frequency,
                                           units, len(self.tdi_sets), PRECISION[precision],
                                           int(tile), ctypes.byref(plan))
        _lib.check(rc)
        self._plan = plan
        info = (ctypes.c_int * 7)()
        lib.flr_batch_plan_info(plan, info, 7)
        self.plan_info = dict(zip(("tile", "y_halo", "win_max", "y_max", "smem_bytes",
                                   "grid", "precision"), list(info)))

    def __del__(self):
        try:
            if getattr(self, "_plan", None) is not None:
                _lib.lib().flr_batch_plan_destroy(self._plan)
                self._plan = None
        except Exception:
            pass

    def __call__(self, h: Sequence, lam, beta, t0=0.0, tdi_set=0, out: Optional[Sequence] = None,
                 stream=None, diagnostics: bool = False):
        """Evaluate the batch.

        Args:
            h: sequence of complex waveforms h+ + i hx (torch/numpy/CAI), one
                per source; lengths may differ.
            lam, beta: ecliptic longitude / latitude per source (scalars
                broadcast).
            t0: start time per source (scalar broadcasts).
            tdi_set: TDI set index per source (scalar broadcasts).
            out: optional list of (3, n) float64 CUDA tensors to write into
                (zeroed by the caller); allocated (zeros) when omitted.
            diagnostics: also return, per source, the link streams and the
                integer delays the kernel used (for the output samples).
        Returns:
            list of (3, n) tensors: rows X, Y, Z (or A, E, T / A, E and a
            zero third row); samples within t_buffer of either end are zero.
            With diagnostics, (outs, diags) where diags[i] is a dict of
            "y" (6, n), "d_rec" / "d_em" (6, n) and "d_tdi" (units, n).
        """
        ns = len(h)
        lam = np.broadcast_to(np.asarray(lam, dtype=np.float64), (ns,))
        beta = np.broadcast_to(np.asarray(beta, dtype=np.float64), (ns,))
        t0 = np.broadcast_to(np.asarray(t0, dtype=np.float64), (ns,))
        sets = np.broadcast_to(np.asarray(tdi_set, dtype=np.int64), (ns,))
        dev = self.device
        hs = [_as_device(x, dev, torch.complex128) for x in h]
        outs = list(out) if out is not None else [
            torch.zeros((3, len(x)), dtype=torch.float64, device=dev) for x in hs]
        srcs = (_Source * ns)()
        diags = []
        for i in range(ns):
            n = len(hs[i])
            o = outs[i]
            if tuple(o.shape) != (3, n) or o.dtype != torch.float64 or not o.is_contiguous():
                raise ValueError(f"out[{i}] must be a contiguous (3, {n}) float64 tensor")
            k, u, v = sky_basis(float(lam[i]), float(beta[i]))
            ptrs = [None] * 4
            if diagnostics:
                nu = self.tdi_sets[int(sets[i])]["num_units"]
                dg = {"y": torch.zeros((6, n), dtype=torch.float64, device=dev),
                      "d_rec": torch.zeros((6, n), dtype=torch.int32, device=dev),
                      "d_em": torch.zeros((6, n), dtype=torch.int32, device=dev),
                      "d_tdi": torch.zeros((nu, n), dtype=torch.int32, device=dev)}
                diags.append(dg)
                ptrs = [dg["y"].data_ptr(), dg["d_rec"].data_ptr(), dg["d_em"].data_ptr(),
                        dg["d_tdi"].data_ptr()]
            srcs[i] = _Source(hs[i].data_ptr(), o.data_ptr(), n, self.projections_start_ind,
                              self.tdi_start_ind, float(t0[i]), (ctypes.c_double * 3)(*k),
                              (ctypes.c_double * 3)(*u), (ctypes.c_double * 3)(*v),
                              int(sets[i]), 0, *ptrs)
        if stream is None:
            stream = torch.cuda.current_stream(dev)
        lib = _plan_fns()
        with torch.cuda.device(dev):
            rc = lib.flr_batch_run(self._plan, srcs, ns, CHANNELS[self.tdi_chan],
                                   ctypes.c_void_p(stream.cuda_stream))
        _lib.check(rc)
        self._last_inputs = hs  # keep the inputs alive until the next call
        return (outs, diags) if diagnostics else outs

    def run_gb(self, params, lengths, lam, beta, t0=0.0, tdi_set=0, h=None, out=None,
               stream=None):
        """Generate galactic-binary waveforms on the device and evaluate them.

        Args:
            params: (num_sources, 6) array of (A, f, fdot, iota, phi0, psi).
            lengths: samples per source.
            lam, beta, t0, tdi_set: as for __call__ (scalars broadcast).
            h: optional list of complex128 CUDA buffers of the given lengths
                that receive the waveforms (allocated when omitted).
            out: optional list of zeroed (3, n) float64 CUDA tensors.
        Returns:
            (outs, hs): the TDI channels and the generated waveforms.
        """
        params = np.asarray(params, dtype=np.float64).reshape(-1, 6)
        ns = len(params)
        lengths = np.broadcast_to(np.asarray(lengths, dtype=np.int64), (ns,))
        lam = np.broadcast_to(np.asarray(lam, dtype=np.float64), (ns,))
        beta = np.broadcast_to(np.asarray(beta, dtype=np.float64), (ns,))
        t0 = np.broadcast_to(np.asarray(t0, dtype=np.float64), (ns,))
        sets = np.broadcast_to(np.asarray(tdi_set, dtype=np.int64), (ns,))
        dev = self.device
        hs = list(h) if h is not None else [
            torch.empty(int(n), dtype=torch.complex128, device=dev) for n in lengths]
        outs = list(out) if out is not None else [
            torch.zeros((3, int(n)), dtype=torch.float64, device=dev) for n in lengths]
        srcs = (_Source * ns)()
        gbs = (_GbParams * ns)()
        for i in range(ns):
            n = int(lengths[i])
            if hs[i].numel() != n or hs[i].dtype != torch.complex128 or not hs[i].is_cuda:
                raise ValueError(f"h[{i}] must be a complex128 CUDA buffer of {n} samples")
            if tuple(outs[i].shape) != (3, n) or outs[i].dtype != torch.float64:
                raise ValueError(f"out[{i}] must be a (3, {n}) float64 tensor")
            k, u, v = sky_basis(float(lam[i]), float(beta[i]))
            srcs[i] = _Source(hs[i].data_ptr(), outs[i].data_ptr(), n, self.projections_start_ind,
                              self.tdi_start_ind, float(t0[i]), (ctypes.c_double * 3)(*k),
                              (ctypes.c_double * 3)(*u), (ctypes.c_double * 3)(*v),
                              int(sets[i]), 0)
            gbs[i] = _GbParams(*[float(x) for x in params[i]])
        if stream is None:
            stream = torch.cuda.current_stream(dev)
        lib = _plan_fns()
        with torch.cuda.device(dev):
            rc = lib.flr_batch_run_gb(self._plan, srcs, gbs, ns, CHANNELS[self.tdi_chan],
                                      ctypes.c_void_p(stream.cuda_stream))
        _lib.check(rc)
        return outs, hs

    def status(self, reset: bool = False) -> int:
        """Kernel status bits (see include/flr_gb300.h; 0x10 = a staging copy
        did not complete); synchronises."""
        return self.cpp_orbits.status(reset=reset)
