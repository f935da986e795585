"""Python classes with the reference backend's native interface, over the C ABI.

The reference exposes its CUDA code through pybind11 classes loaded by its
backend registry (``src/fastlisaresponse/cutils/__init__.py:14-40``):

* ``OrbitsWrapGPU_responselisa(dt, N, n_arr, ltt_arr, x_arr, links, sc_r, sc_e,
  armlength)`` (``cutils/binding_flr.hpp:32-59``)
* ``LISAResponseWrapGPU(orbits)`` with ``get_response_wrap(...)`` and
  ``get_tdi_delays_wrap(...)`` (``binding_flr.hpp:86-100``,
  ``binding_flr.cxx:16-58``)

:class:`OrbitsWrap` and :class:`LISAResponseWrap` take the same arguments in
the same order.  Arrays are torch CUDA tensors or any object exporting
``__cuda_array_interface__``; orbit tables may also be host (numpy) arrays.
Length checks follow the reference's ``return_pointer_and_check_length``
(``binding_flr.hpp:61-76``) and raise ``ValueError`` with its message.
Calls are enqueued on the current torch CUDA stream of the output's device and
return without synchronising.
"""

from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

try:  # torch is the device-array library of this package
    import torch
except ImportError:  # pragma: no cover - torch is a hard requirement on GPU hosts
    torch = None

_TYPESTR = {"f8": np.float64, "i4": np.int32, "c16": np.complex128}
_TORCH_DTYPES = {}
if torch is not None:
    _TORCH_DTYPES = {np.float64: torch.float64, np.int32: torch.int32,
                     np.complex128: torch.complex128}


def _length_error(name: str, expected: int, got: int) -> ValueError:
    return ValueError(f"{name}: input arrays have the incorrect length. Should be {expected}. "
                      f"It's length is {got}.")


class _Array:
    """Pointer, element count and placement of an array argument."""

    def __init__(self, obj, dtype, name: str, allow_host: bool = False):
        self.obj = obj  # keeps the memory alive for the call
        self.name = name
        if torch is not None and isinstance(obj, torch.Tensor):
            if obj.dtype != _TORCH_DTYPES[dtype]:
                raise TypeError(f"{name}: expected dtype {_TORCH_DTYPES[dtype]}, got {obj.dtype}")
            if not obj.is_contiguous():
                raise ValueError(f"{name}: array must be contiguous")
            if not obj.is_cuda and not allow_host:
                raise ValueError(f"{name}: must be a CUDA array")
            self.ptr = obj.data_ptr()
            self.size = obj.numel()
            self.device = obj.device.index if obj.is_cuda else None
            return
        cai = getattr(obj, "__cuda_array_interface__", None)
        if cai is not None:
            kind = cai["typestr"][1:]
            if _TYPESTR.get(kind) is not dtype:
                raise TypeError(f"{name}: expected {np.dtype(dtype)}, got {cai['typestr']}")
            shape = tuple(cai["shape"])
            strides = cai.get("strides")
            item = np.dtype(dtype).itemsize
            if strides is not None:
                expect, acc = [], item
                for dim in reversed(shape):
                    expect.append(acc)
                    acc *= dim
                if tuple(reversed(expect)) != tuple(strides):
                    raise ValueError(f"{name}: array must be contiguous")
            self.ptr = int(cai["data"][0])
            self.size = int(np.prod(shape)) if shape else 1
            self.device = None
            return
        if allow_host:
            arr = np.ascontiguousarray(obj, dtype=dtype)
            self.obj = arr
            self.ptr = arr.ctypes.data
            self.size = arr.size
            self.device = None
            return
        raise TypeError(f"{name}: expected a CUDA array (torch tensor or __cuda_array_interface__)")

    def check_length(self, n: int, multiplier: int = 1) -> "_Array":
        if self.size != n * multiplier:
            raise _length_error(self.name, n * multiplier, self.size)
        return self

    def check_min(self, n: int) -> "_Array":
        if self.size < n:
            raise ValueError(f"{self.name}: needs at least {n} elements, has {self.size}")
        return self


def _stream_for(arr: _Array):
    if torch is None or arr.device is None:
        return None
    return ctypes.c_void_p(torch.cuda.current_stream(arr.device).cuda_stream)


class OrbitsWrap:
    """Device-resident orbit tables (``OrbitsWrapGPU_responselisa``,
    binding_flr.hpp:32-59).  Tables are copied into memory owned by the
    handle; the arguments may be freed afterwards."""

    def __init__(self, dt, N, n_arr, ltt_arr, x_arr, links, sc_r, sc_e, armlength):
        self._handle = None
        N = int(N)
        n_a = _Array(n_arr, np.float64, "n_arr", allow_host=True).check_length(N, 6 * 3)
        ltt = _Array(ltt_arr, np.float64, "ltt_arr", allow_host=True).check_length(N, 6)
        x = _Array(x_arr, np.float64, "x_arr", allow_host=True).check_length(N, 3 * 3)
        lk = _Array(links, np.int32, "links", allow_host=True).check_length(6, 1)
        sr = _Array(sc_r, np.int32, "sc_r", allow_host=True).check_length(6, 1)
        se = _Array(sc_e, np.int32, "sc_e", allow_host=True).check_length(6, 1)
        self.dt = float(dt)
        self.N = N
        self.armlength = float(armlength)
        self.links = np.asarray(_host_copy(lk.obj), dtype=np.int32)
        self.sc_r = np.asarray(_host_copy(sr.obj), dtype=np.int32)
        self.sc_e = np.asarray(_host_copy(se.obj), dtype=np.int32)
        out = ctypes.c_void_p()
        _lib.check(_lib.lib().flr_orbits_create(self.dt, N, n_a.ptr, ltt.ptr, x.ptr, lk.ptr,
                                                sr.ptr, se.ptr, self.armlength,
                                                ctypes.byref(out)))
        self._handle = out

    @property
    def handle(self) -> ctypes.c_void_p:
        if self._handle is None:
            raise ValueError("Must add orbits with add_orbit_information method.")
        return self._handle

    def get_link_ind(self, link: int) -> int:
        hits = np.nonzero(self.links == int(link))[0]
        return int(hits[0]) if hits.size else -1

    def status(self, reset: bool = False, stream=None) -> int:
        """Sticky kernel status bits (see include/flr_gb300.h); synchronises."""
        bits = ctypes.c_uint32()
        _lib.check(_lib.lib().flr_orbits_status(self.handle, ctypes.byref(bits), int(reset),
                                                stream))
        return int(bits.value)

    def close(self) -> None:
        if self._handle is not None:
            _lib.lib().flr_orbits_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _host_copy(obj):
    if torch is not None and isinstance(obj, torch.Tensor):
        return obj.detach().cpu().numpy()
    if hasattr(obj, "__cuda_array_interface__"):
        return np.asarray(obj.get())  # CuPy-style
    return np.asarray(obj)


class LISAResponseWrap:
    """``LISAResponseWrapGPU`` (binding_flr.hpp:78-142) over libflr_gb300."""

    def __init__(self, orbits: OrbitsWrap):
        if not isinstance(orbits, OrbitsWrap):
            raise TypeError("orbits must be an OrbitsWrap")
        self.orbits = orbits
        self._checked_units = {}

    def _check_unit_tables(self, us, ul, bl, lc, sg, ch, num_units, num_channels):
        """The kernel follows unit_starts/unit_lengths into
        tdi_link_combinations and writes the rows named by `channels`; check
        once per set of table arrays that they stay inside their arrays (the
        reference checks neither)."""
        key = tuple((a.ptr, a.size, getattr(a.obj, "_version", None)) for a in
                    (us, ul, bl, lc, sg, ch)) + (num_units, num_channels)
        if key in self._checked_units:
            return
        starts = _host_copy(us.obj).astype(np.int64)[:num_units]
        lengths = _host_copy(ul.obj).astype(np.int64)[:num_units]
        chans = _host_copy(ch.obj)[:num_units]
        if num_units and (starts.min() < 0 or lengths.min() < 0 or
                          (starts + lengths).max() > lc.size):
            raise ValueError("unit_starts/unit_lengths point outside tdi_link_combinations")
        if num_units and (chans.min() < 0 or chans.max() >= num_channels):
            raise ValueError("channels must lie in [0, num_channels)")
        if len(self._checked_units) > 64:
            self._checked_units.clear()
        self._checked_units[key] = True

    def get_response_wrap(self, y_gw, t_data, k_in, u_in, v_in, dt, num_delays, input_in,
                          num_inputs, order, sampling_frequency, buffer_integer, A_in, deps,
                          num_A, E_in, projections_start_ind):
        """Link projections; argument list of binding_flr.cxx:38-58."""
        num_delays, num_inputs, num_A = int(num_delays), int(num_inputs), int(num_A)
        y = _Array(y_gw, np.float64, "y_gw").check_length(num_delays, 6)
        t = _Array(t_data, np.float64, "t_data").check_length(num_delays, 1)
        k = _Array(k_in, np.float64, "k_in").check_length(3, 1)
        u = _Array(u_in, np.float64, "u_in").check_length(3, 1)
        v = _Array(v_in, np.float64, "v_in").check_length(3, 1)
        h = _Array(input_in, np.complex128, "input_in").check_min(num_inputs)
        A = _Array(A_in, np.float64, "A_in").check_length(num_A, 1)
        E = _Array(E_in, np.float64, "E_in").check_min(max(int((order + 1) / 2) - 1, 0))
        rc = _lib.lib().flr_get_response(
            self.orbits.handle, y.ptr, t.ptr, k.ptr, u.ptr, v.ptr, float(dt), num_delays, h.ptr,
            num_inputs, int(order), float(sampling_frequency), int(buffer_integer), A.ptr,
            float(deps), num_A, E.ptr, int(projections_start_ind), _stream_for(y))
        _lib.check(rc)

    def get_tdi_delays_wrap(self, delayed_links, input_links, num_inputs, num_delays, t_arr,
                            unit_starts, unit_lengths, tdi_base_link, tdi_link_combinations,
                            tdi_signs_in, channels, num_units, num_channels, order,
                            sampling_frequency, buffer_integer, A_in, deps, num_A, E_in,
                            tdi_start_ind, aet=None, aet_rows=3):
        """TDI combinations; argument list of binding_flr.cxx:16-35.  With
        ``aet`` (an addition: a float64 array of aet_rows x num_delays), the
        same kernel also writes A, E (, T) of the accumulated X, Y, Z
        (flr_get_tdi_delays_aet)."""
        num_inputs, num_delays, num_units, num_A = (int(num_inputs), int(num_delays),
                                                    int(num_units), int(num_A))
        out = _Array(delayed_links, np.float64, "delayed_links").check_length(num_delays, 3)
        y = _Array(input_links, np.float64, "input_links").check_length(num_inputs, 6)
        t = _Array(t_arr, np.float64, "t_arr").check_length(num_delays, 1)
        us = _Array(unit_starts, np.int32, "unit_starts").check_length(num_units, 1)
        ul = _Array(unit_lengths, np.int32, "unit_lengths").check_length(num_units, 1)
        bl = _Array(tdi_base_link, np.int32, "tdi_base_link").check_min(num_units)
        lc = _Array(tdi_link_combinations, np.int32, "tdi_link_combinations")
        sg = _Array(tdi_signs_in, np.float64, "tdi_signs_in").check_min(num_units)
        ch = _Array(channels, np.int32, "channels").check_min(num_units)
        A = _Array(A_in, np.float64, "A_in").check_length(num_A, 1)
        E = _Array(E_in, np.float64, "E_in").check_min(max(int((order + 1) / 2) - 1, 0))
        out.check_min(int(num_channels) * num_delays)
        self._check_unit_tables(us, ul, bl, lc, sg, ch, num_units, int(num_channels))
        if aet is None:
            rc = _lib.lib().flr_get_tdi_delays(
                self.orbits.handle, out.ptr, y.ptr, num_inputs, num_delays, t.ptr, us.ptr,
                ul.ptr, bl.ptr, lc.ptr, sg.ptr, ch.ptr, num_units, int(num_channels), int(order),
                float(sampling_frequency), int(buffer_integer), A.ptr, float(deps), num_A, E.ptr,
                int(tdi_start_ind), _stream_for(out))
        else:
            ae = _Array(aet, np.float64, "aet").check_length(num_delays, int(aet_rows))
            rc = _lib.lib().flr_get_tdi_delays_aet(
                self.orbits.handle, out.ptr, y.ptr, num_inputs, num_delays, t.ptr, us.ptr,
                ul.ptr, bl.ptr, lc.ptr, sg.ptr, ch.ptr, num_units, int(num_channels), int(order),
                float(sampling_frequency), int(buffer_integer), A.ptr, float(deps), num_A, E.ptr,
                int(tdi_start_ind), ae.ptr, int(aet_rows), _stream_for(out))
        _lib.check(rc)

    # -- diagnostics (no reference counterpart) ---------------------------------
    def response_delay_indices(self, d_rec, d_em, t_data, k_in, num_delays, sampling_frequency,
                               projections_start_ind):
        dr = _Array(d_rec, np.int32, "d_rec").check_length(int(num_delays), 6)
        de = _Array(d_em, np.int32, "d_em").check_length(int(num_delays), 6)
        t = _Array(t_data, np.float64, "t_data").check_length(int(num_delays), 1)
        k = _Array(k_in, np.float64, "k_in").check_length(3, 1)
        _lib.check(_lib.lib().flr_response_delay_indices(
            self.orbits.handle, dr.ptr, de.ptr, t.ptr, k.ptr, int(num_delays),
            float(sampling_frequency), int(projections_start_ind), _stream_for(dr)))

    def tdi_delay_indices(self, d_tdi, num_delays, t_arr, unit_starts, unit_lengths,
                          tdi_link_combinations, num_units, sampling_frequency, tdi_start_ind):
        d = _Array(d_tdi, np.int32, "d_tdi").check_length(int(num_delays), int(num_units))
        t = _Array(t_arr, np.float64, "t_arr").check_length(int(num_delays), 1)
        us = _Array(unit_starts, np.int32, "unit_starts").check_length(int(num_units), 1)
        ul = _Array(unit_lengths, np.int32, "unit_lengths").check_length(int(num_units), 1)
        lc = _Array(tdi_link_combinations, np.int32, "tdi_link_combinations")
        starts, lengths = _host_copy(us.obj).astype(np.int64), _host_copy(ul.obj).astype(np.int64)
        if int(num_units) and (starts.min() < 0 or lengths.min() < 0 or
                               (starts + lengths).max() > lc.size):
            raise ValueError("unit_starts/unit_lengths point outside tdi_link_combinations")
        _lib.check(_lib.lib().flr_tdi_delay_indices(
            self.orbits.handle, d.ptr, int(num_delays), t.ptr, us.ptr, ul.ptr, lc.ptr,
            int(num_units), float(sampling_frequency), int(tdi_start_ind), _stream_for(d)))


# Names under which the reference's backend registry exposes these classes.
OrbitsWrapGPU_responselisa = OrbitsWrap
LISAResponseWrapGPU = LISAResponseWrap
