"""CPU oracle for the LISA response + TDI hot path.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of ``bench.py`` may import this module, and only as the
checker or as the timed CPU baseline; the product never does.

Two parts:

* ctypes bindings of ``liboracle.so`` (``flr_oracle.c``), the plain-C
  restatement of the reference's CPU kernels (``LISAResponse.cu:110-672``);
* numpy restatements of the reference's host-side table builders in
  ``src/fastlisaresponse/response.py`` (A/E Lagrange tables, TDI unit tables,
  sky basis, buffer indices, XYZ->AET), each citing the lines it follows, and
  :class:`OracleResponseTDI`, which chains them like ``pyResponseTDI`` does.

Parity status: pinned.  ``tests/test_oracle.py`` checks this oracle bit for bit
against the reference's own CPU code compiled from its sources
(``make -C oracle ref``) and against the golden fixtures in ``tests/golden/``
produced by the reference's Python layer.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import threading
from math import factorial

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

C_INV = 3.3356409519815204e-09  # response.py:36
NO_LINK = -11  # response.py:390
LINKS = (12, 23, 31, 13, 32, 21)

_build_lock = threading.Lock()


def build(quiet: bool = True) -> None:
    """Compile liboracle.so / liboracle_o3.so (gcc, no GPU needed)."""
    with _build_lock:
        subprocess.run(
            ["make", "-s", "-C", HERE, "all"],
            check=True,
            stdout=subprocess.DEVNULL if quiet else None,
        )


_libs: dict = {}


def load(variant: str = "parity") -> ctypes.CDLL:
    """Load the oracle library; ``variant`` is "parity" (-O2, no FP contraction,
    bit-exact), "o3" (-O3, the CPU-baseline timing build) or "native" (-O3
    -march=native, for comparing with the reference's own build flags)."""
    name = {"parity": "liboracle.so", "o3": "liboracle_o3.so",
            "native": "liboracle_native.so"}[variant]
    if name in _libs:
        return _libs[name]
    path = os.path.join(HERE, name)
    src = os.path.join(HERE, "flr_oracle.c")
    if not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(src):
        if variant == "native":
            subprocess.run(["make", "-s", "-C", HERE, "liboracle_native.so"], check=True)
        else:
            build()
    lib = ctypes.CDLL(path)
    dp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
    lib.orc_get_response.restype = None
    lib.orc_get_response.argtypes = [
        ctypes.POINTER(_OrbitsC), dp, dp, dp, dp, dp, ctypes.c_int, dp, ctypes.c_int,
        ctypes.c_double, dp, ctypes.c_double, dp, ctypes.c_int, ip, ip,
    ]
    lib.orc_get_tdi_delays.restype = None
    lib.orc_get_tdi_delays.argtypes = [
        ctypes.POINTER(_OrbitsC), dp, dp, ctypes.c_int, ctypes.c_int, dp, ip, ip, ip, ip, dp, ip,
        ctypes.c_int, ctypes.c_int, ctypes.c_double, dp, ctypes.c_double, dp, ctypes.c_int, ip,
    ]
    lib.orc_get_response_range.restype = None
    lib.orc_get_response_range.argtypes = lib.orc_get_response.argtypes + [ctypes.c_int,
                                                                           ctypes.c_int]
    lib.orc_get_tdi_delays_range.restype = None
    lib.orc_get_tdi_delays_range.argtypes = lib.orc_get_tdi_delays.argtypes + [ctypes.c_int,
                                                                               ctypes.c_int]
    lib.orc_light_travel_time.restype = ctypes.c_double
    lib.orc_light_travel_time.argtypes = [ctypes.POINTER(_OrbitsC), ctypes.c_double, ctypes.c_int]
    lib.orc_position.restype = None
    lib.orc_position.argtypes = [ctypes.POINTER(_OrbitsC), ctypes.c_double, ctypes.c_int, dp]
    _libs[name] = lib
    return lib


class _OrbitsC(ctypes.Structure):
    _fields_ = [
        ("dt", ctypes.c_double),
        ("N", ctypes.c_int),
        ("ltt", ctypes.POINTER(ctypes.c_double)),
        ("x", ctypes.POINTER(ctypes.c_double)),
        ("links", ctypes.POINTER(ctypes.c_int)),
        ("sc_r", ctypes.POINTER(ctypes.c_int)),
        ("sc_e", ctypes.POINTER(ctypes.c_int)),
    ]


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


class OracleOrbits:
    """Orbit tables given as the 9 ``pycppdetector_args``
    ``[dt, N, n_arr, ltt_arr, x_arr, links, sc_r, sc_e, armlength]``
    (response.py:174, binding_flr.hpp:35-51)."""

    def __init__(self, dt, N, n_arr, ltt_arr, x_arr, links, sc_r, sc_e, armlength):
        self.dt = float(dt)
        self.N = int(N)
        self.ltt = _f64(ltt_arr).reshape(-1)
        self.x = _f64(x_arr).reshape(-1)
        self.links = _i32(links)
        self.sc_r = _i32(sc_r)
        self.sc_e = _i32(sc_e)
        if self.ltt.size != self.N * 6 or self.x.size != self.N * 9:
            raise ValueError("orbit tables have the wrong length")
        self.c = _OrbitsC(self.dt, self.N, _dp(self.ltt), _dp(self.x), _ip(self.links),
                          _ip(self.sc_r), _ip(self.sc_e))

    def light_travel_time(self, t: float, link: int) -> float:
        return load().orc_light_travel_time(ctypes.byref(self.c), float(t), int(link))

    def position(self, t: float, sc: int) -> np.ndarray:
        out = np.zeros(3)
        load().orc_position(ctypes.byref(self.c), float(t), int(sc), _dp(out))
        return out


def get_response(orbits: OracleOrbits, y_gw, t_data, k, u, v, num_delays, input_in, order,
                 sampling_frequency, A, deps, E, start, *, variant="parity",
                 return_indices=False, sample_range=None):
    """Oracle of ``LISAResponse::get_response`` (LISAResponse.cu:674-718).

    ``y_gw`` (float64, 6*num_delays) is written in place for the samples
    ``[start, num_delays-start)``.  With ``return_indices`` the integer receiver
    and emitter delays per (link, sample) are returned as int32 arrays of the
    same shape (-2**31 where not computed).  ``sample_range=(i0, i1)`` limits
    the work to samples in [i0, i1) (a slice of the full result)."""
    lib = load(variant)
    assert y_gw.dtype == np.float64 and y_gw.flags.c_contiguous and y_gw.size == 6 * num_delays
    t_data, k, u, v = _f64(t_data), _f64(k), _f64(u), _f64(v)
    h = np.ascontiguousarray(input_in, dtype=np.complex128).view(np.float64)
    A, E = _f64(A), _f64(E)
    d_rec = d_em = None
    if return_indices:
        d_rec = np.full(6 * num_delays, np.iinfo(np.int32).min, dtype=np.int32)
        d_em = d_rec.copy()
    i0, i1 = sample_range if sample_range is not None else (start, num_delays - start)
    lib.orc_get_response_range(ctypes.byref(orbits.c), _dp(y_gw), _dp(t_data), _dp(k), _dp(u),
                               _dp(v), int(num_delays), _dp(h), int(order),
                               float(sampling_frequency), _dp(A), float(deps), _dp(E), int(start),
                               _ip(d_rec) if d_rec is not None else None,
                               _ip(d_em) if d_em is not None else None, int(i0), int(i1))
    if return_indices:
        return d_rec, d_em
    return None


def get_tdi_delays(orbits: OracleOrbits, delayed_links, input_links, num_inputs, num_delays,
                   t_arr, unit_starts, unit_lengths, tdi_base_link, tdi_link_combinations,
                   tdi_signs, channels, num_units, order, sampling_frequency, A, deps, E, start,
                   *, variant="parity", return_indices=False, sample_range=None):
    """Oracle of ``LISAResponse::get_tdi_delays`` (LISAResponse.cu:399-429).

    ``delayed_links`` (float64, num_channels*num_delays) is accumulated into.
    With ``return_indices`` the integer delay per (unit, sample) is returned,
    shape (num_units, num_delays).  ``sample_range=(i0, i1)`` as in
    :func:`get_response`."""
    lib = load(variant)
    assert delayed_links.dtype == np.float64 and delayed_links.flags.c_contiguous
    y = _f64(input_links)
    t_arr = _f64(t_arr)
    us, ul, bl, lc, ch = (_i32(a) for a in (unit_starts, unit_lengths, tdi_base_link,
                                            tdi_link_combinations, channels))
    sg, A, E = _f64(tdi_signs), _f64(A), _f64(E)
    d_out = None
    if return_indices:
        d_out = np.full(num_units * num_delays, np.iinfo(np.int32).min, dtype=np.int32)
    i0, i1 = sample_range if sample_range is not None else (start, num_delays - start)
    lib.orc_get_tdi_delays_range(ctypes.byref(orbits.c), _dp(delayed_links), _dp(y),
                                 int(num_inputs), int(num_delays), _dp(t_arr), _ip(us), _ip(ul),
                                 _ip(bl), _ip(lc), _dp(sg), _ip(ch), int(num_units), int(order),
                                 float(sampling_frequency), _dp(A), float(deps), _dp(E),
                                 int(start), _ip(d_out) if d_out is not None else None, int(i0),
                                 int(i1))
    if return_indices:
        return d_out.reshape(num_units, num_delays)
    return None


# --------------------------------------------------------------------------
# Host-side tables, restated from src/fastlisaresponse/response.py
# --------------------------------------------------------------------------

def fill_A_E(order: int):
    """A(eps) on a 1001-point grid and the E_j weights (response.py:273-310).

    The reference's factorial table stops at 39! (response.py:276), which
    limits it to order <= 39; the table here is as long as the order needs and
    identical below 40.  Returns ``(A_in, E_in, deps)``; E_in has h entries of
    which the first h-1 are used (h = int((order+1)/2))."""
    h = int((order + 1) / 2)
    facts = np.asarray([float(factorial(n)) for n in range(max(40, 2 * h + 1))])
    num_A = 1001
    deps = 1.0 / (num_A - 1)
    eps = np.arange(num_A) * deps
    denominator = facts[h - 1] * facts[h]
    A_in = np.zeros_like(eps)
    for j, eps_i in enumerate(eps):
        acc = 1.0
        for i in range(1, h):
            acc *= (i + eps_i) * (i + 1 - eps_i)
        acc /= denominator
        A_in[j] = acc
    E_in = np.zeros((h,))
    for j in range(1, h):
        value = (facts[h - 1] / facts[h - 1 - j]) * (facts[h] / facts[h + j])
        E_in[j - 1] = value * (-1.0) ** j
    return A_in, E_in, deps


TDI_GEN1 = [  # response.py:318-327
    {"link": 13, "links_for_delay": [], "sign": +1},
    {"link": 31, "links_for_delay": [13], "sign": +1},
    {"link": 12, "links_for_delay": [13, 31], "sign": +1},
    {"link": 21, "links_for_delay": [13, 31, 12], "sign": +1},
    {"link": 12, "links_for_delay": [], "sign": -1},
    {"link": 21, "links_for_delay": [12], "sign": -1},
    {"link": 13, "links_for_delay": [12, 21], "sign": -1},
    {"link": 31, "links_for_delay": [12, 21, 13], "sign": -1},
]

TDI_GEN2_EXTRA = [  # response.py:331-356
    {"link": 12, "links_for_delay": [13, 31, 12, 21], "sign": +1},
    {"link": 21, "links_for_delay": [13, 31, 12, 21, 12], "sign": +1},
    {"link": 13, "links_for_delay": [13, 31, 12, 21, 12, 21], "sign": +1},
    {"link": 31, "links_for_delay": [13, 31, 12, 21, 12, 21, 13], "sign": +1},
    {"link": 13, "links_for_delay": [12, 21, 13, 31], "sign": -1},
    {"link": 31, "links_for_delay": [12, 21, 13, 31, 13], "sign": -1},
    {"link": 12, "links_for_delay": [12, 21, 13, 31, 13, 31], "sign": -1},
    {"link": 21, "links_for_delay": [12, 21, 13, 31, 13, 31, 12], "sign": -1},
]


def tdi_combinations(tdi):
    """response.py:316-365."""
    if tdi == "1st generation":
        return list(TDI_GEN1)
    if tdi == "2nd generation":
        return list(TDI_GEN1) + list(TDI_GEN2_EXTRA)
    if isinstance(tdi, list):
        return tdi
    raise ValueError("tdi kwarg should be '1st generation', '2nd generation', or a list "
                     "with a specific tdi combination.")


def cyclic_permutation(link: int, permutation: int) -> int:
    """response.py:421-433."""
    out = ""
    for ch in str(link)[:2]:
        temp = int(ch) + permutation
        if temp > 3:
            temp = temp % 3
        out += str(temp)
    return int(out)


def tdi_tables(combos) -> dict:
    """Unit tables expanded over the three cyclic permutations
    (response.py:372-419) plus unit starts/lengths (response.py:619-633)."""
    base, combs, signs, chans, op = [], [], [], [], []
    idx = 0
    for p in range(3):
        for c in combos:
            base.append(cyclic_permutation(c["link"], p))
            signs.append(float(c["sign"]))
            chans.append(p)
            if len(c["links_for_delay"]) == 0:
                combs.append(NO_LINK)
                op.append(idx)
            else:
                for ld in c["links_for_delay"]:
                    combs.append(cyclic_permutation(ld, p))
                    op.append(idx)
            idx += 1
    op = np.asarray(op, dtype=np.int32)
    _, starts, lengths = np.unique(op, return_index=True, return_counts=True)
    return dict(
        tdi_base_links=np.asarray(base, dtype=np.int32),
        tdi_link_combinations=np.asarray(combs, dtype=np.int32),
        tdi_signs=np.asarray(signs, dtype=np.float64),
        channels=np.asarray(chans, dtype=np.int32),
        tdi_operation_index=op,
        unit_starts=starts.astype(np.int32),
        unit_lengths=lengths.astype(np.int32),
        num_units=int(op.max() + 1),
    )


def sky_basis(lam: float, beta: float):
    """k, u, v of response.py:503-523 (ecliptic latitude beta)."""
    cb, sb, cl, sl = np.cos(beta), np.sin(beta), np.cos(lam), np.sin(lam)
    k = np.zeros(3)
    u = np.zeros(3)
    v = np.zeros(3)
    v[0] = -sb * cl
    v[1] = -sb * sl
    v[2] = cb
    u[0] = sl
    u[1] = -cl
    u[2] = 0.0
    k[0] = -cb * cl
    k[1] = -cb * sl
    k[2] = -sb
    return k, u, v


def buffer_indices(order: int, sampling_frequency: float, t_buffer: float, x_base) -> dict:
    """tdi_start_ind / projections_start_ind of response.py:474-500."""
    dt = 1 / sampling_frequency
    tdi_start_ind = int(t_buffer / dt)
    check_tdi_buffer = int(100.0 * sampling_frequency) + 4 * order
    x_base = np.asarray(x_base, dtype=np.float64)
    projection_buffer = int((np.sum(x_base * x_base, axis=-1) ** (1 / 2)).max() * C_INV) + 4 * order
    projections_start_ind = tdi_start_ind - 2 * check_tdi_buffer
    if projections_start_ind < projection_buffer:
        raise ValueError("Need to increase t_buffer. The initial buffer is not large enough.")
    return dict(tdi_start_ind=tdi_start_ind, projections_start_ind=projections_start_ind,
                check_tdi_buffer=check_tdi_buffer, projection_buffer=projection_buffer)


def AET(X, Y, Z):
    """XYZ -> AET as lisaanalysistools defines it (lisatools.utils.utility.AET,
    called at response.py:665): A=(Z-X)/sqrt2, E=(X-2Y+Z)/sqrt6, T=(X+Y+Z)/sqrt3."""
    return ((Z - X) / np.sqrt(2.0), (X - 2.0 * Y + Z) / np.sqrt(6.0), (X + Y + Z) / np.sqrt(3.0))


class OracleResponseTDI:
    """CPU chain of ``pyResponseTDI.get_projections`` + ``get_tdi_delays``
    (response.py:455-673) on the oracle kernels.  ``orbit_args`` are the
    ``pycppdetector_args``; ``x_base`` the untabulated positions used for the
    projection buffer (response.py:481)."""

    def __init__(self, sampling_frequency, num_pts, orbit_args, x_base, order=25,
                 tdi="1st generation", tdi_chan="XYZ", variant="parity"):
        self.sampling_frequency = sampling_frequency
        self.dt = 1 / sampling_frequency
        self.num_pts = int(num_pts)
        self.order = order
        self.tdi_chan = tdi_chan
        self.variant = variant
        self.A_in, self.E_in, self.deps = fill_A_E(order)
        self.tables = tdi_tables(tdi_combinations(tdi))
        self.orbits = OracleOrbits(*orbit_args)
        self.x_base = x_base

    def get_projections(self, input_in, lam, beta, t0=0.0, t_buffer=10000.0,
                        return_indices=False):
        idx = buffer_indices(self.order, self.sampling_frequency, t_buffer, self.x_base)
        self.tdi_start_ind = idx["tdi_start_ind"]
        self.projections_start_ind = idx["projections_start_ind"]
        self.t0 = t0
        k, u, v = sky_basis(lam, beta)
        input_in = np.ascontiguousarray(input_in, dtype=np.complex128)
        n = len(input_in)
        t_data = t0 + np.arange(n) * self.dt
        y_gw = np.zeros(6 * n)
        out = get_response(self.orbits, y_gw, t_data, k, u, v, n, input_in, self.order,
                           self.sampling_frequency, self.A_in, self.deps, self.E_in,
                           self.projections_start_ind, variant=self.variant,
                           return_indices=return_indices)
        self.y_gw_flat = y_gw
        self.y_gw_length = n
        return out

    @property
    def y_gw(self):
        return self.y_gw_flat.reshape(6, -1)

    def get_tdi_delays(self, return_indices=False):
        n = self.y_gw_length
        t_data = self.t0 + np.arange(n) * self.dt
        xyz = np.zeros(3 * n)
        tb = self.tables
        out = get_tdi_delays(self.orbits, xyz, self.y_gw_flat, n, n, t_data, tb["unit_starts"],
                             tb["unit_lengths"], tb["tdi_base_links"],
                             tb["tdi_link_combinations"], tb["tdi_signs"], tb["channels"],
                             tb["num_units"], self.order, self.sampling_frequency, self.A_in,
                             self.deps, self.E_in, self.tdi_start_ind, variant=self.variant,
                             return_indices=return_indices)
        self.XYZ = xyz.reshape(3, n)
        if return_indices:
            return out
        X, Y, Z = self.XYZ
        if self.tdi_chan == "XYZ":
            return X, Y, Z
        A, E, T = AET(X, Y, Z)
        return (A, E, T) if self.tdi_chan == "AET" else (A, E)
