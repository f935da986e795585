"""``pyResponseTDI`` and ``ResponseWrapper`` with the reference's signatures,
running on the sm_103a kernels of libflr_gb300.

Mirrors ``src/fastlisaresponse/response.py`` (classes at :39-673 and
:676-863): same constructor and call signatures, same attributes and the same
host-side tables, so code written against the reference runs unchanged.
Differences, all deliberate:

* arrays are torch tensors on the GPU (the reference returns CuPy arrays);
  inputs may be numpy arrays, torch tensors or ``__cuda_array_interface__``
  objects;
* there is one backend (this GPU library); ``force_backend="cpu"`` raises;
* ``orbits`` may be an orbit class (instantiated with defaults) or an instance;
* tables (A/E, TDI units, unit starts) are built once and kept on the device,
  not rebuilt per call (response.py:481-494, 619-633 redo them each call);
* the TDI sum over units is deterministic (no atomics);
* ``get_tdi_delays(y_gw=...)`` checks the shape against the 6 links (the
  reference asserts against an attribute it never sets, response.py:606).
"""

from __future__ import annotations

import warnings
from math import factorial
from typing import List, Optional

import numpy as np

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None

from . import _lib
from .binding import LISAResponseWrap, OrbitsWrap
from .orbits import EqualArmlengthOrbits, Orbits

YRSID_SI = 31558149.763545603
C_inv = 3.3356409519815204e-09  # response.py:36
NLINKS = 6
NO_LINK = -11


# --------------------------------------------------------------------------
# host-side tables
# --------------------------------------------------------------------------

def lagrange_tables(order: int):
    """A(eps) on 1001 points and the E_j weights of the Lagrange kernel
    (response.py:273-310), evaluated with the same float64 operations.

    The reference's factorial table ends at 39! (response.py:276), so it
    supports order <= 39; here the table is extended with exact integers
    rounded to float64 (identical entries below 40), which adds order 41-79.
    Returns (A_in, E_in, deps) as numpy arrays; E_in has h entries."""
    h = int((order + 1) / 2)
    facts = np.asarray([float(factorial(n)) for n in range(max(40, 2 * h + 1))])
    num_A = 1001
    deps = 1.0 / (num_A - 1)
    eps = np.arange(num_A) * deps
    denominator = facts[h - 1] * facts[h]
    A_in = np.zeros_like(eps)
    for j, eps_i in enumerate(eps):
        A = 1.0
        for i in range(1, h):
            A *= (i + eps_i) * (i + 1 - eps_i)
        A /= denominator
        A_in[j] = A
    E_in = np.zeros((h,))
    for j in range(1, h):
        first_term = facts[h - 1] / facts[h - 1 - j]
        second_term = facts[h] / facts[h + j]
        E_in[j - 1] = first_term * second_term * (-1.0) ** j
    return A_in, E_in, deps


TDI_FIRST_GENERATION = [  # response.py:318-327
    {"link": 13, "links_for_delay": [], "sign": +1},
    {"link": 31, "links_for_delay": [13], "sign": +1},
    {"link": 12, "links_for_delay": [13, 31], "sign": +1},
    {"link": 21, "links_for_delay": [13, 31, 12], "sign": +1},
    {"link": 12, "links_for_delay": [], "sign": -1},
    {"link": 21, "links_for_delay": [12], "sign": -1},
    {"link": 13, "links_for_delay": [12, 21], "sign": -1},
    {"link": 31, "links_for_delay": [12, 21, 13], "sign": -1},
]

TDI_SECOND_GENERATION_EXTRA = [  # response.py:331-356
    {"link": 12, "links_for_delay": [13, 31, 12, 21], "sign": +1},
    {"link": 21, "links_for_delay": [13, 31, 12, 21, 12], "sign": +1},
    {"link": 13, "links_for_delay": [13, 31, 12, 21, 12, 21], "sign": +1},
    {"link": 31, "links_for_delay": [13, 31, 12, 21, 12, 21, 13], "sign": +1},
    {"link": 13, "links_for_delay": [12, 21, 13, 31], "sign": -1},
    {"link": 31, "links_for_delay": [12, 21, 13, 31, 13], "sign": -1},
    {"link": 12, "links_for_delay": [12, 21, 13, 31, 13, 31], "sign": -1},
    {"link": 21, "links_for_delay": [12, 21, 13, 31, 13, 31, 12], "sign": -1},
]


def cyclic_permutation(link: int, permutation: int) -> int:
    """Spacecraft relabelling 1->2->3->1 applied `permutation` times to both
    digits of a link number (response.py:421-433)."""
    digits = []
    for ch in str(link)[:2]:
        sc = int(ch) + permutation
        digits.append(str(sc % 3 if sc > 3 else sc))
    return int("".join(digits))


def tdi_unit_tables(tdi_combinations) -> dict:
    """Flatten a TDI combination list over the 3 cyclic permutations into the
    int32/float64 unit tables of the kernel (response.py:372-419, 619-633)."""
    base, combos, signs, channels, op = [], [], [], [], []
    unit = 0
    for perm in range(3):
        for term in tdi_combinations:
            base.append(cyclic_permutation(term["link"], perm))
            signs.append(float(term["sign"]))
            channels.append(perm)
            delays = term["links_for_delay"]
            if len(delays) == 0:
                combos.append(NO_LINK)
                op.append(unit)
            else:
                for link in delays:
                    combos.append(cyclic_permutation(link, perm))
                    op.append(unit)
            unit += 1
    op = np.asarray(op, dtype=np.int32)
    if op.size and not np.all((np.diff(op) == 0) | (np.diff(op) == 1)):
        raise ValueError("TDI operation indices must be contiguous")
    _, starts, lengths = np.unique(op, return_index=True, return_counts=True)
    return {
        "tdi_base_links": np.asarray(base, dtype=np.int32),
        "tdi_link_combinations": np.asarray(combos, dtype=np.int32),
        "tdi_signs": np.asarray(signs, dtype=np.float64),
        "channels": np.asarray(channels, dtype=np.int32),
        "tdi_operation_index": op,
        "unit_starts": starts.astype(np.int32),
        "unit_lengths": lengths.astype(np.int32),
        "num_units": int(op.max() + 1) if op.size else 0,
    }


def sky_basis(lam: float, beta: float):
    """Propagation direction k and polarisation basis u, v (response.py:503-523)."""
    cosbeta, sinbeta = np.cos(beta), np.sin(beta)
    coslam, sinlam = np.cos(lam), np.sin(lam)
    v = np.array([-sinbeta * coslam, -sinbeta * sinlam, cosbeta])
    u = np.array([sinlam, -coslam, 0.0])
    k = np.array([-cosbeta * coslam, -cosbeta * sinlam, -sinbeta])
    return k, u, v


def _resolve_device(force_backend):
    if torch is None:
        raise RuntimeError("torch is required (device arrays and streams)")
    if isinstance(force_backend, torch.device):
        return force_backend
    if isinstance(force_backend, int):
        return torch.device("cuda", force_backend)
    if force_backend in (None, "gpu", "cuda", "cuda13x", "gb300", "fastlisaresponse_gb300"):
        if not torch.cuda.is_available():
            raise RuntimeError("no CUDA device: this library runs on the GPU only "
                               "(there is no CPU backend)")
        return torch.device("cuda", torch.cuda.current_device())
    if isinstance(force_backend, str) and force_backend.startswith("cuda:"):
        return torch.device(force_backend)
    if force_backend == "cpu":
        raise ValueError("force_backend='cpu': this library has no CPU backend; "
                         "it runs the response on the GPU only")
    raise ValueError(f"unknown backend {force_backend!r}")


def _as_device(x, device, dtype):
    if isinstance(x, torch.Tensor):
        return x.to(device=device, dtype=dtype).contiguous()
    if hasattr(x, "__cuda_array_interface__"):
        return torch.as_tensor(x, device=device).to(dtype).contiguous()
    return torch.as_tensor(np.asarray(x), dtype=dtype).to(device).contiguous()


def _orbit_instance(orbits):
    if orbits is None:
        orbits = EqualArmlengthOrbits()
    elif isinstance(orbits, type):
        orbits = orbits()
    if not hasattr(orbits, "pycppdetector_args"):
        raise TypeError("orbits must provide pycppdetector_args (an Orbits instance)")
    return orbits


# --------------------------------------------------------------------------
# pyResponseTDI
# --------------------------------------------------------------------------

class pyResponseTDI:
    """Time-domain LISA response: projections onto the 6 links and TDI.

    Args (as response.py:113-123):
        sampling_frequency (float): sampling rate [Hz].
        num_pts (int): number of samples of the output.
        order (int): Lagrange interpolation order (default 25).
        tdi (str or list): "1st generation", "2nd generation" or a list of
            {"link", "links_for_delay", "sign"} terms.
        orbits: orbit class or instance (default :class:`EqualArmlengthOrbits`).
        tdi_orbits: accepted for compatibility; as in the reference, the TDI
            delays use the response orbits.
        tdi_chan (str): "XYZ", "AET" or "AE".
        force_backend: None/"gpu"/"cuda13x"/device; "cpu" raises.
    """

    def __init__(self, sampling_frequency, num_pts, order=25, tdi="1st generation",
                 orbits: Optional[Orbits] = EqualArmlengthOrbits,
                 tdi_orbits: Optional[Orbits] = None, tdi_chan="XYZ", force_backend=None):
        self.sampling_frequency = sampling_frequency
        self.dt = 1 / sampling_frequency
        self.tdi_buffer = 200
        self.num_pts = num_pts
        self.order = order
        self.buffer_integer = self.order * 2 + 1
        self.half_order = int((order + 1) / 2)
        self.tdi = tdi
        self.tdi_chan = tdi_chan
        self.device = _resolve_device(force_backend)
        self._fill_A_E()

        self.response_orbits = orbits
        if tdi_orbits is None:
            tdi_orbits = self.response_orbits
        self.tdi_orbits = tdi_orbits

        if self.num_pts * self.dt > self.response_orbits.t_base.max():
            warnings.warn("Input number of points is longer in time than available orbital "
                          "information. Trimming to fit orbital information.")
            self.num_pts = int(self.response_orbits.t_base.max() / self.dt)

        self._init_TDI_delays()
        with torch.cuda.device(self.device):
            self.cpp_orbits = OrbitsWrap(*self.response_orbits.pycppdetector_args)
        self.cpp_response = LISAResponseWrap(self.cpp_orbits)
        self.y_gw_flat = None
        self.t0_projection = None
        self.nlinks = NLINKS

    # -- reference-compatible properties ----------------------------------------
    @property
    def xp(self):
        return torch

    @property
    def response_gen(self):
        """GPU function for the projections (response.py:208-211)."""
        return self.cpp_response.get_response_wrap

    @property
    def tdi_gen(self):
        """GPU function for TDI (response.py:213-216)."""
        return self.cpp_response.get_tdi_delays_wrap

    @property
    def citation(self):
        return "Katz et al., arXiv:2204.06633 (fastlisaresponse)"

    @classmethod
    def supported_backends(cls):
        return ["fastlisaresponse_gb300"]

    @property
    def response_orbits(self):
        return self._response_orbits

    @response_orbits.setter
    def response_orbits(self, orbits):
        orbits = _orbit_instance(orbits)
        from copy import deepcopy

        self._response_orbits = deepcopy(orbits)
        if not self._response_orbits.configured:
            self._response_orbits.configure(linear_interp_setup=True)
        x_base = np.asarray(self._response_orbits.x_base, dtype=np.float64)
        self._max_sc_distance = float((np.sum(x_base * x_base, axis=-1) ** (1 / 2)).max())

    @property
    def tdi_orbits(self):
        return self._tdi_orbits

    @tdi_orbits.setter
    def tdi_orbits(self, orbits):
        from copy import deepcopy

        orbits = _orbit_instance(orbits)
        self._tdi_orbits = deepcopy(orbits)
        if not self._tdi_orbits.configured:
            self._tdi_orbits.configure(linear_interp_setup=True)

    def _fill_A_E(self):
        A_in, E_in, deps = lagrange_tables(self.order)
        self.num_A = len(A_in)
        self.deps = deps
        self.A_in_host, self.E_in_host = A_in, E_in
        self.A_in = torch.as_tensor(A_in, device=self.device)
        self.E_in = torch.as_tensor(E_in, device=self.device)

    def _init_TDI_delays(self):
        if self.tdi in ["1st generation", "2nd generation"]:
            combos = list(TDI_FIRST_GENERATION)
            if self.tdi == "2nd generation":
                combos += TDI_SECOND_GENERATION_EXTRA
        elif isinstance(self.tdi, list):
            combos = self.tdi
        else:
            raise ValueError("tdi kwarg should be '1st generation', '2nd generation', or a list "
                             "with a specific tdi combination.")
        self.tdi_combinations = combos

    @property
    def tdi_combinations(self) -> List:
        return self._tdi_combinations

    @tdi_combinations.setter
    def tdi_combinations(self, tdi_combinations: List) -> None:
        tables = tdi_unit_tables(tdi_combinations)
        known = set(int(x) for x in self._response_orbits.LINKS)
        used = set(tables["tdi_base_links"].tolist()) | \
            set(x for x in tables["tdi_link_combinations"].tolist() if x != NO_LINK)
        if not used <= known:
            raise ValueError(f"TDI combinations use links {sorted(used - known)} that the "
                             "orbits do not define")
        self._tdi_combinations = tdi_combinations
        self.tdi_tables_host = tables
        dev = self.device
        self.tdi_operation_index = torch.as_tensor(tables["tdi_operation_index"], device=dev)
        self.tdi_base_links = torch.as_tensor(tables["tdi_base_links"], device=dev)
        self.tdi_link_combinations = torch.as_tensor(tables["tdi_link_combinations"], device=dev)
        self.tdi_signs = torch.as_tensor(tables["tdi_signs"], device=dev)
        self.channels = torch.as_tensor(tables["channels"], device=dev)
        self.unit_starts = torch.as_tensor(tables["unit_starts"], device=dev)
        self.unit_lengths = torch.as_tensor(tables["unit_lengths"], device=dev)
        self.num_units = tables["num_units"]

    # -- projections --------------------------------------------------------------
    @property
    def y_gw(self):
        """Projections along the arms, shape (6, num_pts)."""
        return self.y_gw_flat.reshape(self.nlinks, -1)

    def buffer_indices(self, t_buffer: float) -> dict:
        """tdi_start_ind and projections_start_ind (response.py:474-500)."""
        tdi_start_ind = int(t_buffer / self.dt)
        check_tdi_buffer = int(100.0 * self.sampling_frequency) + 4 * self.order
        projection_buffer = int(self._max_sc_distance * C_inv) + 4 * self.order
        projections_start_ind = tdi_start_ind - 2 * check_tdi_buffer
        if projections_start_ind < projection_buffer:
            raise ValueError("Need to increase t_buffer. The initial buffer is not large enough.")
        return dict(tdi_start_ind=tdi_start_ind, check_tdi_buffer=check_tdi_buffer,
                    projection_buffer=projection_buffer,
                    projections_start_ind=projections_start_ind)

    def _data_time_check(self, t_data, input_in):
        t_last = float(self._t_first) + (len(input_in) - 1) * self.dt
        t_max = float(np.max(self.response_orbits.t))
        if t_last > t_max:
            warnings.warn("Input waveform is longer than available orbital information. "
                          "Trimming to fit orbital information.")
            keep = int(np.floor((t_max - float(self._t_first)) / self.dt)) + 1
            while keep > 0 and float(self._t_first) + (keep - 1) * self.dt > t_max:
                keep -= 1
            t_data = t_data[:max(keep - 1, 0)]
            input_in = input_in[:max(keep - 1, 0)]
        return t_data, input_in

    def get_projections(self, input_in, lam, beta, t0=0.0, t_buffer=10000.0):
        """Project h+ + i hx onto the six links (response.py:455-560).

        Args:
            input_in: complex h+ + i hx, length num_pts (numpy, torch or CAI).
            lam, beta: ecliptic longitude / latitude [rad].
            t0: time of the first input sample [s].
            t_buffer: garbage time removed at each end [s].
        """
        idx = self.buffer_indices(t_buffer)
        self.tdi_start_ind = idx["tdi_start_ind"]
        self.check_tdi_buffer = idx["check_tdi_buffer"]
        self.projection_buffer = idx["projection_buffer"]
        self.projections_start_ind = idx["projections_start_ind"]
        self.t0_projection = t0

        k, u, v = sky_basis(lam, beta)
        dev = self.device
        self.num_total_points = len(input_in)
        k_in = torch.as_tensor(k, device=dev)
        u_in = torch.as_tensor(u, device=dev)
        v_in = torch.as_tensor(v, device=dev)
        input_in = _as_device(input_in, dev, torch.complex128)
        self._t_first = t0
        t_data = t0 + torch.arange(len(input_in), dtype=torch.float64, device=dev) * self.dt
        t_data, input_in = self._data_time_check(t_data, input_in)
        if len(input_in) < self.num_pts:
            raise ValueError(f"input_in has {len(input_in)} samples, fewer than num_pts="
                             f"{self.num_pts}")
        y_gw = torch.zeros((self.nlinks * self.num_pts,), dtype=torch.float64, device=dev)
        with torch.cuda.device(dev), _lib.nvtx_range("flr.get_response"):
            self.response_gen(y_gw, t_data, k_in, u_in, v_in, self.dt, len(input_in), input_in,
                              len(input_in), self.order, self.sampling_frequency,
                              self.buffer_integer, self.A_in, self.deps, len(self.A_in),
                              self.E_in, self.projections_start_ind)
        self.y_gw_flat = y_gw
        self.y_gw_length = self.num_pts

    # -- TDI -----------------------------------------------------------------------
    @property
    def XYZ(self):
        """TDI X, Y, Z, shape (3, num_pts)."""
        return self.delayed_links_flat.reshape(3, -1)

    def get_tdi_delays(self, t0=None, y_gw=None):
        """TDI combinations from the projections (response.py:567-673).

        Returns (X, Y, Z), (A, E, T) or (A, E) per ``tdi_chan``."""
        dev = self.device
        self.delayed_links_flat = torch.zeros((3, self.num_pts), dtype=torch.float64, device=dev)
        if t0 is None:
            t0 = self.t0_projection
            if t0 is None:
                t0 = 0.0
        elif self.t0_projection is not None and self.t0_projection != t0:
            raise ValueError("If running projections with a t0 value, that t0 value needs to be "
                             "the same for TDI. If you want to force otherwise, need to run "
                             "'del class.t0_projections' before TDI computation.")
        if y_gw is not None:
            y_gw = _as_device(y_gw, dev, torch.float64)
            if tuple(y_gw.shape) != (self.nlinks, self.num_pts):
                raise ValueError(f"y_gw must have shape ({self.nlinks}, {self.num_pts})")
            self.y_gw_flat = y_gw.flatten().clone()
            self.y_gw_length = self.num_pts
            if not hasattr(self, "tdi_start_ind"):
                raise ValueError("run get_projections first or set tdi_start_ind")
        elif self.y_gw_flat is None:
            raise ValueError("Need to either enter projection array or have this code "
                             "determine projections.")
        self.delayed_links_flat = self.delayed_links_flat.flatten()
        t_data = t0 + torch.arange(self.y_gw_length, dtype=torch.float64, device=dev) * self.dt
        if self.tdi_chan not in ("XYZ", "AET", "AE"):
            raise ValueError("tdi_chan must be 'XYZ', 'AET' or 'AE'.")
        # lisatools' AET (response.py:659-673) in the TDI kernel's epilogue: the
        # same values (zero outside the TDI range, as lisatools' AET of zeros)
        rows = {"XYZ": 0, "AET": 3, "AE": 2}[self.tdi_chan]
        aet = torch.zeros((rows, self.num_pts), dtype=torch.float64, device=dev) if rows else None
        with torch.cuda.device(dev), _lib.nvtx_range("flr.get_tdi_delays"):
            self.tdi_gen(self.delayed_links_flat, self.y_gw_flat, self.y_gw_length, self.num_pts,
                         t_data, self.unit_starts, self.unit_lengths, self.tdi_base_links,
                         self.tdi_link_combinations, self.tdi_signs, self.channels,
                         self.num_units, 3, self.order, self.sampling_frequency,
                         self.buffer_integer, self.A_in, self.deps, len(self.A_in), self.E_in,
                         self.tdi_start_ind, **({"aet": aet, "aet_rows": rows} if rows else {}))
        if not rows:
            X, Y, Z = self.XYZ
            return X, Y, Z
        return tuple(aet[r] for r in range(rows))

    def status(self, reset: bool = False) -> int:
        """Kernel status bits of this instance's orbit handle (synchronises)."""
        return self.cpp_orbits.status(reset=reset)


# --------------------------------------------------------------------------
# ResponseWrapper
# --------------------------------------------------------------------------

class ResponseWrapper:
    """Waveform generator + LISA response + TDI (response.py:676-863).

    Args: waveform_gen, Tobs [yr], dt [s], index_lambda, index_beta, t0=0.0,
    t_buffer=10000.0, flip_hx=False, remove_sky_coords=False,
    is_ecliptic_latitude=True, force_backend=None, remove_garbage=True,
    n_overide=None, orbits=EqualArmlengthOrbits, **kwargs for pyResponseTDI.

    One addition, off by default: ``precision="fp64"`` or ``"mixed"`` computes
    the channels with the fused kernel (:class:`BatchedResponseTDI`; one
    launch, the link streams never stored) instead of get_projections +
    get_tdi_delays: "fp64" gives the same bits, "mixed" the bit-exact integer
    delays and the channels within 1e-6 relative L2 at ~16x the speed.
    ``chunks`` splits that launch (long observations; see
    BatchedResponseTDI.__call__).
    """

    def __init__(self, waveform_gen, Tobs, dt, index_lambda, index_beta, t0=0.0,
                 t_buffer=10000.0, flip_hx=False, remove_sky_coords=False,
                 is_ecliptic_latitude=True, force_backend=None, remove_garbage=True,
                 n_overide=None, orbits: Optional[Orbits] = EqualArmlengthOrbits,
                 precision: Optional[str] = None, chunks: int = 1, **kwargs):
        self.waveform_gen = waveform_gen
        self.index_lambda = index_lambda
        self.index_beta = index_beta
        self.dt = dt
        self.t0 = t0
        self.t_buffer = t_buffer
        self.sampling_frequency = 1.0 / dt
        orbits = _orbit_instance(orbits)
        if Tobs * YRSID_SI > orbits.t_base.max():
            warnings.warn("Tobs is larger than available orbital information time array. "
                          f"Reducing Tobs to {orbits.t_base.max()}")
            Tobs = orbits.t_base.max() / YRSID_SI
        if n_overide is not None:
            if not isinstance(n_overide, int):
                raise ValueError("n_overide must be an integer if not None.")
            self.n = n_overide
        else:
            self.n = int(Tobs * YRSID_SI / dt)
        self.Tobs = self.n * dt
        self.is_ecliptic_latitude = is_ecliptic_latitude
        self.remove_sky_coords = remove_sky_coords
        self.flip_hx = flip_hx
        self.remove_garbage = remove_garbage
        self.response_model = pyResponseTDI(self.sampling_frequency, self.n, orbits=orbits,
                                            force_backend=force_backend, **kwargs)
        self.Tobs = (self.n * self.response_model.dt) / YRSID_SI
        self.precision = precision
        self.chunks = int(chunks)
        self._fused = None
        if precision is not None:
            from .batch import BatchedResponseTDI

            self._fused = BatchedResponseTDI(
                self.sampling_frequency, order=kwargs.get("order", 25),
                tdi=kwargs.get("tdi", "1st generation"), orbits=orbits,
                tdi_chan=kwargs.get("tdi_chan", "XYZ"), precision=precision,
                t_buffer=t_buffer, force_backend=self.response_model.device)
            self._nchan = 2 if kwargs.get("tdi_chan", "XYZ") == "AE" else 3

    @property
    def xp(self):
        return torch

    @property
    def citation(self):
        return self.response_model.citation

    @classmethod
    def supported_backends(cls):
        return ["fastlisaresponse_gb300"]

    def __call__(self, *args, **kwargs):
        args = list(args)
        beta = args[self.index_beta]
        lam = args[self.index_lambda]
        if self.remove_sky_coords:
            args.pop(self.index_beta)
            args.pop(self.index_lambda)
        if not self.is_ecliptic_latitude:
            beta = np.pi / 2.0 - beta
        kwargs["T"] = self.Tobs
        kwargs["dt"] = self.dt
        h = self.waveform_gen(*args, **kwargs)
        if self.flip_hx:
            h = h.real - 1j * h.imag if not isinstance(h, torch.Tensor) else h.conj().resolve_conj()
        if self._fused is not None:
            chans = self._fused([h], lam, beta, t0=self.t0, chunks=self.chunks)[0]
            out = [chans[c] for c in range(self._nchan)]
        else:
            self.response_model.get_projections(h, lam, beta, t0=self.t0,
                                                t_buffer=self.t_buffer)
            out = list(self.response_model.get_tdi_delays())
        ts = (self._fused or self.response_model).tdi_start_ind
        if self.remove_garbage is True:
            for i in range(len(out)):
                out[i] = out[i][ts:-ts]
        elif isinstance(self.remove_garbage, str):
            if self.remove_garbage != "zero":
                raise ValueError("remove_garbage must be True, False, or 'zero'.")
            for i in range(len(out)):
                out[i][:ts] = 0.0
                out[i][-ts:] = 0.0
        return out
