"""LISA orbit tables in the layout the response kernels consume.

The reference takes its orbits from lisaanalysistools (``lisatools.detector``:
``Orbits``, ``EqualArmlengthOrbits``; used at ``response.py:13,119,227-259``),
which reads LISA Orbits HDF5 files.  Neither the package nor the files are
available here, so this module provides the part of that interface the
response path uses -- ``t_base``, ``x_base``, ``configure(...)``,
``configured``, ``LINKS``, ``t``, ``pycppdetector_args`` -- and two analytic
constellations:

* :class:`EqualArmlengthOrbits` -- a rigid equilateral triangle whose centre
  follows a circular 1 AU orbit and which rotates once per year in a plane
  tilted by 60 degrees (the first-order "cartwheel" solution); light travel
  times are all equal to armlength/c, as in LISA Orbits' equal-armlength
  product.
* :class:`KeplerianOrbits` -- each spacecraft on an exact Keplerian ellipse
  (Kepler's equation solved per sample); the arms breathe.  Keplerian
  elements at L = 2.5e9 m flex by about +-0.25 %; ``flex_scale`` takes the
  formation of a ``flex_scale`` times larger constellation and shrinks it
  about its centre, which multiplies the flexing (the default gives about
  +-1 %).  Light travel times solve c*L = |x_r(t) - x_e(t - L)| by fixed-point
  iteration.

Any object exposing ``pycppdetector_args`` (e.g. a real lisatools ``Orbits``
configured with ``linear_interp_setup=True``) works as well.
"""

from __future__ import annotations

import copy

import numpy as np

C_SI = 299792458.0
AU_SI = 1.495978707e11
YRSID_SI = 31558149.763545603

LINKS = [12, 23, 31, 13, 32, 21]
SC = [1, 2, 3]


class Orbits:
    """Tabulated orbits on a uniform grid starting at t = 0.

    Args:
        t_base: (N,) knot times [s], uniformly spaced from 0.
        x_base: (N, 3, 3) spacecraft positions [m] (spacecraft 1..3).
        ltt_base: (N, 6) light travel times [s] per link in ``LINKS`` order.
        n_base: (N, 6, 3) link unit vectors (receiver minus emitter direction).
        armlength: nominal arm length [m].
    """

    LINKS = LINKS
    SC = SC

    def __init__(self, t_base, x_base, ltt_base, n_base, armlength=2.5e9):
        self.t_base = np.ascontiguousarray(t_base, dtype=np.float64)
        self.x_base = np.ascontiguousarray(x_base, dtype=np.float64)
        self.ltt_base = np.ascontiguousarray(ltt_base, dtype=np.float64)
        self.n_base = np.ascontiguousarray(n_base, dtype=np.float64)
        self.armlength = float(armlength)
        n = len(self.t_base)
        if self.x_base.shape != (n, 3, 3) or self.ltt_base.shape != (n, 6) or \
                self.n_base.shape != (n, 6, 3):
            raise ValueError("orbit arrays must have shapes (N,3,3), (N,6), (N,6,3)")
        self._configured = False

    # -- lisatools-compatible surface -----------------------------------------
    @property
    def configured(self) -> bool:
        return self._configured

    def configure(self, t_arr=None, dt=None, linear_interp_setup=False):
        """Fix the grid the kernels interpolate on.

        With ``linear_interp_setup`` (what the response uses,
        response.py:239) the tables are put on a uniform grid from 0 with
        spacing ``dt`` (default: the base spacing).  Analytic subclasses
        re-evaluate their formulas on the new grid; plain tables are linearly
        resampled."""
        if t_arr is not None:
            t_arr = np.asarray(t_arr, dtype=np.float64)
            dt = float(t_arr[1] - t_arr[0])
        if dt is None:
            dt = float(self.t_base[1] - self.t_base[0])
        t = np.arange(0.0, self.t_base[-1] + 0.5 * dt, dt)
        if np.array_equal(t, self.t_base):
            self.t, self.x, self.ltt, self.n = self.t_base, self.x_base, self.ltt_base, self.n_base
        else:
            self.t = t
            self.x, self.ltt, self.n = self._evaluate(t)
        self.dt = float(dt)
        self._configured = True
        return self

    def _evaluate(self, t):
        x = np.stack([np.stack([np.interp(t, self.t_base, self.x_base[:, s, c]) for c in range(3)],
                               -1) for s in range(3)], 1)
        ltt = np.stack([np.interp(t, self.t_base, self.ltt_base[:, j]) for j in range(6)], -1)
        n = np.stack([np.stack([np.interp(t, self.t_base, self.n_base[:, j, c]) for c in range(3)],
                               -1) for j in range(6)], 1)
        return x, ltt, n

    @property
    def sc_r(self) -> np.ndarray:
        return np.asarray([int(str(link)[0]) for link in self.LINKS], dtype=np.int32)

    @property
    def sc_e(self) -> np.ndarray:
        return np.asarray([int(str(link)[1]) for link in self.LINKS], dtype=np.int32)

    @property
    def pycppdetector_args(self) -> list:
        """``[dt, N, n_arr, ltt_arr, x_arr, links, sc_r, sc_e, armlength]``
        (response.py:174, binding_flr.hpp:35-51)."""
        if not self._configured:
            self.configure(linear_interp_setup=True)
        return [
            float(self.dt),
            int(len(self.t)),
            np.ascontiguousarray(self.n.reshape(-1)),
            np.ascontiguousarray(self.ltt.reshape(-1)),
            np.ascontiguousarray(self.x.reshape(-1)),
            np.asarray(self.LINKS, dtype=np.int32),
            self.sc_r,
            self.sc_e,
            float(self.armlength),
        ]

    def __deepcopy__(self, memo):
        new = copy.copy(self)
        memo[id(self)] = new
        return new


def _link_tables(pos, t, L_guess, iterations=6, equal_ltt=None):
    """Light travel times and unit vectors for every link at times t."""
    xt = pos(t)
    ltt = np.empty((len(t), 6))
    n = np.empty((len(t), 6, 3))
    for j, link in enumerate(LINKS):
        r, e = int(str(link)[0]) - 1, int(str(link)[1]) - 1
        if equal_ltt is not None:
            L = np.full(len(t), equal_ltt)
        else:
            L = np.full(len(t), L_guess)
            for _ in range(iterations):
                L = np.linalg.norm(xt[:, r] - pos(t - L)[:, e], axis=-1) / C_SI
        d = xt[:, r] - pos(t - L)[:, e]
        ltt[:, j] = L
        n[:, j] = d / np.linalg.norm(d, axis=-1)[:, None]
    return xt, ltt, n


class _AnalyticOrbits(Orbits):
    def __init__(self, armlength, dt, t_max):
        self.armlength = float(armlength)
        t = np.arange(0.0, float(t_max) + 0.5 * dt, float(dt))
        x, ltt, n = self._evaluate(t)
        super().__init__(t, x, ltt, n, armlength)

    def positions(self, t):  # pragma: no cover - abstract
        raise NotImplementedError


class EqualArmlengthOrbits(_AnalyticOrbits):
    """Rigid equilateral constellation (first-order cartwheel), ltt = L/c.

    Args:
        armlength: arm length [m] (default 2.5e9).
        dt: table spacing [s] (default 1e4).
        t_max: last tabulated time [s] (default 10 years).
        R: radius of the guiding-centre orbit [m] (default 1 AU).
    """

    def __init__(self, armlength=2.5e9, dt=1e4, t_max=10 * YRSID_SI, R=AU_SI, phase=0.0):
        self.R = float(R)
        self.phase = float(phase)
        super().__init__(armlength, dt, t_max)

    def positions(self, t):
        t = np.asarray(t, dtype=np.float64)
        R = self.R
        e = self.armlength / (2.0 * np.sqrt(3.0) * R)
        alpha = 2.0 * np.pi * t / YRSID_SI + self.phase
        out = np.empty((t.size, 3, 3))
        for k in range(3):
            beta = 2.0 * np.pi * k / 3.0
            out[:, k, 0] = R * np.cos(alpha) + 0.5 * e * R * (np.cos(2 * alpha - beta)
                                                               - 3 * np.cos(beta))
            out[:, k, 1] = R * np.sin(alpha) + 0.5 * e * R * (np.sin(2 * alpha - beta)
                                                               - 3 * np.sin(beta))
            out[:, k, 2] = -np.sqrt(3.0) * e * R * np.cos(alpha - beta)
        return out

    def _evaluate(self, t):
        return _link_tables(self.positions, t, self.armlength / C_SI,
                            equal_ltt=self.armlength / C_SI)


class KeplerianOrbits(_AnalyticOrbits):
    """Three exact Keplerian orbits forming a breathing triangle.

    Each spacecraft k has semi-major axis R, eccentricity a/sqrt(3) and
    inclination a (a = flex_scale*L / (2R), the first-order stable-formation
    elements), with node and mean anomaly shifted by 2*pi*k/3.  Positions are
    then shrunk towards the three-spacecraft centre by 1/flex_scale, so the
    mean arm is L and the arm flexing is flex_scale times that of the Keplerian
    L-formation.
    """

    def __init__(self, armlength=2.5e9, dt=1e4, t_max=10 * YRSID_SI, R=AU_SI, flex_scale=4.2,
                 phase=0.0):
        self.R = float(R)
        self.flex_scale = float(flex_scale)
        self.phase = float(phase)
        super().__init__(armlength, dt, t_max)

    def positions(self, t):
        t = np.atleast_1d(np.asarray(t, dtype=np.float64))
        R = self.R
        a = self.flex_scale * self.armlength / (2.0 * R)
        ecc = a / np.sqrt(3.0)
        inc = a
        omega = 2.0 * np.pi / YRSID_SI
        out = np.empty((t.size, 3, 3))
        for k in range(3):
            sig = 2.0 * np.pi * k / 3.0
            M = omega * t + self.phase - sig
            E = M.copy()
            for _ in range(12):  # Newton on Kepler's equation E - e sin E = M
                E = E - (E - ecc * np.sin(E) - M) / (1.0 - ecc * np.cos(E))
            X = R * (np.cos(E) - ecc)
            Y = R * np.sqrt(1.0 - ecc * ecc) * np.sin(E)
            x, y, z = X * np.cos(inc), Y, -X * np.sin(inc)
            out[:, k, 0] = x * np.cos(sig) - y * np.sin(sig)
            out[:, k, 1] = x * np.sin(sig) + y * np.cos(sig)
            out[:, k, 2] = z
        centre = out.mean(axis=1, keepdims=True)
        return centre + (out - centre) / self.flex_scale

    def _evaluate(self, t):
        return _link_tables(self.positions, t, self.armlength / C_SI)


def read_lisa_orbits(path, armlength=2.5e9, h5py_module=None) -> Orbits:
    """Orbits from a LISA Orbits HDF5 file, the files lisatools' ``Orbits``
    reads for the reference (``response.py:13,119``): the barycentric (TCB)
    tables ``tcb/x`` (N, 3, 3) spacecraft positions [m], ``tcb/ltt`` (N, 6)
    light travel times [s] and ``tcb/n`` (N, 6, 3) link unit vectors, links in
    the order 12, 23, 31, 13, 32, 21, and the root attributes ``dt`` [s] and
    ``size`` (N); knot i is at i * dt.

    The file is read with h5py when it is installed, else with this
    package's own reader (:mod:`.h5lite`, the HDF5 structures h5py writes by
    default); ``h5py_module`` overrides both with any module that has h5py's
    ``File`` interface.  The tables can also be read by any other HDF5 reader
    and given to ``Orbits(t, x, ltt, n)`` directly."""
    if h5py_module is None:
        try:
            import h5py as h5py_module
        except ImportError:
            from . import h5lite as h5py_module
    with h5py_module.File(path, "r") as f:
        dt = float(f.attrs["dt"])
        size = int(f.attrs["size"])
        x = np.asarray(f["tcb"]["x"], dtype=np.float64)
        ltt = np.asarray(f["tcb"]["ltt"], dtype=np.float64)
        n = np.asarray(f["tcb"]["n"], dtype=np.float64)
    if not (dt > 0.0) or size < 2:
        raise ValueError(f"{path}: bad time grid (dt={dt}, size={size})")
    if x.shape[0] != size or ltt.shape[0] != size or n.shape[0] != size:
        raise ValueError(f"{path}: tables do not have `size` = {size} rows")
    return Orbits(np.arange(size) * dt, x.reshape(size, 3, 3), ltt.reshape(size, 6),
                  n.reshape(size, 6, 3), armlength)
