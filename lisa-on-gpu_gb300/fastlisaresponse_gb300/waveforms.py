"""Galactic-binary waveform generators producing complex h+ + i hx.

* :func:`gb_waveform` -- the monochromatic-with-drift binary of the benchmark
  configurations: h+ = A(1+cos^2 i) cos(Phi), hx = -2A cos(i) sin(Phi),
  Phi = phi0 + 2 pi (f t + fdot t^2 / 2), rotated by the polarisation psi.
* :class:`GBWave` -- the generator of the reference's test-suite
  (``tests/test_fastlisaresponse.py:34-63``: third-order phase with
  fddot = 11/3 fdot^2/f, phase origin -phi0), so a ResponseWrapper set up
  like the reference's test produces the same input.

Both evaluate in float64 with numpy (host) or torch (any device).
"""

from __future__ import annotations

import math

import numpy as np

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None

YRSID_SI = 31558149.763545603


def _ns(device):
    if device is None:
        return np
    if torch is None:
        raise RuntimeError("torch is required for device waveforms")
    return torch


def time_grid(n: int, dt: float, t0: float = 0.0, device=None):
    """t0 + arange(n) * dt, the sample times used throughout (response.py:532)."""
    if device is None:
        return t0 + np.arange(n) * dt
    return t0 + torch.arange(n, dtype=torch.float64, device=device) * dt


def gb_waveform(A, f, fdot, iota, phi0, psi, t):
    """Complex h+ + i hx of a drifting monochromatic binary at times t."""
    xp = torch if (torch is not None and isinstance(t, torch.Tensor)) else np
    phase = phi0 + 2.0 * math.pi * (f * t + 0.5 * fdot * t * t)
    cosi = math.cos(iota)
    hp0 = A * (1.0 + cosi * cosi) * xp.cos(phase)
    hc0 = -2.0 * A * cosi * xp.sin(phase)
    c2, s2 = math.cos(2.0 * psi), math.sin(2.0 * psi)
    hp = hp0 * c2 - hc0 * s2
    hc = hp0 * s2 + hc0 * c2
    if xp is np:
        return hp + 1j * hc
    return torch.complex(hp, hc)


class GBWave:
    """Waveform generator of the reference's tests (tests/test_fastlisaresponse.py:34-63).

    ``GBWave(device=None)(A, f, fdot, iota, phi0, psi, T=1.0, dt=10.0)``
    returns h+ + i hx on ``t = arange(0, T*YRSID_SI, dt)``; numpy when
    ``device`` is None, else a torch tensor on that device."""

    def __init__(self, device=None):
        self.device = device

    def __call__(self, A, f, fdot, iota, phi0, psi, T=1.0, dt=10.0):
        if self.device is None:
            t = np.arange(0.0, T * YRSID_SI, dt)
            xp = np
        else:
            t = torch.arange(0.0, T * YRSID_SI, dt, dtype=torch.float64, device=self.device)
            xp = torch
        cos2psi, sin2psi = math.cos(2.0 * psi), math.sin(2.0 * psi)
        cosiota = math.cos(iota)
        fddot = 11.0 / 3.0 * fdot**2 / f
        phase = 2 * np.pi * (f * t + 1.0 / 2.0 * fdot * t**2 + 1.0 / 6.0 * fddot * t**3) - phi0
        hSp = -xp.cos(phase) * A * (1.0 + cosiota * cosiota)
        hSc = -xp.sin(phase) * 2.0 * A * cosiota
        hp = hSp * cos2psi - hSc * sin2psi
        hc = hSp * sin2psi + hSc * cos2psi
        if xp is np:
            return hp + 1j * hc
        return torch.complex(hp, hc)


def draw_gb_parameters(rng: np.random.Generator, n: int, f_range=(1e-4, 1e-2),
                       fdot_range=(1e-18, 1e-13), amp_range=(1e-23, 1e-21)):
    """Seeded draws of (A, f, fdot, iota, phi0, psi, lam, beta) for n sources:
    log-uniform A, f, fdot; isotropic sky and inclination; uniform phases."""
    def logu(lo, hi):
        return np.exp(rng.uniform(np.log(lo), np.log(hi), n))

    return dict(
        A=logu(*amp_range), f=logu(*f_range), fdot=logu(*fdot_range),
        iota=np.arccos(rng.uniform(-1.0, 1.0, n)), phi0=rng.uniform(0.0, 2 * np.pi, n),
        psi=rng.uniform(0.0, np.pi, n), lam=rng.uniform(0.0, 2 * np.pi, n),
        beta=np.arcsin(rng.uniform(-1.0, 1.0, n)),
    )
