"""Generate the golden fixtures in this folder from the reference's own code.

Run where the reference checkout exists (FLR_REFERENCE_ROOT, or the location
``oracle/Makefile`` names):

    python tests/golden/make_golden.py

Each case builds orbit tables and an input waveform, then runs the
reference's ``pyResponseTDI`` (``src/fastlisaresponse/response.py``, imported
from source) whose native calls go to the reference's ``LISAResponse.cu`` CPU
branch compiled by ``make -C oracle ref``; see ``oracle/refdrive.py`` for the
stand-ins of the absent third-party modules.  Inputs, the reference's host
tables and its outputs are stored in ``<case>.npz``; ``tests/test_oracle.py``
and the GPU parity tests compare against them.  Inputs are stored explicitly
(not regenerated) so the fixtures do not depend on the host's libm.
"""

from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.normpath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "lisa-on-gpu_gb300"))

import refdrive  # noqa: E402
from fastlisaresponse_gb300 import orbits as orbit_models  # noqa: E402
from fastlisaresponse_gb300 import waveforms  # noqa: E402

CUSTOM_TDI = [  # a user-supplied combination list (response.py:58-66 format)
    {"link": 12, "links_for_delay": [21, 13], "sign": 1},
    {"link": 23, "links_for_delay": [], "sign": -1},
    {"link": 31, "links_for_delay": [13, 32, 23], "sign": 1},
]

CASES = {
    # name: (orbits, dt, n, order, tdi, tdi_chan, t0, waveform parameters, lam, beta)
    "rigid_gen1_o25": dict(orbits="equal", dt=10.0, n=4096, order=25, tdi="1st generation",
                           chan="XYZ", t0=0.0, wave=("config", 1e-22, 2e-3, 1e-14, 0.7, 1.1, 0.4),
                           lam=1.3, beta=0.45),
    "flex_gen2_o25_dt5": dict(orbits="kepler", dt=5.0, n=6144, order=25, tdi="2nd generation",
                              chan="XYZ", t0=0.0,
                              wave=("config", 2e-22, 5e-3, 3e-14, 2.1, 0.2, 1.9),
                              lam=4.2, beta=-0.8),
    "flex_gen1_o11_aet_t0": dict(orbits="kepler", dt=10.0, n=4096, order=11,
                                 tdi="1st generation", chan="AET", t0=1.2345e6,
                                 wave=("reftest", 1.084702251e-22, 2.35962078e-3,
                                       1.47197271e-17, 1.11820901, 4.91128699, 2.3290324),
                                 lam=5.22979888, beta=0.9805742971871619),
    "flex_custom_o31": dict(orbits="kepler", dt=10.0, n=4096, order=31, tdi=CUSTOM_TDI,
                            chan="XYZ", t0=3.0e5,
                            wave=("config", 1e-21, 8e-3, 1e-15, 0.1, 3.0, 2.6), lam=0.2,
                            beta=1.3),
    "rigid_gen2_lowf_o25": dict(orbits="equal", dt=10.0, n=4096, order=25,
                                tdi="2nd generation", chan="AE", t0=0.0,
                                wave=("config", 1e-23, 1e-4, 1e-18, 1.4, 0.6, 0.3), lam=2.9,
                                beta=-0.1),
    # the highest order the reference's factorial table supports (39!)
    "flex_gen2_o39": dict(orbits="kepler", dt=10.0, n=4096, order=39, tdi="2nd generation",
                          chan="XYZ", t0=5.0e4,
                          wave=("config", 3e-22, 1e-3, 1e-15, 0.9, 2.2, 1.0), lam=3.3,
                          beta=0.2),
}


def make_orbits(kind: str, t_end: float):
    t_max = (np.floor(t_end / 1e4) + 3) * 1e4
    if kind == "equal":
        return orbit_models.EqualArmlengthOrbits(t_max=t_max)
    return orbit_models.KeplerianOrbits(t_max=t_max)


def make_wave(spec, n, dt, t0):
    kind, *p = spec
    if kind == "config":
        return waveforms.gb_waveform(*p, t0 + np.arange(n) * dt)
    return waveforms.GBWave()(*p, T=n * dt / waveforms.YRSID_SI, dt=dt)[:n]


def run_case(name: str, c: dict) -> dict:
    ref = refdrive.import_reference_response()
    orb = make_orbits(c["orbits"], c["t0"] + c["n"] * c["dt"])
    stub = refdrive.StubOrbits(orb)
    resp = ref.pyResponseTDI(1.0 / c["dt"], c["n"], order=c["order"], tdi=c["tdi"], orbits=stub,
                             tdi_chan=c["chan"])
    h = np.ascontiguousarray(make_wave(c["wave"], c["n"], c["dt"], c["t0"]), dtype=np.complex128)
    assert h.shape == (c["n"],)
    resp.get_projections(h, c["lam"], c["beta"], t0=c["t0"], t_buffer=1e4)
    chans = resp.get_tdi_delays()
    args = orb.pycppdetector_args
    return dict(
        meta=json.dumps(dict(name=name, dt=c["dt"], n=c["n"], order=c["order"], tdi=c["tdi"],
                             tdi_chan=c["chan"], t0=c["t0"], lam=c["lam"], beta=c["beta"],
                             orbits=c["orbits"], t_buffer=1e4)),
        orb_dt=np.float64(args[0]), orb_N=np.int64(args[1]), orb_n=args[2], orb_ltt=args[3],
        orb_x=args[4], orb_links=args[5], orb_sc_r=args[6], orb_sc_e=args[7],
        orb_armlength=np.float64(args[8]), x_base=orb.x_base,
        h=h, A_in=resp.A_in, E_in=resp.E_in, deps=np.float64(resp.deps),
        tdi_base_links=resp.tdi_base_links, tdi_link_combinations=resp.tdi_link_combinations,
        tdi_signs=resp.tdi_signs, channels=resp.channels,
        tdi_operation_index=resp.tdi_operation_index,
        tdi_start_ind=np.int64(resp.tdi_start_ind),
        projections_start_ind=np.int64(resp.projections_start_ind),
        y_gw=resp.y_gw_flat.reshape(6, -1), XYZ=resp.XYZ.copy(),
        chans=np.stack(chans),
    )


def main(names=None):
    """Write every case, or only the named ones (python make_golden.py NAME ...)."""
    for name, c in CASES.items():
        if names and name not in names:
            continue
        out = run_case(name, c)
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **out)
        print(f"{path}: y_gw max {np.abs(out['y_gw']).max():.3e}, "
              f"XYZ max {np.abs(out['XYZ']).max():.3e}, {os.path.getsize(path) / 1e3:.0f} kB")


if __name__ == "__main__":
    main(sys.argv[1:])
