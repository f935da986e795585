"""Batched, fused response + TDI (BatchedResponseTDI) on the GPU.

fp64 precision: bit-identical to the reference fixtures and to the plain path.
mixed precision: relative L2 per TDI channel against the FP64 result below
MIXED_TOL, the bound stated for the mixed-precision form.
"""

import numpy as np
import pytest

from conftest import TableOrbits, golden_names, load_golden, rel_l2

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6


def _np(x):
    return x.detach().cpu().numpy()


@pytest.mark.parametrize("name", golden_names())
def test_batch_fp64_matches_golden(gpu_lib, name):
    import fastlisaresponse_gb300 as flr

    g = load_golden(name)
    m = g["meta"]
    bat = flr.BatchedResponseTDI(1.0 / m["dt"], order=m["order"], tdi=m["tdi"],
                                 orbits=TableOrbits(g), tdi_chan=m["tdi_chan"], precision="fp64",
                                 t_buffer=m["t_buffer"])
    (out,) = bat([g["h"]], m["lam"], m["beta"], t0=m["t0"])
    want = g["chans"]
    got = _np(out)[: want.shape[0]]
    assert np.array_equal(got, want)
    assert bat.status() == 0


def _sources(orb, dt, lengths, seed, f=None):
    import fastlisaresponse_gb300 as flr

    rng = np.random.default_rng(seed)
    p = flr.waveforms.draw_gb_parameters(rng, len(lengths))
    if f is not None:
        p["f"] = np.asarray(f, dtype=float)
    hs, t0s = [], []
    for i, n in enumerate(lengths):
        t0 = float(rng.uniform(0, 2e5))
        hs.append(flr.gb_waveform(p["A"][i], p["f"][i], p["fdot"][i], p["iota"][i], p["phi0"][i],
                                  p["psi"][i], t0 + np.arange(n) * dt))
        t0s.append(t0)
    return hs, p["lam"], p["beta"], np.asarray(t0s)


def test_batch_fp64_many_sources_match_plain(gpu_lib):
    """Uneven lengths (one to several tiles), different start times and TDI
    sets in one launch; each equals the single-source plain path bit for bit."""
    import fastlisaresponse_gb300 as flr

    dt = 10.0
    lengths = [2500, 4096, 9000, 20000, 70001]
    orb = flr.KeplerianOrbits(t_max=1.2e6)
    hs, lam, beta, t0 = _sources(orb, dt, lengths, seed=7)
    sets = [0, 1, 0, 1, 1]
    bat = flr.BatchedResponseTDI(1 / dt, order=25, tdi=["1st generation", "2nd generation"],
                                 orbits=orb, precision="fp64")
    outs = bat(hs, lam, beta, t0=t0, tdi_set=sets)
    assert bat.status() == 0
    for i, n in enumerate(lengths):
        gen = ["1st generation", "2nd generation"][sets[i]]
        r = flr.pyResponseTDI(1 / dt, n, order=25, tdi=gen, orbits=orb)
        r.get_projections(hs[i], lam[i], beta[i], t0=t0[i], t_buffer=1e4)
        X, Y, Z = r.get_tdi_delays()
        want = np.stack([_np(X), _np(Y), _np(Z)])
        assert np.array_equal(_np(outs[i]), want), f"source {i}"


@pytest.mark.parametrize("order", [25, 45])
@pytest.mark.parametrize("gen", ["1st generation", "2nd generation"])
def test_batch_mixed_accuracy(gpu_lib, order, gen):
    """Mixed precision against FP64 over 1e-4..1e-2 Hz, flexing orbits."""
    import fastlisaresponse_gb300 as flr

    dt = 10.0
    f = [1e-4, 3e-4, 1e-3, 3e-3, 1e-2]
    lengths = [40000] * len(f)
    orb = flr.KeplerianOrbits(t_max=8e5)
    hs, lam, beta, t0 = _sources(orb, dt, lengths, seed=11, f=f)
    tb = 1e4 if order <= 25 else 2e4  # order 45 needs the longer garbage margin
    ref = flr.BatchedResponseTDI(1 / dt, order=order, tdi=gen, orbits=orb, precision="fp64",
                                 t_buffer=tb)
    mix = flr.BatchedResponseTDI(1 / dt, order=order, tdi=gen, orbits=orb, precision="mixed",
                                 t_buffer=tb)
    want = [_np(o) for o in ref(hs, lam, beta, t0=t0)]
    got = [_np(o) for o in mix(hs, lam, beta, t0=t0)]
    assert mix.status() == 0
    worst = 0.0
    for i in range(len(f)):
        for c in range(3):
            err = rel_l2(got[i][c], want[i][c])
            worst = max(worst, err)
            assert err <= MIXED_TOL, f"f={f[i]} channel {c}: rel L2 {err:.3e}"
    print(f"order {order} {gen}: worst rel L2 {worst:.3e}")
