"""Batch graphs (flr_batch_graph_*): a captured launch replays batches of any
lengths up to its source capacity with results bit-identical to direct runs;
outputs are written in full (no clearing needed); launches alternate staging
buffers and may move between streams."""

import numpy as np
import pytest

from test_gpu_batch import _np, _sources

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_replays_match_direct_runs(gpu_lib, precision):
    import fastlisaresponse_gb300 as flr

    dt = 10.0
    orb = flr.KeplerianOrbits(t_max=1.2e6)
    bat = flr.BatchedResponseTDI(1 / dt, order=25, tdi=["1st generation", "2nd generation"],
                                 orbits=orb, precision=precision)
    g = bat.graph(6)
    # three launches of one graph with different counts and lengths
    for seed, lengths in ((1, [2500, 70001, 9000]), (2, [4096] * 6), (3, [30000])):
        hs, lam, beta, t0 = _sources(orb, dt, lengths, seed=seed)
        sets = [i % 2 for i in range(len(lengths))]
        want = bat(hs, lam, beta, t0=t0, tdi_set=sets)
        got = g(hs, lam, beta, t0=t0, tdi_set=sets)
        for a, b in zip(got, want):
            assert np.array_equal(_np(a), _np(b))
    assert bat.status() == 0
    with pytest.raises(ValueError):
        g(hs * 7, np.repeat(lam, 7), np.repeat(beta, 7))


def test_graph_buckets_and_waveforms(gpu_lib):
    """use_graph picks the power-of-two bucket; run_gb through a graph equals
    the direct run_gb (waveforms and channels)."""
    import fastlisaresponse_gb300 as flr

    dt = 10.0
    orb = flr.EqualArmlengthOrbits(t_max=1.2e6)
    bat = flr.BatchedResponseTDI(1 / dt, tdi=["1st generation", "2nd generation"], orbits=orb,
                                 precision="mixed")
    rng = np.random.default_rng(8)
    for ns in (3, 11, 5):
        p = flr.waveforms.draw_gb_parameters(rng, ns)
        prm = np.stack([p[k] for k in ("A", "f", "fdot", "iota", "phi0", "psi")], axis=1)
        lengths = rng.integers(2100, 60000, ns)
        sets = rng.integers(0, 2, ns)
        o1, h1 = bat.run_gb(prm, lengths, p["lam"], p["beta"], tdi_set=sets)
        o2, h2 = bat.run_gb(prm, lengths, p["lam"], p["beta"], tdi_set=sets, use_graph=True)
        for a, b in zip(o1 + h1, o2 + h2):
            assert np.array_equal(_np(a), _np(b))
    assert sorted(k[0] for k in bat._graphs) == [8, 16]
    assert bat.status() == 0


@pytest.mark.parametrize("chan", ["XYZ", "AE"])
def test_outputs_written_in_full(gpu_lib, chan):
    """Edge zones and the unused AE row come out zero over NaN-filled buffers."""
    import torch

    import fastlisaresponse_gb300 as flr

    dt = 10.0
    orb = flr.EqualArmlengthOrbits(t_max=1.2e6)
    lengths = [2100, 5000, 33333]
    hs, lam, beta, t0 = _sources(orb, dt, lengths, seed=4)
    bat = flr.BatchedResponseTDI(1 / dt, orbits=orb, tdi_chan=chan, precision="fp64")
    ref = bat(hs, lam, beta, t0=t0, out=[torch.zeros((3, n), dtype=torch.float64,
                                                     device=bat.device) for n in lengths])
    nan = [torch.full((3, n), float("nan"), dtype=torch.float64, device=bat.device)
           for n in lengths]
    got = bat(hs, lam, beta, t0=t0, out=nan)
    ts = bat.tdi_start_ind
    for a, b, n in zip(got, ref, lengths):
        a, b = _np(a), _np(b)
        assert np.array_equal(a, b)
        assert not np.any(a[:, :ts]) and not np.any(a[:, n - ts:])
        if chan == "AE":
            assert not np.any(a[2])


def test_graph_launches_on_two_streams(gpu_lib):
    """Launches of one graph alternate between two streams (each waits for
    the previous launch on the device); results match direct runs."""
    import torch

    import fastlisaresponse_gb300 as flr

    dt = 10.0
    orb = flr.EqualArmlengthOrbits(t_max=1.2e6)
    bat = flr.BatchedResponseTDI(1 / dt, orbits=orb, precision="mixed")
    g = bat.graph(4)
    streams = [torch.cuda.Stream(device=bat.device) for _ in range(2)]
    cases = [_sources(orb, dt, [3000 + 997 * i, 40000 - 1000 * i], seed=20 + i) for i in range(6)]
    got = []
    for i, (hs, lam, beta, t0) in enumerate(cases):
        got.append(g(hs, lam, beta, t0=t0, stream=streams[i % 2]))
    torch.cuda.synchronize(bat.device)
    for (hs, lam, beta, t0), outs in zip(cases, got):
        want = bat(hs, lam, beta, t0=t0)
        for a, b in zip(outs, want):
            assert np.array_equal(_np(a), _np(b))
    assert bat.status() == 0
