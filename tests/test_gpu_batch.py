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
# link streams of the mixed flavour (no TDI cancellation yet): the
# double-float form (AET / AE outputs) gives ~1e-13, the difference forms (XYZ
# outputs) ~2e-10; the channel bound is MIXED_TOL
LINK_TOL = 5e-12
LINK_TOL_DIFF = 5e-9


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


@pytest.mark.parametrize("orbit_kind", ["kepler", "equal"])
@pytest.mark.parametrize("order", [25, 45])
@pytest.mark.parametrize("gen", ["1st generation", "2nd generation"])
def test_batch_mixed_accuracy(gpu_lib, order, gen, orbit_kind):
    """Mixed precision against FP64 over 1e-4..1e-2 Hz; flexing orbits (per-unit
    TDI) and equal-arm orbits (TDI units in equal-delay groups)."""
    import fastlisaresponse_gb300 as flr

    dt = 10.0
    f = [1e-4, 3e-4, 1e-3, 3e-3, 1e-2]
    lengths = [40000] * len(f)
    orb = flr.KeplerianOrbits(t_max=8e5) if orbit_kind == "kepler" else \
        flr.EqualArmlengthOrbits(t_max=8e5)
    hs, lam, beta, t0 = _sources(orb, dt, lengths, seed=11, f=f)
    tb = 1e4 if order <= 25 else 2e4  # order 45 needs the longer garbage margin
    ref = flr.BatchedResponseTDI(1 / dt, order=order, tdi=gen, orbits=orb, precision="fp64",
                                 t_buffer=tb)
    mix = flr.BatchedResponseTDI(1 / dt, order=order, tdi=gen, orbits=orb, precision="mixed",
                                 t_buffer=tb)
    assert mix.plan_info["grouped"] == (orbit_kind == "equal")
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


@pytest.mark.parametrize("orbit_kind", ["equal", "kepler"])
@pytest.mark.parametrize("precision,chan", [("fp64", "XYZ"), ("mixed", "XYZ"), ("mixed", "AET")])
def test_batch_indices_and_links_match_plain(gpu_lib, orbit_kind, precision, chan):
    """The integer delays the fused kernel uses (receiver, emitter, every TDI
    unit) equal the plain path's bit for bit, in both flavours and both mixed
    forms; the fp64 link streams equal the plain y_gw bit for bit, the mixed
    ones within LINK_TOL (double-float form, AET) or LINK_TOL_DIFF
    (difference forms, XYZ) per link."""
    import torch

    import fastlisaresponse_gb300 as flr

    dt = 10.0
    lengths = [6000, 23000]
    orb = flr.EqualArmlengthOrbits(t_max=4e5) if orbit_kind == "equal" else \
        flr.KeplerianOrbits(t_max=4e5)
    hs, lam, beta, t0 = _sources(orb, dt, lengths, seed=5)
    bat = flr.BatchedResponseTDI(1 / dt, order=25, tdi="2nd generation", orbits=orb,
                                 precision=precision, tdi_chan=chan)
    outs, diags = bat(hs, lam, beta, t0=t0, diagnostics=True)
    ts = bat.tdi_start_ind
    tol = LINK_TOL_DIFF if (precision, chan) == ("mixed", "XYZ") else LINK_TOL
    for i, n in enumerate(lengths):
        r = flr.pyResponseTDI(1 / dt, n, order=25, tdi="2nd generation", orbits=orb)
        r.get_projections(hs[i], lam[i], beta[i], t0=t0[i], t_buffer=1e4)
        dev = r.device
        tt = torch.as_tensor(t0[i] + np.arange(n) * r.dt, device=dev)
        k, _, _ = flr.sky_basis(lam[i], beta[i])
        d_rec = torch.zeros(6 * n, dtype=torch.int32, device=dev)
        d_em = torch.zeros_like(d_rec)
        r.cpp_response.response_delay_indices(d_rec, d_em, tt, torch.as_tensor(k, device=dev), n,
                                              1 / dt, r.projections_start_ind)
        d_tdi = torch.zeros(r.num_units * n, dtype=torch.int32, device=dev)
        r.cpp_response.tdi_delay_indices(d_tdi, n, tt, r.unit_starts, r.unit_lengths,
                                         r.tdi_link_combinations, r.num_units, 1 / dt, ts)
        sl = slice(ts, n - ts)
        dg = diags[i]
        assert np.array_equal(_np(dg["d_rec"])[:, sl], _np(d_rec).reshape(6, n)[:, sl])
        assert np.array_equal(_np(dg["d_em"])[:, sl], _np(d_em).reshape(6, n)[:, sl])
        assert np.array_equal(_np(dg["d_tdi"])[:, sl], _np(d_tdi).reshape(r.num_units, n)[:, sl])
        y_plain = _np(r.y_gw)[:, sl]
        y_fused = _np(dg["y"])[:, sl]
        if precision == "fp64":
            assert np.array_equal(y_fused, y_plain)
        else:
            for link in range(6):
                err = rel_l2(y_fused[link], y_plain[link])
                assert err <= tol, f"source {i} link {link}: rel L2 {err:.2e}"


@pytest.mark.parametrize("chan", ["AET", "AE"])
def test_batch_mixed_grouped_channels_and_sets(gpu_lib, chan):
    """Equal-arm orbits, two TDI sets in one launch, AET / AE outputs: the
    grouped mixed path against FP64 per channel."""
    import fastlisaresponse_gb300 as flr

    dt = 10.0
    orb = flr.EqualArmlengthOrbits(t_max=1.2e6)
    lengths = [3000, 30000, 77777, 12000]
    hs, lam, beta, t0 = _sources(orb, dt, lengths, seed=13)
    sets = [0, 1, 1, 0]
    kw = dict(order=25, tdi=["1st generation", "2nd generation"], orbits=orb, tdi_chan=chan)
    ref = flr.BatchedResponseTDI(1 / dt, precision="fp64", **kw)
    mix = flr.BatchedResponseTDI(1 / dt, precision="mixed", **kw)
    assert mix.plan_info["grouped"] == 1
    want = [_np(o) for o in ref(hs, lam, beta, t0=t0, tdi_set=sets)]
    got = [_np(o) for o in mix(hs, lam, beta, t0=t0, tdi_set=sets)]
    assert mix.status() == 0
    for i in range(len(lengths)):
        for c in range(2):
            assert rel_l2(got[i][c], want[i][c]) <= MIXED_TOL
        if chan == "AE":
            assert not np.any(got[i][2])


@pytest.mark.parametrize("orbit_kind", ["equal", "kepler"])
def test_batch_mixed_bits_do_not_depend_on_the_tile(gpu_lib, orbit_kind):
    """Every output sample of the mixed kernel is a function of its own
    source and time alone: the per-item input scale is a power of two, the
    differences are formed from the same samples, and the equal-delay
    groups' tabulated weights equal the computed ones.  So tiles of 128, 512
    and 1024 samples give the same bits."""
    import fastlisaresponse_gb300 as flr

    dt = 10.0
    orb = flr.EqualArmlengthOrbits(t_max=2e6) if orbit_kind == "equal" else \
        flr.KeplerianOrbits(t_max=2e6)
    lengths = [3000, 41000, 123457, 9000]
    hs, lam, beta, t0 = _sources(orb, dt, lengths, seed=61,
                                 f=[3e-3, 1e-4, 2e-3, 8e-3])
    outs = {}
    for tile in (128, 512, 1024):
        bat = flr.BatchedResponseTDI(1 / dt, tdi="2nd generation", orbits=orb, precision="mixed",
                                     tile=tile)
        outs[tile] = [_np(o) for o in bat(hs, lam, beta, t0=t0)]
        assert bat.status() == 0
    for tile in (128, 1024):
        for a, b in zip(outs[tile], outs[512]):
            assert np.array_equal(a, b), f"tile {tile}"


@pytest.mark.parametrize("orbit_kind", ["equal", "kepler"])
def test_t0_zero_instance_matches_general(gpu_lib, orbit_kind):
    """Sources that all start at t0 = +0 take the fused kernel's instance
    without the t0 operations; the same sources beside one with t0 != 0 (or
    with t0 = -0) take the general instance: the same bits, in direct runs and
    in graph replays."""
    import fastlisaresponse_gb300 as flr

    dt = 10.0
    orb = flr.EqualArmlengthOrbits(t_max=1.2e6) if orbit_kind == "equal" else \
        flr.KeplerianOrbits(t_max=1.2e6)
    bat = flr.BatchedResponseTDI(1 / dt, order=25, tdi=["1st generation", "2nd generation"],
                                 orbits=orb, precision="mixed")
    hs, lam, beta, _ = _sources(orb, dt, [2500, 9000, 40000, 70001, 30000], seed=11)
    sets = [0, 1, 1, 0, 1]
    zero = np.zeros(4)
    alone = [_np(o) for o in bat(hs[:4], lam[:4], beta[:4], t0=zero, tdi_set=sets[:4])]
    beside = bat(hs, lam, beta, t0=np.append(zero, 5e3), tdi_set=sets)
    negzero = bat(hs[:4], lam[:4], beta[:4], t0=np.full(4, -0.0), tdi_set=sets[:4])
    for a, b, c in zip(alone, beside, negzero):
        assert np.array_equal(a, _np(b)) and np.array_equal(a, _np(c))
    g = bat.graph(8)
    via_graph = g(hs[:4], lam[:4], beta[:4], t0=zero, tdi_set=sets[:4])
    via_graph_beside = g(hs, lam, beta, t0=np.append(zero, 5e3), tdi_set=sets)
    for a, b, c in zip(alone, via_graph, via_graph_beside):
        assert np.array_equal(a, _np(b)) and np.array_equal(a, _np(c))
    assert bat.status() == 0
