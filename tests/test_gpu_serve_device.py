"""Device-resident serving (DeviceLoopServer, flr_server_*): requests
submitted while the persistent kernel runs, and after it has left on its
idle timeout, give the bits of a batched run of the same requests."""

import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests(rng, count, n_lo, n_hi, sets):
    import fastlisaresponse_gb300 as flr

    p = flr.waveforms.draw_gb_parameters(rng, count)
    reqs = []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi))))
        prm = (p["A"][i], p["f"][i], p["fdot"][i], p["iota"][i], p["phi0"][i], p["psi"][i],
               p["lam"][i], p["beta"][i])
        reqs.append(dict(params=prm, n=n, tdi_set=int(rng.integers(sets)),
                         t0=float(rng.choice([0.0, 5e3])),
                         model=("config", "gbwave")[i % 2]))
    return reqs


def _batched(srv, reqs):
    """The same requests through the batch path of the server's own plan."""
    import fastlisaresponse_gb300 as flr

    want = []
    for model in ("config", "gbwave"):
        sel = [r for r in reqs if r["model"] == model]
        if not sel:
            continue
        prm = np.asarray([r["params"][:6] for r in sel])
        outs, _ = srv.plan.run_gb(prm, [r["n"] for r in sel], [r["params"][6] for r in sel],
                                  [r["params"][7] for r in sel], t0=[r["t0"] for r in sel],
                                  tdi_set=[r["tdi_set"] for r in sel], model=model,
                                  keep_waveforms=False)
        want += list(zip(sel, outs))
    return {id(r): o for r, o in want}


@pytest.mark.parametrize("orbit_kind,chan", [("equal", "XYZ"), ("kepler", "XYZ"),
                                             ("equal", "AET")])
def test_device_loop_matches_batch(gpu_lib, orbit_kind, chan):
    import torch

    import fastlisaresponse_gb300 as flr

    dt = 10.0
    t_max = 3e6
    orb = flr.EqualArmlengthOrbits(t_max=t_max) if orbit_kind == "equal" else \
        flr.KeplerianOrbits(t_max=t_max)
    rng = np.random.default_rng(71)
    reqs = _requests(rng, 24, 2**12, 2**17, 2)
    with flr.DeviceLoopServer(1 / dt, orbits=orb, tdi_chan=chan, capacity=256,
                              idle_seconds=0.05) as srv:
        tickets = [srv.submit(r["params"], r["n"], r["tdi_set"], r["t0"], r["model"])
                   for r in reqs]
        got = [t.result(timeout=60) for t in tickets]
        assert all(t.latency is not None for t in tickets)
        # the kernel leaves after its idle time; later requests relaunch it
        time.sleep(0.3)
        assert srv.info()["launches"] >= 1
        more = _requests(rng, 6, 2**12, 2**15, 2)
        tickets2 = [srv.submit(r["params"], r["n"], r["tdi_set"], r["t0"], r["model"])
                    for r in more]
        got2 = [t.result(timeout=60) for t in tickets2]
        info = srv.info()
        assert info["launches"] >= 2 and info["submitted"] == 30 and info["first_open"] == 30
        torch.cuda.synchronize()
        want = _batched(srv, reqs + more)
        for r, g in zip(reqs + more, got + got2):
            assert torch.equal(g, want[id(r)]), (r["n"], r["model"])
        assert srv.status() == 0


def test_device_loop_stored_waveforms(gpu_lib):
    """Requests with a stored waveform (h) beside generated ones: the bits of
    a batch run of the same waveforms."""
    import torch

    import fastlisaresponse_gb300 as flr

    dt = 10.0
    orb = flr.KeplerianOrbits(t_max=2e6)
    rng = np.random.default_rng(83)
    reqs = _requests(rng, 6, 2**13, 2**16, 2)
    with flr.DeviceLoopServer(1 / dt, orbits=orb, capacity=16, idle_seconds=0.05) as srv:
        hs, tickets = [], []
        for r in reqs:
            t = r["t0"] + torch.arange(r["n"], dtype=torch.float64, device=srv.device) * dt
            hs.append(flr.gb_waveform(*r["params"][:6], t))
            tickets.append(srv.submit(r["params"], r["n"], r["tdi_set"], r["t0"], h=hs[-1]))
        got = [t.result(timeout=60) for t in tickets]
        want = srv.plan(hs, [r["params"][6] for r in reqs], [r["params"][7] for r in reqs],
                        t0=[r["t0"] for r in reqs], tdi_set=[r["tdi_set"] for r in reqs])
        torch.cuda.synchronize()
        for g, w in zip(got, want):
            assert torch.equal(g, w)
        with pytest.raises(ValueError, match="complex128"):
            srv.submit(reqs[0]["params"], reqs[0]["n"] + 1, h=hs[0])
        assert srv.status() == 0


def test_device_loop_rejects_bad_requests(gpu_lib):
    import fastlisaresponse_gb300 as flr

    with flr.DeviceLoopServer(0.1, orbits=flr.EqualArmlengthOrbits(t_max=1e6), capacity=2,
                              idle_seconds=0.01) as srv:
        prm = (1e-22, 2e-3, 1e-14, 0.3, 0.1, 0.2, 1.0, 0.5)
        with pytest.raises(ValueError, match="tdi_start < n/2"):
            srv.submit(prm, 1000, tdi_set=0)  # shorter than both edge zones
        with pytest.raises(ValueError, match="tdi_set"):
            srv.submit(prm, 30000, tdi_set=5)  # no such TDI set
        a = srv.submit(prm, 30000)
        b = srv.submit(prm, 30000, tdi_set=1)
        with pytest.raises(ValueError, match="full"):
            srv.submit(prm, 30000)
        a.result(timeout=30)
        b.result(timeout=30)
