"""The serving loop on the GPU: every result is identical, bit for bit, when
its request runs alone and when it runs mixed with others (continuous
batching over two streams), equals a direct batched evaluation, and stays
within 1e-6 relative L2 of the FP64 evaluation of the same device waveform."""

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _requests(rng, count):
    import fastlisaresponse_gb300 as flr

    p = flr.waveforms.draw_gb_parameters(rng, count)
    lengths = np.exp(rng.uniform(np.log(2**14), np.log(2**16), count)).astype(int)
    params = [(p["A"][i], p["f"][i], p["fdot"][i], p["iota"][i], p["phi0"][i], p["psi"][i],
               p["lam"][i], p["beta"][i]) for i in range(count)]
    return params, lengths, [i % 2 for i in range(count)]


def test_same_result_alone_and_in_the_mix(gpu_lib):
    import fastlisaresponse_gb300 as flr

    dt = 10.0
    orb = flr.KeplerianOrbits(t_max=8e5)
    params, lengths, sets = _requests(np.random.default_rng(21), 24)
    with flr.ResponseServer(1 / dt, orbits=orb, num_streams=2) as srv:
        mixed = [srv.submit(p, n, s) for p, n, s in zip(params, lengths, sets)]
        mix_out = [r.result(timeout=120).cpu().numpy() for r in mixed]
        alone_out = []
        for p, n, s in zip(params, lengths, sets):
            alone_out.append(srv.submit(p, n, s).result(timeout=120).cpu().numpy())
    assert srv.batches >= 2
    for a, b in zip(mix_out, alone_out):
        assert np.array_equal(a, b)

    direct = flr.BatchedResponseTDI(1 / dt, tdi=["1st generation", "2nd generation"],
                                    orbits=orb, precision="mixed")
    exact = flr.BatchedResponseTDI(1 / dt, tdi=["1st generation", "2nd generation"],
                                   orbits=orb, precision="fp64")
    prm = np.asarray([p[:6] for p in params])
    lam = [p[6] for p in params]
    beta = [p[7] for p in params]
    outs, hs = direct.run_gb(prm, lengths, lam, beta, tdi_set=sets)
    ref = exact(hs, lam, beta, tdi_set=sets)
    for i in range(len(params)):
        got = outs[i].cpu().numpy()
        assert np.array_equal(got, mix_out[i])
        want = ref[i].cpu().numpy()
        for c in range(3):
            assert rel_l2(got[c], want[c]) <= 1e-6


def test_device_waveform_matches_host_generator(gpu_lib):
    """Both device models against their host generators: the configurations'
    binary (waveforms.gb_waveform) and the reference tests' GBWave."""
    import fastlisaresponse_gb300 as flr

    dt = 10.0
    orb = flr.EqualArmlengthOrbits(t_max=5e5)
    bat = flr.BatchedResponseTDI(1 / dt, orbits=orb, precision="mixed")
    prm = np.array([[1e-22, 2e-3, 1e-14, 0.4, 1.2, 0.7], [3e-23, 1e-4, 1e-18, 2.0, 5.0, 2.9]])
    n = [20000, 30000]
    t0 = [0.0, 12345.0]
    _, hs = bat.run_gb(prm, n, [1.0, 2.0], [0.3, -0.4], t0=t0)
    for i in range(2):
        host = flr.gb_waveform(*prm[i], t0[i] + np.arange(n[i]) * dt)
        dev = hs[i].cpu().numpy()
        assert np.max(np.abs(dev - host)) <= 1e-12 * np.max(np.abs(host))
    # the reference tests' generator (t from 0, as GBWave's arange)
    _, hs = bat.run_gb(prm, n, [1.0, 2.0], [0.3, -0.4], model="gbwave")
    for i in range(2):
        host = flr.GBWave()(*prm[i], T=n[i] * dt / flr.waveforms.YRSID_SI, dt=dt)[:n[i]]
        dev = hs[i].cpu().numpy()
        assert np.max(np.abs(dev - host)) <= 1e-12 * np.max(np.abs(host))


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("model", ["config", "gbwave"])
def test_waveforms_generated_in_the_kernel(gpu_lib, precision, model):
    """keep_waveforms=False generates each waveform straight into the fused
    kernel's staged window (nothing written to memory): the same bits as the
    run that stores the waveforms first, directly and through a graph."""
    import torch

    import fastlisaresponse_gb300 as flr

    dt = 10.0
    orb = flr.EqualArmlengthOrbits(t_max=1.3e6)
    bat = flr.BatchedResponseTDI(1 / dt, tdi="2nd generation", orbits=orb, precision=precision)
    rng = np.random.default_rng(9)
    p = flr.waveforms.draw_gb_parameters(rng, 5)
    prm = np.stack([p[k] for k in ("A", "f", "fdot", "iota", "phi0", "psi")], axis=1)
    n = [4000, 31000, 2**16 + 7, 9000, 100001]
    t0 = [0.0, 1000.0, 0.0, 2.5e4, 0.0]
    kw = dict(t0=t0, tdi_set=0, model=model)
    want, hs = bat.run_gb(prm, n, p["lam"], p["beta"], **kw)
    got, none = bat.run_gb(prm, n, p["lam"], p["beta"], keep_waveforms=False, **kw)
    assert none is None
    for a, b in zip(got, want):
        assert torch.equal(a, b)
    got, _ = bat.run_gb(prm, n, p["lam"], p["beta"], keep_waveforms=False, use_graph=True, **kw)
    for a, b in zip(got, want):
        assert torch.equal(a, b)
    assert bat.status() == 0