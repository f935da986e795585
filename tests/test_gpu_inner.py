"""Inner products formed inside the fused kernel (flr_batch_source.data /
.inner; BatchedResponseTDI.inner_products): the per-source channel products
<h|d> and <h|h> equal those of the stored channels to 1e-12 relative (only the
summation order differs), repeat bit for bit, and leave the channels unstored
unless asked."""

import numpy as np
import pytest

from test_gpu_batch import _sources

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _expected(outs, data, ts):
    import torch

    rows = []
    for o, d in zip(outs, data):
        n = o.shape[1]
        sl = slice(ts, n - ts)
        hd = (o[:, sl] * d[:, sl]).sum(dim=1)
        hh = (o[:, sl] * o[:, sl]).sum(dim=1)
        rows.append(torch.stack([hd, hh]))
    return torch.stack(rows)


def _close(got, want):
    g, w = got.cpu().numpy(), want.cpu().numpy()
    scale = np.abs(w).max(axis=-1, keepdims=True) + 1e-300
    return np.abs(g - w) / scale


@pytest.mark.parametrize("precision,orbit_kind,chan", [
    ("fp64", "kepler", "XYZ"), ("mixed", "kepler", "XYZ"), ("mixed", "equal", "XYZ"),
    ("mixed", "equal", "AE"), ("fp64", "equal", "AET")])
def test_inner_products_match_stored_channels(gpu_lib, precision, orbit_kind, chan):
    import torch

    import fastlisaresponse_gb300 as flr

    dt = 10.0
    orb = flr.KeplerianOrbits(t_max=1.2e6) if orbit_kind == "kepler" else \
        flr.EqualArmlengthOrbits(t_max=1.2e6)
    lengths = [2600, 30000, 77777]
    hs, lam, beta, t0 = _sources(orb, dt, lengths, seed=31)
    bat = flr.BatchedResponseTDI(1 / dt, tdi=["1st generation", "2nd generation"], orbits=orb,
                                 tdi_chan=chan, precision=precision)
    sets = [1, 0, 1]
    outs = bat(hs, lam, beta, t0=t0, tdi_set=sets)
    g = torch.Generator(device=bat.device).manual_seed(7)
    data = [o + 1e-3 * o.abs().max() * torch.randn(o.shape, generator=g, dtype=torch.float64,
                                                   device=bat.device) for o in outs]
    inner = bat.inner_products(hs, lam, beta, data, t0=t0, tdi_set=sets)
    want = _expected(outs, data, bat.tdi_start_ind)
    assert _close(inner, want).max() <= TOL
    again = bat.inner_products(hs, lam, beta, data, t0=t0, tdi_set=sets)
    assert torch.equal(inner, again)  # fixed reduction order
    inner2, outs2 = bat.inner_products(hs, lam, beta, data, t0=t0, tdi_set=sets, write_out=True)
    assert torch.equal(inner2, inner)
    for a, b in zip(outs2, outs):
        assert torch.equal(a, b)
    assert bat.status() == 0


def test_inner_products_of_device_waveforms(gpu_lib):
    import torch

    import fastlisaresponse_gb300 as flr

    dt = 10.0
    orb = flr.EqualArmlengthOrbits(t_max=1.2e6)
    bat = flr.BatchedResponseTDI(1 / dt, tdi="2nd generation", orbits=orb, precision="mixed")
    rng = np.random.default_rng(12)
    p = flr.waveforms.draw_gb_parameters(rng, 5)
    prm = np.stack([p[k] for k in ("A", "f", "fdot", "iota", "phi0", "psi")], axis=1)
    lengths = [3000, 9000, 40000, 2500, 65536]
    outs, _ = bat.run_gb(prm, lengths, p["lam"], p["beta"])
    data = [torch.roll(o, 7, dims=1).contiguous() for o in outs]
    inner, hs = bat.inner_products_gb(prm, lengths, p["lam"], p["beta"], data)
    assert _close(inner, _expected(outs, data, bat.tdi_start_ind)).max() <= TOL
    assert [len(x) for x in hs] == lengths
    with pytest.raises(ValueError):
        bat.inner_products_gb(prm, lengths, p["lam"], p["beta"], data[:4])
    assert bat.status() == 0
