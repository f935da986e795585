"""The batched kernel's bounded wait for a work item's staging copy.

Each work item stages its input window with one bulk copy and waits for it on
an mbarrier with a bounded number of polls.  These tests make that first wait
give up (its bound set to 0 polls through the plan's test hook) without any
stalled copy: a second wait with the full bound lets the copy land, the item's
outputs must become NaN, the status word must carry FLR_STATUS_STAGING (0x10)
and not FLR_STATUS_STAGING_LOST (0x20), the kernel must return normally, and
the next run with the default bound must give the bits of a normal run.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STAGING, STAGING_LOST = 0x10, 0x20


def _batch(precision, tdi_chan="XYZ"):
    import torch

    import fastlisaresponse_gb300 as flr

    dt = 10.0
    lengths = [2**14, 5000, 3 * 2**12 + 17]
    rng = np.random.default_rng(11)
    p = flr.waveforms.draw_gb_parameters(rng, len(lengths))
    hs = [flr.gb_waveform(p["A"][i], p["f"][i], p["fdot"][i], p["iota"][i], p["phi0"][i],
                          p["psi"][i], torch.arange(n, dtype=torch.float64, device="cuda") * dt)
          for i, n in enumerate(lengths)]
    orb = flr.EqualArmlengthOrbits(t_max=(max(lengths) * dt // 1e4 + 3) * 1e4)
    bat = flr.BatchedResponseTDI(1 / dt, order=25, tdi="2nd generation", orbits=orb,
                                 precision=precision, tdi_chan=tdi_chan)
    return bat, hs, p["lam"], p["beta"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_first_wait_gives_up_cleanly(gpu_lib, precision):
    import torch

    bat, hs, lam, beta = _batch(precision)
    want = [o.clone() for o in bat(hs, lam, beta)]
    assert bat.status(reset=True) == 0

    bat._set_wait_limit(0)
    got = bat(hs, lam, beta)
    torch.cuda.synchronize()
    bits = bat.status(reset=True)
    assert bits & STAGING and not bits & STAGING_LOST, hex(bits)
    ts = bat.tdi_start_ind
    for o in got:
        n = o.shape[1]
        assert torch.isnan(o[:, ts:n - ts]).all()  # every item gave up: NaN, not stale data
        assert (o[:, :ts] == 0).all() and (o[:, n - ts:] == 0).all()  # edge zones still written

    bat._set_wait_limit(-1)
    again = bat(hs, lam, beta)
    assert bat.status(reset=True) == 0
    for a, b in zip(again, want):
        assert torch.equal(a, b)


def test_first_wait_gives_up_in_inner_products(gpu_lib):
    """The inner-product instance: a tile that gave up contributes NaN."""
    import torch

    bat, hs, lam, beta = _batch("mixed", tdi_chan="AE")
    data = [o.clone() for o in bat(hs, lam, beta)]
    ok = bat.inner_products(hs, lam, beta, data)
    assert bat.status(reset=True) == 0 and torch.isfinite(ok).all()
    bat._set_wait_limit(0)
    bad = bat.inner_products(hs, lam, beta, data)
    bits = bat.status(reset=True)
    assert bits & STAGING and not bits & STAGING_LOST
    assert torch.isnan(bad).all()
    bat._set_wait_limit(-1)
    assert torch.equal(bat.inner_products(hs, lam, beta, data), ok)
    assert bat.status() == 0
