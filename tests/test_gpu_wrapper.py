"""ResponseWrapper(precision=...): the fused kernel behind the reference's
wrapper API.  "fp64" gives the default path's bits; "mixed" (also chunked)
stays within the channel bound; channel counts and garbage handling match."""

import numpy as np
import pytest

from conftest import rel_l2
from test_gpu_batch import MIXED_TOL

pytestmark = pytest.mark.gpu


def _np(x):
    return x.detach().cpu().numpy()


@pytest.mark.parametrize("tdi_chan,remove_garbage", [("AET", True), ("XYZ", "zero"),
                                                     ("AE", False)])
def test_wrapper_fused_precisions(gpu_lib, tdi_chan, remove_garbage):
    import fastlisaresponse_gb300 as flr

    dt = 10.0
    n = 30000
    T = n * dt / flr.orbits.YRSID_SI
    orb = flr.KeplerianOrbits(t_max=(n * dt // 1e4 + 3) * 1e4)
    params = (1.084702251e-22, 2.35962078e-3, 1.47197271e-17, 1.11820901, 4.91128699, 2.3290324)
    lam, beta = 5.22979888, 0.9805742971871619
    h_host = flr.GBWave()(*params, T=T, dt=dt)[:n]

    def wave(*args, T=1.0, dt=10.0):
        return h_host

    kw = dict(t_buffer=1e4, remove_sky_coords=True, remove_garbage=remove_garbage, n_overide=n,
              orbits=orb, order=25, tdi="2nd generation", tdi_chan=tdi_chan, t0=3e3)
    base = [_np(c) for c in flr.ResponseWrapper(wave, T, dt, 6, 7, **kw)(*params, lam, beta)]
    same = [_np(c) for c in flr.ResponseWrapper(wave, T, dt, 6, 7, precision="fp64",
                                                **kw)(*params, lam, beta)]
    assert len(same) == len(base) == (2 if tdi_chan == "AE" else 3)
    for a, b in zip(same, base):
        assert np.array_equal(a, b)
    for chunks in (1, 4):
        mixed = [_np(c) for c in flr.ResponseWrapper(wave, T, dt, 6, 7, precision="mixed",
                                                     chunks=chunks, **kw)(*params, lam, beta)]
        for a, b in zip(mixed, base):
            assert a.shape == b.shape
            assert rel_l2(a, b) <= MIXED_TOL
