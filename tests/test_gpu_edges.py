"""Edge cases of the batched path: an empty batch, a source with a single
output sample, the largest supported Lagrange order (79), and a batch that
mixes all of these with ordinary sources."""

import numpy as np
import pytest

from conftest import rel_l2
from test_gpu_batch import MIXED_TOL, _np, _sources

pytestmark = pytest.mark.gpu


def test_empty_batch(gpu_lib):
    import fastlisaresponse_gb300 as flr

    bat = flr.BatchedResponseTDI(0.1, orbits=flr.EqualArmlengthOrbits(t_max=4e5),
                                 precision="mixed")
    assert bat([], [], []) == []
    assert bat.run_gb(np.zeros((0, 6)), [], [], [])[0] == []
    assert bat.status() == 0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_single_output_sample_and_ragged_batch(gpu_lib, precision):
    """n = 2 ts + 1: one computed sample, the rest edge zeros; batched with
    long sources, each equal to its own plain-path (fp64) or fp64-batch
    (mixed) result."""
    import fastlisaresponse_gb300 as flr

    dt = 10.0
    orb = flr.KeplerianOrbits(t_max=1.2e6)
    ts = int(1e4 / dt)
    lengths = [2 * ts + 1, 50001, 2 * ts + 2, 7000]
    hs, lam, beta, t0 = _sources(orb, dt, lengths, seed=61)
    bat = flr.BatchedResponseTDI(1 / dt, tdi="2nd generation", orbits=orb, precision=precision)
    outs = [_np(o) for o in bat(hs, lam, beta, t0=t0)]
    assert bat.status() == 0
    ref = flr.BatchedResponseTDI(1 / dt, tdi="2nd generation", orbits=orb, precision="fp64")
    for i, n in enumerate(lengths):
        one = _np(ref([hs[i]], lam[i], beta[i], t0=t0[i])[0])
        assert not np.any(outs[i][:, :ts]) and not np.any(outs[i][:, n - ts:])
        if precision == "fp64":
            assert np.array_equal(outs[i], one)
        else:
            for c in range(3):
                assert rel_l2(outs[i][c], one[c]) <= MIXED_TOL
    if precision == "fp64":  # the plain path agrees on the single computed sample
        r = flr.pyResponseTDI(1 / dt, lengths[0], order=25, tdi="2nd generation", orbits=orb)
        r.get_projections(hs[0], lam[0], beta[0], t0=t0[0], t_buffer=1e4)
        X, Y, Z = r.get_tdi_delays()
        assert np.array_equal(outs[0], np.stack([_np(X), _np(Y), _np(Z)]))


def test_largest_order(gpu_lib):
    """Order 79 (h = 40, the kernel's limit): the fp64 batch equals the plain
    path bit for bit and the mixed one is within the channel bound."""
    import fastlisaresponse_gb300 as flr

    dt = 10.0
    orb = flr.KeplerianOrbits(t_max=1.2e6)
    lengths = [12000, 30000]
    hs, lam, beta, t0 = _sources(orb, dt, lengths, seed=62)
    kw = dict(order=79, tdi="2nd generation", orbits=orb, t_buffer=2e4)
    fp = flr.BatchedResponseTDI(1 / dt, precision="fp64", **kw)
    mx = flr.BatchedResponseTDI(1 / dt, precision="mixed", **kw)
    got64 = [_np(o) for o in fp(hs, lam, beta, t0=t0)]
    gotmx = [_np(o) for o in mx(hs, lam, beta, t0=t0)]
    for i, n in enumerate(lengths):
        r = flr.pyResponseTDI(1 / dt, n, order=79, tdi="2nd generation", orbits=orb)
        r.get_projections(hs[i], lam[i], beta[i], t0=t0[i], t_buffer=2e4)
        X, Y, Z = r.get_tdi_delays()
        want = np.stack([_np(X), _np(Y), _np(Z)])
        assert np.array_equal(got64[i], want)
        for c in range(3):
            assert rel_l2(gotmx[i][c], want[c]) <= MIXED_TOL
    assert fp.status() == 0 and mx.status() == 0
    with pytest.raises(ValueError):
        flr.BatchedResponseTDI(1 / dt, precision="mixed", order=81, tdi="2nd generation",
                               orbits=orb, t_buffer=2e4)


def test_outer_taps_split(gpu_lib):
    """The mixed kernel evaluates the outermost TDI taps in FP32 (weights below
    5e-6 together): taps 10..12 at order 25, 14..22 at order 45; the fp64
    flavour keeps every tap in FP64; the mixed channels stay within the bound
    at both orders (test_largest_order and the batch tests cover the rest)."""
    import fastlisaresponse_gb300 as flr

    orb = flr.EqualArmlengthOrbits(t_max=1.2e6)
    for order, first in ((25, 10), (45, 14)):
        kw = dict(order=order, tdi="2nd generation", orbits=orb, t_buffer=2e4)
        mx = flr.BatchedResponseTDI(0.1, precision="mixed", **kw)
        fp = flr.BatchedResponseTDI(0.1, precision="fp64", **kw)
        assert mx.plan_info["fp32_tap_from"] == first
        assert fp.plan_info["fp32_tap_from"] == (order + 1) // 2
