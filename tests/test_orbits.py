"""Analytic orbit tables: geometry, light travel times and the table layout."""

import numpy as np
import pytest

import oracle
from fastlisaresponse_gb300 import EqualArmlengthOrbits, KeplerianOrbits
from fastlisaresponse_gb300.orbits import C_SI, LINKS


def test_equal_armlength_is_rigid():
    o = EqualArmlengthOrbits(t_max=3.2e7)
    for a, b in [(0, 1), (1, 2), (2, 0)]:
        d = np.linalg.norm(o.x_base[:, a] - o.x_base[:, b], axis=-1)
        assert np.allclose(d, 2.5e9, rtol=1e-12)
    assert np.all(o.ltt_base == 2.5e9 / C_SI)
    centre = o.x_base.mean(axis=1)
    assert np.allclose(np.linalg.norm(centre, axis=-1), 1.495978707e11, rtol=1e-12)


def test_keplerian_flexes_about_one_percent():
    o = KeplerianOrbits(t_max=3.2e7)
    L = o.ltt_base * C_SI / 2.5e9
    assert 0.985 < L.min() < 0.995 and 1.005 < L.max() < 1.015
    # light-cone consistency: c L = |x_r(t) - x_e(t - L)|
    t = o.t_base[100:110]
    for j, link in enumerate(LINKS):
        r, e = int(str(link)[0]) - 1, int(str(link)[1]) - 1
        Lj = o.ltt_base[100:110, j]
        d = np.linalg.norm(o.positions(t)[:, r] - o.positions(t - Lj)[:, e], axis=-1)
        assert np.allclose(d / C_SI, Lj, rtol=1e-13)


def test_pycppdetector_args_layout():
    o = KeplerianOrbits(t_max=1e6)
    dt, N, n_arr, ltt, x, links, sc_r, sc_e, arm = o.pycppdetector_args
    assert dt == 1e4 and N == len(o.t_base)
    assert n_arr.size == N * 18 and ltt.size == N * 6 and x.size == N * 9
    assert list(links) == LINKS and list(sc_r) == [1, 2, 3, 1, 3, 2]
    assert list(sc_e) == [2, 3, 1, 3, 2, 1]
    assert np.array_equal(x.reshape(N, 3, 3), o.x_base)


def test_oracle_orbit_interpolation_rules():
    o = KeplerianOrbits(t_max=1e6)
    orb = oracle.OracleOrbits(*o.pycppdetector_args)
    # knots are reproduced exactly, midpoints are linear
    assert orb.light_travel_time(3e4, 12) == o.ltt_base[3, 0]
    mid = orb.light_travel_time(3.5e4, 23)
    assert mid == pytest.approx(0.5 * (o.ltt_base[3, 1] + o.ltt_base[4, 1]), rel=1e-15)
    # outside the table: zero
    assert orb.light_travel_time(-2e4, 12) == 0.0
    assert np.all(orb.position(o.t_base[-1] + 2e4, 1) == 0.0)
    # the last knot time uses the last segment
    assert orb.light_travel_time(o.t_base[-1], 12) == pytest.approx(o.ltt_base[-1, 0], rel=1e-15)


def test_configure_resamples():
    o = EqualArmlengthOrbits(t_max=1e6)
    o.configure(dt=5e3, linear_interp_setup=True)
    assert o.dt == 5e3 and len(o.t) == 2 * (len(o.t_base) - 1) + 1
    assert o.pycppdetector_args[0] == 5e3
