"""The CPU oracle against the reference: golden fixtures, the reference's own
compiled CPU code, and known-answer properties of the interpolation."""

import numpy as np
import pytest

import oracle
import refdrive
from conftest import golden_names, golden_orbit_args, load_golden

GOLDEN = golden_names()


def run_oracle_on_golden(g):
    m = g["meta"]
    orc = oracle.OracleResponseTDI(1.0 / m["dt"], m["n"], golden_orbit_args(g), g["x_base"],
                                   order=m["order"], tdi=m["tdi"], tdi_chan=m["tdi_chan"])
    orc.get_projections(g["h"], m["lam"], m["beta"], t0=m["t0"], t_buffer=m["t_buffer"])
    chans = orc.get_tdi_delays()
    return orc, chans


def test_golden_fixtures_present():
    assert len(GOLDEN) >= 5


@pytest.mark.parametrize("name", GOLDEN)
def test_oracle_tables_match_reference(name):
    g = load_golden(name)
    m = g["meta"]
    A, E, deps = oracle.fill_A_E(m["order"])
    assert np.array_equal(A, g["A_in"]) and np.array_equal(E, g["E_in"])
    assert deps == float(g["deps"])
    tb = oracle.tdi_tables(oracle.tdi_combinations(m["tdi"]))
    for key in ("tdi_base_links", "tdi_link_combinations", "tdi_signs", "channels",
                "tdi_operation_index"):
        assert np.array_equal(tb[key], g[key]), key
    idx = oracle.buffer_indices(m["order"], 1.0 / m["dt"], m["t_buffer"], g["x_base"])
    assert idx["tdi_start_ind"] == int(g["tdi_start_ind"])
    assert idx["projections_start_ind"] == int(g["projections_start_ind"])


@pytest.mark.parametrize("name", GOLDEN)
def test_oracle_bit_exact_on_golden(name):
    g = load_golden(name)
    orc, chans = run_oracle_on_golden(g)
    assert np.array_equal(orc.y_gw, g["y_gw"])
    assert np.array_equal(orc.XYZ, g["XYZ"])
    assert np.array_equal(np.stack(chans), g["chans"])


def test_golden_outputs_are_nontrivial():
    for name in GOLDEN:
        g = load_golden(name)
        ps, ts, n = int(g["projections_start_ind"]), int(g["tdi_start_ind"]), g["meta"]["n"]
        assert np.all(np.isfinite(g["y_gw"]))
        assert np.all(g["y_gw"][:, ps:n - ps] != 0.0)
        assert np.all(g["y_gw"][:, :ps] == 0.0) and np.all(g["y_gw"][:, n - ps:] == 0.0)
        assert np.all(g["XYZ"][:, ts:n - ts] != 0.0)


requires_reference = pytest.mark.skipif(not refdrive.available(),
                                        reason="reference sources not present")


@requires_reference
@pytest.mark.parametrize("order,tdi,orbit_kind,dt,seed", [
    (25, "1st generation", "equal", 10.0, 0),
    (25, "2nd generation", "kepler", 10.0, 1),
    (3, "1st generation", "kepler", 10.0, 2),
    (7, "2nd generation", "equal", 5.0, 3),
    (39, "1st generation", "kepler", 10.0, 4),
    (26, "1st generation", "kepler", 10.0, 5),
])
def test_oracle_matches_reference_build(order, tdi, orbit_kind, dt, seed):
    """Random sources through the reference's Python layer and compiled CPU
    kernels vs the oracle: identical bits."""
    from fastlisaresponse_gb300 import orbits as om, waveforms as wf

    rng = np.random.default_rng(seed)
    n = 3000 + int(rng.integers(0, 2000))
    t0 = float(rng.uniform(0, 1e6))
    t_max = (np.floor((t0 + n * dt) / 1e4) + 3) * 1e4
    orb = om.EqualArmlengthOrbits(t_max=t_max) if orbit_kind == "equal" else \
        om.KeplerianOrbits(t_max=t_max)
    p = wf.draw_gb_parameters(rng, 1)
    h = wf.gb_waveform(p["A"][0], p["f"][0], p["fdot"][0], p["iota"][0], p["phi0"][0],
                       p["psi"][0], t0 + np.arange(n) * dt)
    ref = refdrive.import_reference_response()
    r = ref.pyResponseTDI(1.0 / dt, n, order=order, tdi=tdi, orbits=refdrive.StubOrbits(orb))
    r.get_projections(h, p["lam"][0], p["beta"][0], t0=t0, t_buffer=1e4)
    X, Y, Z = r.get_tdi_delays()

    o = oracle.OracleResponseTDI(1.0 / dt, n, orb.pycppdetector_args, orb.x_base, order=order,
                                 tdi=tdi)
    o.get_projections(h, p["lam"][0], p["beta"][0], t0=t0, t_buffer=1e4)
    Xo, Yo, Zo = o.get_tdi_delays()
    assert np.array_equal(r.y_gw_flat, o.y_gw_flat)
    assert np.array_equal(X, Xo) and np.array_equal(Y, Yo) and np.array_equal(Z, Zo)


def test_range_variant_is_a_slice():
    g = load_golden(GOLDEN[0])
    m = g["meta"]
    full, _ = run_oracle_on_golden(g)
    orb = oracle.OracleOrbits(*golden_orbit_args(g))
    k, u, v = oracle.sky_basis(m["lam"], m["beta"])
    n = m["n"]
    t = m["t0"] + np.arange(n) * m["dt"]
    y = np.zeros(6 * n)
    ps = int(g["projections_start_ind"])
    oracle.get_response(orb, y, t, k, u, v, n, g["h"], m["order"], 1 / m["dt"], g["A_in"],
                        float(g["deps"]), g["E_in"], ps, sample_range=(1500, 1700))
    y = y.reshape(6, n)
    assert np.array_equal(y[:, 1500:1700], full.y_gw[:, 1500:1700])
    assert np.all(y[:, :1500] == 0) and np.all(y[:, 1700:] == 0)


# -- known answers of the Lagrange kernel ----------------------------------------

def _interp_via_tdi(x, delay_samples, order):
    """Interpolate a real series at t - delay with the oracle's TDI path: one
    unit, base link 12, no delay links, so the TDI delay is t and the sample
    grid is shifted by moving t_arr instead."""
    n = len(x)
    A, E, deps = oracle.fill_A_E(order)
    ltt = np.zeros((4, 6))
    xs = np.zeros((4, 3, 3))
    orb = oracle.OracleOrbits(1e9, 4, np.zeros(4 * 18), ltt, xs, oracle.LINKS, [1, 2, 3, 1, 3, 2],
                              [2, 3, 1, 3, 2, 1], 2.5e9)
    y = np.zeros((6, n))
    y[0] = x
    out = np.zeros(n)
    t = np.arange(n) - delay_samples
    t[0] = 0.0  # t_arr[0] is the time origin of the series
    oracle.get_tdi_delays(orb, out, y.reshape(-1), n, n, t, [0], [1], [12], [-11], [1.0], [0], 1,
                          order, 1.0, A, deps, E, 40)
    return out


def test_integer_delay_reproduces_samples():
    x = np.random.default_rng(0).standard_normal(200)
    out = _interp_via_tdi(x, 3.0, 25)
    assert np.allclose(out[40:160], x[37:157], rtol=0, atol=1e-15)


def test_constant_input_error_is_the_A_table_lerp():
    out = _interp_via_tdi(np.ones(200), 2.3717, 25)  # eps between A knots
    # exact Lagrange reproduces 1; the tabulated A(eps) deviates by < 2.2e-7
    assert np.all(np.abs(out[40:160] - 1.0) < 2.2e-7)
    assert np.any(np.abs(out[40:160] - 1.0) > 1e-9)


def test_fractional_delay_of_smooth_signal():
    n = 400
    tt = np.arange(n, dtype=np.float64)
    x = np.sin(2 * np.pi * 0.01 * tt)
    out = _interp_via_tdi(x, 5.3, 25)
    expect = np.sin(2 * np.pi * 0.01 * (tt - 5.3))
    assert np.max(np.abs(out[40:360] - expect[40:360])) < 3e-7
