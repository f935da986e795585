"""Host-side logic of the product package (tables, basis, buffers, argument
validation) against the oracle and the reference's golden tables; CPU only."""

import numpy as np
import pytest

import oracle
from conftest import golden_names, load_golden
from fastlisaresponse_gb300 import response as R
from fastlisaresponse_gb300.binding import _Array, _length_error


@pytest.mark.parametrize("name", golden_names())
def test_tables_equal_reference_golden(name):
    g = load_golden(name)
    m = g["meta"]
    A, E, deps = R.lagrange_tables(m["order"])
    assert np.array_equal(A, g["A_in"]) and np.array_equal(E, g["E_in"])
    assert deps == float(g["deps"])
    tdi = m["tdi"]
    if tdi == "1st generation":
        combos = R.TDI_FIRST_GENERATION
    elif tdi == "2nd generation":
        combos = R.TDI_FIRST_GENERATION + R.TDI_SECOND_GENERATION_EXTRA
    else:
        combos = tdi
    tb = R.tdi_unit_tables(combos)
    for key in ("tdi_base_links", "tdi_link_combinations", "tdi_signs", "channels",
                "tdi_operation_index"):
        assert np.array_equal(tb[key], g[key]), key
    k, u, v = R.sky_basis(m["lam"], m["beta"])
    ko, uo, vo = oracle.sky_basis(m["lam"], m["beta"])
    assert np.array_equal(k, ko) and np.array_equal(u, uo) and np.array_equal(v, vo)


@pytest.mark.parametrize("order", [1, 3, 5, 11, 25, 26, 39, 45, 61, 79])
def test_lagrange_tables_all_orders(order):
    A, E, deps = R.lagrange_tables(order)
    h = int((order + 1) / 2)
    assert A.shape == (1001,) and E.shape == (h,)
    assert np.all(np.isfinite(A)) and np.all(np.isfinite(E))
    assert A[0] == pytest.approx(1.0, rel=1e-14)  # A(0) = 1
    assert np.all(np.sign(E[: h - 1]) == (-1.0) ** np.arange(1, h))
    if order <= 39:
        Ao, Eo, _ = oracle.fill_A_E(order)
        assert np.array_equal(A, Ao) and np.array_equal(E, Eo)


def test_tdi_unit_counts():
    g1 = R.tdi_unit_tables(R.TDI_FIRST_GENERATION)
    g2 = R.tdi_unit_tables(R.TDI_FIRST_GENERATION + R.TDI_SECOND_GENERATION_EXTRA)
    assert g1["num_units"] == 24 and len(g1["tdi_link_combinations"]) == 42
    assert g2["num_units"] == 48 and len(g2["tdi_link_combinations"]) == 174
    assert np.array_equal(np.bincount(g2["channels"]), [16, 16, 16])


def test_cyclic_permutation():
    assert [R.cyclic_permutation(12, p) for p in range(3)] == [12, 23, 31]
    assert [R.cyclic_permutation(31, p) for p in range(3)] == [31, 12, 23]
    for link in (12, 23, 31, 13, 32, 21):
        for p in range(3):
            assert R.cyclic_permutation(link, p) == oracle.cyclic_permutation(link, p)


def test_cpu_backend_is_refused():
    with pytest.raises(ValueError, match="no CPU backend"):
        R._resolve_device("cpu")
    with pytest.raises(ValueError):
        R._resolve_device("rocm")


def test_bad_tdi_kwarg():
    class Dummy(R.pyResponseTDI):
        def __init__(self):
            self.tdi = "3rd generation"

    with pytest.raises(ValueError, match="tdi kwarg"):
        Dummy()._init_TDI_delays()


def test_length_check_message_matches_reference():
    err = _length_error("y_gw", 60, 59)
    assert str(err) == ("y_gw: input arrays have the incorrect length. Should be 60. "
                        "It's length is 59.")
    arr = _Array(np.zeros(10), np.float64, "t_arr", allow_host=True)
    with pytest.raises(ValueError, match="t_arr: input arrays have the incorrect length"):
        arr.check_length(5, 3)
    with pytest.raises(TypeError):
        _Array(np.zeros(10), np.float64, "y_gw")  # device array required
    # host tables are converted like pybind11's py::array_t<double> does
    conv = _Array(np.zeros(10, dtype=np.float32), np.float64, "x", allow_host=True)
    assert conv.obj.dtype == np.float64 and conv.size == 10


def test_buffer_indices_match_oracle():
    from fastlisaresponse_gb300 import EqualArmlengthOrbits

    orb = EqualArmlengthOrbits(t_max=1e6)
    for order, dt, tb in [(25, 10.0, 1e4), (25, 5.0, 1e4), (11, 10.0, 2e4)]:
        obj = R.pyResponseTDI.__new__(R.pyResponseTDI)
        obj.sampling_frequency, obj.dt, obj.order = 1 / dt, 1 / (1 / dt), order
        x = orb.x_base
        obj._max_sc_distance = float((np.sum(x * x, axis=-1) ** 0.5).max())
        mine = obj.buffer_indices(tb)
        ref = oracle.buffer_indices(order, 1 / dt, tb, x)
        for key in ("tdi_start_ind", "projections_start_ind"):
            assert mine[key] == ref[key]
    with pytest.raises(ValueError, match="increase t_buffer"):
        obj.buffer_indices(3000.0)
