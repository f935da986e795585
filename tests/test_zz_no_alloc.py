"""The allocation-free response entry point (flr_get_response_noalloc).

It exists for callers that cannot call cudaMalloc: code inside a framework
that has already claimed the GPU's memory, and sampler loops that must not pay
the device-wide synchronisation of cudaMalloc/cudaFree.  It keeps its scratch (orbit segment slopes and the status word)
in a fixed array inside the library instead of an orbit handle.

The GPU test calls it through the C ABI, three times in a row with two
different orbit tables (so each call must rebuild the shared scratch), and
checks every output against flr_get_response: identical bits, which implies
the suite's relative-L2 bound of 1e-12 per link.  The test buffers are made
with torch; only the entry point itself must not allocate.  This file is
named to be collected last.
"""

import ctypes

import numpy as np
import pytest

from conftest import TableOrbits, golden_orbit_args, load_golden, rel_l2

_d, _i, _p = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
_ARGTYPES = [_d, _i] + [_p] * 10 + [_d, _i, _p, _i, _i, _d, _i, _p, _d, _i, _p, _i, _p]
MAX_KNOTS = 32768  # FLR_NOALLOC_MAX_KNOTS


def _entry():
    import fastlisaresponse_gb300 as flr

    flr.build()
    lib = ctypes.CDLL(flr.library_path())
    fn = lib.flr_get_response_noalloc
    fn.argtypes = _ARGTYPES
    fn.restype = _i
    lib.flr_last_error.restype = ctypes.c_char_p
    return fn, lib


def test_rejects_tables_beyond_the_limit():
    """Sizes over the stated maximum fail with a clear error before any GPU work."""
    fn, lib = _entry()
    links = (ctypes.c_int * 6)(12, 23, 31, 13, 32, 21)
    sc = (ctypes.c_int * 6)(1, 2, 3, 1, 3, 2)
    rc = fn(1e4, MAX_KNOTS + 1, None, None, links, sc, sc, None, None, None, None, None, 10.0,
            100, None, 100, 25, 0.1, 51, None, 1e-3, 1001, None, 10, None)
    assert rc == -1
    assert b"orbit_N must be in [2, 32768]" in lib.flr_last_error()


def _call_noalloc(fn, lib, resp, g, orb_args):
    import torch

    m = g["meta"]
    n = m["n"]
    dev = resp.device
    dt_o, N_o = orb_args[0], orb_args[1]
    ltt = torch.as_tensor(np.ascontiguousarray(orb_args[3]), device=dev)
    x = torch.as_tensor(np.ascontiguousarray(orb_args[4]), device=dev)
    links = (ctypes.c_int * 6)(*[int(v) for v in orb_args[5]])
    sc_r = (ctypes.c_int * 6)(*[int(v) for v in orb_args[6]])
    sc_e = (ctypes.c_int * 6)(*[int(v) for v in orb_args[7]])
    import fastlisaresponse_gb300 as flr

    k, u, v = (torch.as_tensor(a, device=dev) for a in flr.sky_basis(m["lam"], m["beta"]))
    t = torch.as_tensor(m["t0"] + np.arange(n) * resp.dt, device=dev)
    h = torch.as_tensor(g["h"], device=dev)
    y = torch.zeros(6 * n, dtype=torch.float64, device=dev)
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    ps = resp.buffer_indices(m["t_buffer"])["projections_start_ind"]
    rc = fn(dt_o, N_o, ltt.data_ptr(), x.data_ptr(), links, sc_r, sc_e, y.data_ptr(),
            t.data_ptr(), k.data_ptr(), u.data_ptr(), v.data_ptr(), resp.dt, n, h.data_ptr(), n,
            m["order"], 1 / resp.dt, resp.buffer_integer, resp.A_in.data_ptr(), resp.deps,
            len(resp.A_in), resp.E_in.data_ptr(), ps, stream)
    assert rc == 0, lib.flr_last_error()
    torch.cuda.synchronize(dev)
    return y.cpu().numpy().reshape(6, n)


@pytest.mark.gpu
def test_noalloc_matches_the_allocating_entry_point(gpu_lib):
    import fastlisaresponse_gb300 as flr

    fn, lib = _entry()
    cases = ["rigid_gen1_o25", "flex_gen2_o25_dt5", "rigid_gen1_o25"]
    for name in cases:
        g = load_golden(name)
        m = g["meta"]
        resp = flr.pyResponseTDI(1.0 / m["dt"], m["n"], order=m["order"], tdi=m["tdi"],
                                 orbits=TableOrbits(g))
        resp.get_projections(g["h"], m["lam"], m["beta"], t0=m["t0"], t_buffer=m["t_buffer"])
        want = resp.y_gw.cpu().numpy()
        got = _call_noalloc(fn, lib, resp, g, golden_orbit_args(g))
        for link in range(6):
            assert rel_l2(got[link], want[link]) <= 1e-12
        assert np.array_equal(got, want), name
        assert np.array_equal(got, g["y_gw"]), name
