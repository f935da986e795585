"""The allocation-free response entry point (flr_get_response_noalloc).

It exists for callers that cannot call cudaMalloc: code inside a framework
that has already claimed the GPU's memory, and sampler loops that must not pay
the device-wide synchronisation of cudaMalloc/cudaFree.  It keeps its scratch (orbit segment slopes and the status word)
in a fixed array inside the library instead of an orbit handle.

The GPU tests call it through the C ABI: three times in a row with two
different orbit tables (so each call must rebuild the shared scratch),
checking every output against flr_get_response (identical bits, which implies
the suite's relative-L2 bound of 1e-12 per link) and the device's free memory
before and after the calls after the first (unchanged: the calls allocate
nothing); and once with a start index whose interpolation windows leave the
input, whose status bits flr_noalloc_status must report (and a clean call
then clear).  The test buffers are made with torch before the calls; only the
entry point itself must not allocate.  This file is named to be collected
last.
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
    lib.flr_noalloc_status.argtypes = [ctypes.POINTER(ctypes.c_uint32), _i, _p]
    lib.flr_noalloc_status.restype = _i
    return fn, lib


def _status(lib, stream, reset=False):
    bits = ctypes.c_uint32(0xffffffff)
    rc = lib.flr_noalloc_status(ctypes.byref(bits), int(reset), stream)
    assert rc == 0, lib.flr_last_error()
    return bits.value


def test_rejects_tables_beyond_the_limit():
    """Sizes over the stated maximum fail with a clear error before any GPU work."""
    fn, lib = _entry()
    links = (ctypes.c_int * 6)(12, 23, 31, 13, 32, 21)
    sc = (ctypes.c_int * 6)(1, 2, 3, 1, 3, 2)
    rc = fn(1e4, MAX_KNOTS + 1, None, None, links, sc, sc, None, None, None, None, None, 10.0,
            100, None, 100, 25, 0.1, 51, None, 1e-3, 1001, None, 10, None)
    assert rc == -1
    assert b"orbit_N must be in [2, 32768]" in lib.flr_last_error()


def _prepare(resp, g, orb_args):
    """Device buffers of one call (made before the call: the test's own
    allocations are not the entry point's)."""
    import torch

    import fastlisaresponse_gb300 as flr

    m = g["meta"]
    n = m["n"]
    dev = resp.device
    k, u, v = (torch.as_tensor(a, device=dev) for a in flr.sky_basis(m["lam"], m["beta"]))
    return dict(
        n=n, m=m, dt_o=orb_args[0], N_o=orb_args[1],
        ltt=torch.as_tensor(np.ascontiguousarray(orb_args[3]), device=dev),
        x=torch.as_tensor(np.ascontiguousarray(orb_args[4]), device=dev),
        links=(ctypes.c_int * 6)(*[int(v) for v in orb_args[5]]),
        sc_r=(ctypes.c_int * 6)(*[int(v) for v in orb_args[6]]),
        sc_e=(ctypes.c_int * 6)(*[int(v) for v in orb_args[7]]),
        k=k, u=u, v=v,
        t=torch.as_tensor(m["t0"] + np.arange(n) * resp.dt, device=dev),
        h=torch.as_tensor(g["h"], device=dev),
        y=torch.zeros(6 * n, dtype=torch.float64, device=dev),
        stream=ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream),
        ps=resp.buffer_indices(m["t_buffer"])["projections_start_ind"])


def _call(fn, lib, resp, b, start=None):
    """One call on prepared buffers; returns the (6, n) links on the host."""
    import torch

    n, m = b["n"], b["m"]
    rc = fn(b["dt_o"], b["N_o"], b["ltt"].data_ptr(), b["x"].data_ptr(), b["links"], b["sc_r"],
            b["sc_e"], b["y"].data_ptr(), b["t"].data_ptr(), b["k"].data_ptr(),
            b["u"].data_ptr(), b["v"].data_ptr(), resp.dt, n, b["h"].data_ptr(), n, m["order"],
            1 / resp.dt, resp.buffer_integer, resp.A_in.data_ptr(), resp.deps,
            len(resp.A_in), resp.E_in.data_ptr(), b["ps"] if start is None else start,
            b["stream"])
    assert rc == 0, lib.flr_last_error()
    torch.cuda.synchronize(resp.device)
    return b["y"].cpu().numpy().reshape(6, n)


@pytest.mark.gpu
def test_noalloc_matches_the_allocating_entry_point(gpu_lib):
    import torch

    import fastlisaresponse_gb300 as flr

    fn, lib = _entry()
    cases = ["rigid_gen1_o25", "flex_gen2_o25_dt5", "rigid_gen1_o25"]
    runs = []
    for name in cases:  # every buffer first, so that only the calls run below
        g = load_golden(name)
        m = g["meta"]
        resp = flr.pyResponseTDI(1.0 / m["dt"], m["n"], order=m["order"], tdi=m["tdi"],
                                 orbits=TableOrbits(g))
        resp.get_projections(g["h"], m["lam"], m["beta"], t0=m["t0"], t_buffer=m["t_buffer"])
        runs.append((name, g, resp, resp.y_gw.cpu().numpy(),
                     _prepare(resp, g, golden_orbit_args(g))))
    torch.cuda.synchronize()
    free_after = []
    for i, (name, g, resp, want, b) in enumerate(runs):
        got = _call(fn, lib, resp, b)
        free_after.append(torch.cuda.mem_get_info()[0])
        for link in range(6):
            assert rel_l2(got[link], want[link]) <= 1e-12
        assert np.array_equal(got, want), name
        assert np.array_equal(got, g["y_gw"]), name
        assert _status(lib, b["stream"]) == 0, name
    # the first call may load the module; the later ones leave free memory as it was
    assert free_after[1] == free_after[0] and free_after[2] == free_after[0], free_after


@pytest.mark.gpu
def test_noalloc_status_reports_bad_windows(gpu_lib):
    """A start index of 0 makes the first samples' windows reach before the
    input: NaN there, the tap bit in the status word, and the next clean call
    clears it."""
    import fastlisaresponse_gb300 as flr

    fn, lib = _entry()
    g = load_golden("rigid_gen1_o25")
    m = g["meta"]
    resp = flr.pyResponseTDI(1.0 / m["dt"], m["n"], order=m["order"], tdi=m["tdi"],
                             orbits=TableOrbits(g))
    b = _prepare(resp, g, golden_orbit_args(g))
    y = _call(fn, lib, resp, b, start=0)
    assert np.isnan(y[:, 0]).all()
    assert _status(lib, b["stream"]) & 0x1
    assert _status(lib, b["stream"], reset=True) & 0x1
    assert _status(lib, b["stream"]) == 0
    _call(fn, lib, resp, b, start=0)
    assert _status(lib, b["stream"]) & 0x1
    y = _call(fn, lib, resp, b)
    assert _status(lib, b["stream"]) == 0
    ps = b["ps"]
    assert np.array_equal(y[:, ps:m["n"] - ps], g["y_gw"][:, ps:m["n"] - ps])
