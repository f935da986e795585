"""The C oracle over a whole long source on all host cores -- TEST HELPER.

The oracle's kernels take a sample range (``oracle.get_response`` /
``get_tdi_delays`` with ``sample_range``), so a long source splits into
disjoint ranges evaluated by a process pool (``spawn``: safe after CUDA is
initialised in the parent).  Inputs and outputs live in shared memory:

1. every worker writes the link streams y of its range of [ps, n - ps);
2. after all of them, every worker accumulates the TDI channels of its range
   of [ts, n - ts), reading the shared y.

Each output sample is computed by the same C code on the same values as a
single-process run, so the result is bit-identical to it.
"""

from __future__ import annotations

import multiprocessing as mp
import os
from concurrent.futures import ProcessPoolExecutor
from multiprocessing import shared_memory

import numpy as np

import oracle

_state = {}


def _attach(name, shape, dtype):
    shm = shared_memory.SharedMemory(name=name)
    return shm, np.ndarray(shape, dtype=dtype, buffer=shm.buf)


def _init(spec):
    n = spec["n"]
    shms = []
    arrays = {}
    for key, shape, dtype in (("h", (n,), np.complex128), ("y", (6 * n,), np.float64),
                              ("xyz", (3 * n,), np.float64)):
        shm, arr = _attach(spec["shm"][key], shape, dtype)
        shms.append(shm)
        arrays[key] = arr
    o = oracle.OracleResponseTDI(1.0 / spec["dt"], n, spec["orbit_args"], spec["x_base"],
                                 order=spec["order"], tdi=spec["tdi"])
    idx = oracle.buffer_indices(spec["order"], 1.0 / spec["dt"], spec["t_buffer"],
                                spec["x_base"])
    k, u, v = oracle.sky_basis(spec["lam"], spec["beta"])
    t = spec["t0"] + np.arange(n) * spec["dt"]
    _state.update(spec=spec, shms=shms, arrays=arrays, o=o, idx=idx, k=k, u=u, v=v, t=t)


def _response(rng):
    s = _state
    sp, o = s["spec"], s["o"]
    oracle.get_response(o.orbits, s["arrays"]["y"], s["t"], s["k"], s["u"], s["v"], sp["n"],
                        s["arrays"]["h"], sp["order"], 1.0 / sp["dt"], o.A_in, o.deps, o.E_in,
                        s["idx"]["projections_start_ind"], sample_range=rng)
    return rng


def _tdi(rng):
    s = _state
    sp, o, tb = s["spec"], s["o"], s["o"].tables
    oracle.get_tdi_delays(o.orbits, s["arrays"]["xyz"], s["arrays"]["y"], sp["n"], sp["n"],
                          s["t"], tb["unit_starts"], tb["unit_lengths"], tb["tdi_base_links"],
                          tb["tdi_link_combinations"], tb["tdi_signs"], tb["channels"],
                          tb["num_units"], sp["order"], 1.0 / sp["dt"], o.A_in, o.deps, o.E_in,
                          s["idx"]["tdi_start_ind"], sample_range=rng)
    return rng


def _ranges(lo, hi, parts):
    edges = np.linspace(lo, hi, parts + 1).astype(np.int64)
    return [(int(a), int(b)) for a, b in zip(edges[:-1], edges[1:]) if b > a]


def response_tdi(h, lam, beta, orbit_args, x_base, dt, order=25, tdi="1st generation",
                 t0=0.0, t_buffer=1e4, workers=None):
    """y_gw (6, n) and XYZ (3, n) of the oracle chain (get_projections +
    get_tdi_delays as the reference's pyResponseTDI runs them) for one source,
    computed in parallel; also the start indices."""
    h = np.ascontiguousarray(h, dtype=np.complex128)
    n = len(h)
    workers = workers or os.cpu_count() or 1
    idx = oracle.buffer_indices(order, 1.0 / dt, t_buffer, x_base)
    ps, ts = idx["projections_start_ind"], idx["tdi_start_ind"]
    shms = {}
    try:
        for key, nbytes in (("h", 16 * n), ("y", 48 * n), ("xyz", 24 * n)):
            shms[key] = shared_memory.SharedMemory(create=True, size=nbytes)
        np.ndarray((n,), np.complex128, buffer=shms["h"].buf)[:] = h
        np.ndarray((6 * n,), np.float64, buffer=shms["y"].buf)[:] = 0.0
        np.ndarray((3 * n,), np.float64, buffer=shms["xyz"].buf)[:] = 0.0
        spec = dict(n=n, dt=dt, order=order, tdi=tdi, t0=t0, t_buffer=t_buffer, lam=lam,
                    beta=beta, orbit_args=orbit_args, x_base=np.asarray(x_base),
                    shm={k: v.name for k, v in shms.items()})
        parts = 4 * workers
        # a worker that dies breaks the executor (an exception, not a hang)
        with ProcessPoolExecutor(workers, mp_context=mp.get_context("spawn"), initializer=_init,
                                 initargs=(spec,)) as pool:
            list(pool.map(_response, _ranges(ps, n - ps, parts)))
            list(pool.map(_tdi, _ranges(ts, n - ts, parts)))
        y = np.ndarray((6, n), np.float64, buffer=shms["y"].buf).copy()
        xyz = np.ndarray((3, n), np.float64, buffer=shms["xyz"].buf).copy()
    finally:
        for shm in shms.values():
            shm.close()
            shm.unlink()
    return y, xyz, idx
