"""Host-memory runs (BatchedResponseTDI.run_host): sources split into
tile-aligned chunks (flr_batch_source.out_begin/out_end) or short sources
grouped into shared launches, copies overlapped with the launches on two
compute streams; the channels equal those of a device run bit for bit, edge
zones included, for any chunk count and grouping."""

import numpy as np
import pytest

from test_gpu_batch import _np, _sources

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,orbit_kind,chan", [
    ("mixed", "kepler", "XYZ"), ("mixed", "equal", "XYZ"), ("fp64", "kepler", "XYZ"),
    ("mixed", "equal", "AE")])
def test_run_host_matches_device_run(gpu_lib, precision, orbit_kind, chan):
    import torch

    import fastlisaresponse_gb300 as flr

    dt = 10.0
    orb = flr.KeplerianOrbits(t_max=1.6e6) if orbit_kind == "kepler" else \
        flr.EqualArmlengthOrbits(t_max=1.6e6)
    lengths = [2300, 41000, 123457]
    hs, lam, beta, t0 = _sources(orb, dt, lengths, seed=41)
    bat = flr.BatchedResponseTDI(1 / dt, tdi="2nd generation", orbits=orb, tdi_chan=chan,
                                 precision=precision)
    want = [_np(o) for o in bat(hs, lam, beta, t0=t0)]
    h_host = [torch.from_numpy(np.asarray(x)).pin_memory() for x in hs]
    for chunks in (1, 3, 7):
        outs = [torch.full((3, n), float("nan"), dtype=torch.float64).pin_memory()
                for n in lengths]
        got = bat.run_host(h_host, lam, beta, t0=t0, out=outs, chunks=chunks)
        torch.cuda.synchronize(bat.device)
        for g, w in zip(got, want):
            assert np.array_equal(g.numpy(), w), f"chunks={chunks}"
    assert bat.status() == 0


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_run_host_groups_short_sources(gpu_lib, precision):
    """group_samples: runs of short sources share launches (long ones are
    still chunked), with page-locked NumPy host arrays (HostArray); same
    bits as one device run."""
    import torch

    import fastlisaresponse_gb300 as flr

    dt = 10.0
    orb = flr.EqualArmlengthOrbits(t_max=1.6e6)
    lengths = [2300, 5000, 41000, 3000, 123457, 9000, 2500, 60001, 4100]
    hs, lam, beta, t0 = _sources(orb, dt, lengths, seed=47)
    bat = flr.BatchedResponseTDI(1 / dt, tdi="2nd generation", orbits=orb, precision=precision)
    want = [_np(o) for o in bat(hs, lam, beta, t0=t0)]
    h_host = [flr.HostArray(n, np.complex128) for n in lengths]
    o_host = [flr.HostArray((3, n)) for n in lengths]
    for a, x in zip(h_host, hs):
        a.array[:] = np.asarray(x)
    try:
        units = bat._launch_units(lengths, 3, 50000)
        assert sorted(i for u in units for i, r in u if r is None or r[0] == bat.tdi_start_ind) \
            == list(range(len(lengths)))
        assert any(len(u) > 1 for u in units)
        for group in (50000, 10**9):
            for o in o_host:
                o.array.fill(np.nan)
            got = bat.run_host([a.tensor for a in h_host], lam, beta, t0=t0,
                               out=[o.tensor for o in o_host], chunks=3, group_samples=group)
            torch.cuda.synchronize(bat.device)
            for g, w in zip(got, want):
                assert np.array_equal(g.numpy(), w), f"group_samples={group}"
    finally:
        for a in h_host + o_host:
            a.release()
    assert bat.status() == 0


def test_run_host_adjacent_views_share_copies(gpu_lib):
    """Sources that are consecutive views of one HostArray (inputs and
    channels) are moved with one copy per launch each way; same bits as one
    device run, including a gap that breaks the run."""
    import torch

    import fastlisaresponse_gb300 as flr
    from fastlisaresponse_gb300.batch import _contiguous_runs

    dt = 10.0
    orb = flr.EqualArmlengthOrbits(t_max=1.6e6)
    lengths = [2300, 5000, 41000, 3000, 12345, 9000]
    hs, lam, beta, t0 = _sources(orb, dt, lengths, seed=53)
    bat = flr.BatchedResponseTDI(1 / dt, tdi="2nd generation", orbits=orb, precision="mixed")
    want = [_np(o) for o in bat(hs, lam, beta, t0=t0)]
    tot = sum(lengths) + 7  # a gap of 7 samples after the third source
    h_all = flr.HostArray(tot, np.complex128)
    o_all = flr.HostArray(3 * tot)
    try:
        h_v, o_v, off = [], [], 0
        for j, (n, x) in enumerate(zip(lengths, hs)):
            h_v.append(h_all.tensor[off:off + n])
            h_v[-1].copy_(torch.from_numpy(np.asarray(x)))
            o_v.append(o_all.tensor[3 * off:3 * (off + n)].view(3, n))
            off += n + (7 if j == 2 else 0)
        assert [(a, b) for a, b, _ in _contiguous_runs(h_v)] == [(0, 3), (3, 6)]
        assert [(a, b) for a, b, _ in _contiguous_runs(o_v)] == [(0, 3), (3, 6)]
        o_all.array.fill(np.nan)
        got = bat.run_host(h_v, lam, beta, t0=t0, out=o_v, group_samples=10**9)
        torch.cuda.synchronize(bat.device)
        for g, w in zip(got, want):
            assert np.array_equal(g.numpy(), w)
    finally:
        h_all.release()
        o_all.release()
    assert bat.status() == 0


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_chunked_device_call_matches_one_launch(gpu_lib, precision):
    """__call__(chunks=k): tile-aligned launches over two streams, same bits."""
    import fastlisaresponse_gb300 as flr

    dt = 10.0
    orb = flr.KeplerianOrbits(t_max=1.6e6)
    lengths = [41000, 123457]
    hs, lam, beta, t0 = _sources(orb, dt, lengths, seed=43)
    bat = flr.BatchedResponseTDI(1 / dt, tdi="2nd generation", orbits=orb, precision=precision)
    want = [_np(o) for o in bat(hs, lam, beta, t0=t0)]
    for chunks in (2, 5, 64):
        got = bat(hs, lam, beta, t0=t0, chunks=chunks)
        for g, w in zip(got, want):
            assert np.array_equal(_np(g), w), f"chunks={chunks}"
    assert bat.status() == 0


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_grouped_device_call_matches_one_launch(gpu_lib, precision):
    """__call__(group_samples=g): runs of short sources share launches, long
    ones are chunked, over two streams; same bits as one launch."""
    import fastlisaresponse_gb300 as flr

    dt = 10.0
    orb = flr.EqualArmlengthOrbits(t_max=1.6e6)
    lengths = [2300, 5000, 41000, 3000, 123457, 9000, 2500, 60001, 4100, 7000]
    hs, lam, beta, t0 = _sources(orb, dt, lengths, seed=59)
    bat = flr.BatchedResponseTDI(1 / dt, tdi="2nd generation", orbits=orb, precision=precision)
    want = [_np(o) for o in bat(hs, lam, beta, t0=t0)]
    for group in (10000, 50000, 10**9):
        got = bat(hs, lam, beta, t0=t0, chunks=3, group_samples=group)
        for g, w in zip(got, want):
            assert np.array_equal(_np(g), w), f"group_samples={group}"
    assert bat.status() == 0


def test_output_range_rejects_bad_ranges(gpu_lib):
    import fastlisaresponse_gb300 as flr

    dt = 10.0
    orb = flr.EqualArmlengthOrbits(t_max=1.2e6)
    hs, lam, beta, t0 = _sources(orb, dt, [20000], seed=3)
    bat = flr.BatchedResponseTDI(1 / dt, orbits=orb, precision="mixed")
    import torch

    h = [torch.as_tensor(hs[0], device=bat.device)]
    with pytest.raises(ValueError):
        bat._run(h, None, [20000], lam[:1], beta[:1], t0[:1], 0, None, None, False, None,
                 out_range=(10, 500))  # starts inside the garbage zone
