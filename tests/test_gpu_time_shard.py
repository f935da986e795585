"""One long source sharded by time (BatchedResponseTDI.run_time_shard).

The ranks of a 2-, 3- and 4-way split run one after another on this GPU, each
with only its input slice on the device (the rest NaN): every rank's output
range is free of NaN (no read left the slice), and the ranges put together
equal one launch over the whole source bit for bit, edge zones included.
"""

import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_time_shards_equal_one_launch(gpu_lib, precision):
    import torch

    import fastlisaresponse_gb300 as flr

    dt, n = 5.0, 2**20 + 12345
    orb = flr.KeplerianOrbits(t_max=(math.floor(n * dt / 1e4) + 3) * 1e4)
    rng = np.random.default_rng(17)
    p = flr.waveforms.draw_gb_parameters(rng, 1)
    h = flr.gb_waveform(p["A"][0], p["f"][0], p["fdot"][0], p["iota"][0], p["phi0"][0],
                        p["psi"][0], np.arange(n) * dt)
    bat = flr.BatchedResponseTDI(1 / dt, order=25, tdi="2nd generation", orbits=orb,
                                 precision=precision)
    (want,) = bat([h], p["lam"][0], p["beta"][0])
    ts = bat.tdi_start_ind
    h_host = torch.from_numpy(np.ascontiguousarray(h))
    for world in (2, 3, 4):
        got = torch.full((3, n), float("nan"), dtype=torch.float64, device=want.device)
        ranges = []
        for rank in range(world):
            out, r, (lo, hi) = bat.run_time_shard(h_host, p["lam"][0], p["beta"][0], rank, world)
            a, b = r
            ranges.append(r)
            assert lo < a and hi > b
            if rank == 0:
                a = 0
            if rank == world - 1:
                b = n
            assert not torch.isnan(out[:, a:b]).any(), f"rank {rank} of {world}"
            got[:, a:b] = out[:, a:b]
        assert ranges[0][0] == ts and ranges[-1][1] == n - ts
        assert all(r0[1] == r1[0] for r0, r1 in zip(ranges, ranges[1:]))
        assert torch.equal(got, want), f"world {world}"
    assert bat.status() == 0
