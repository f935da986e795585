"""tile="auto" on the GPU: the autotuner times its candidates, caches the
choice, and the tuned plan's FP64 results equal a fixed-tile plan's bit for
bit (per-sample arithmetic does not depend on the tiling)."""

import numpy as np
import pytest

from test_gpu_batch import _np, _sources

pytestmark = pytest.mark.gpu


def test_auto_tile_tunes_caches_and_matches(gpu_lib, tmp_path, monkeypatch):
    import fastlisaresponse_gb300 as flr
    from fastlisaresponse_gb300 import autotune

    monkeypatch.setenv("FLR_TUNE_CACHE", str(tmp_path / "tiles.json"))
    monkeypatch.setattr(autotune, "TILE_CANDIDATES", (128, 512, 8192))
    autotune._memo.clear()
    dt = 10.0
    orb = flr.KeplerianOrbits(t_max=1.2e6)
    kw = dict(order=25, tdi="2nd generation", orbits=orb, precision="fp64")
    lengths = [20000, 50000]
    # 8192 does not fit in shared memory and is skipped
    r = autotune.best_tile(1 / dt, lengths=lengths, candidates=autotune.TILE_CANDIDATES, **kw)
    assert r["tile"] in (128, 512) and set(r["timings"]) == {"128", "512"} and not r["cached"]
    bat = flr.BatchedResponseTDI(1 / dt, tile="auto", tune_lengths=lengths, **kw)
    assert bat.tune["cached"] and bat.plan_info["tile"] == r["tile"]
    # the plan reports the knobs it runs with: the tuned tile, the fixed CTA
    # size and staging depth
    assert (bat.tune["threads"], bat.tune["staging_depth"]) == (256, 1)
    assert (bat.plan_info["threads"], bat.plan_info["staging_depth"]) == (256, 1)
    other = 512 if r["tile"] == 128 else 128
    ref = flr.BatchedResponseTDI(1 / dt, tile=other, **kw)
    hs, lam, beta, t0 = _sources(orb, dt, lengths, seed=9)
    for a, b in zip(bat(hs, lam, beta, t0=t0), ref(hs, lam, beta, t0=t0)):
        assert np.array_equal(_np(a), _np(b))
    assert bat.status() == 0 and ref.status() == 0
