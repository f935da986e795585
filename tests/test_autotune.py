"""Autotuner host logic (CPU): cache keys, size classes, the JSON cache, and
the choice of the fastest candidate with a fake timing function."""

import json

import numpy as np
import pytest

from fastlisaresponse_gb300 import autotune
from fastlisaresponse_gb300.orbits import EqualArmlengthOrbits, KeplerianOrbits
from fastlisaresponse_gb300.response import tdi_unit_tables
from fastlisaresponse_gb300.batch import _combinations


def test_equal_arms_detection():
    assert autotune.equal_arms(EqualArmlengthOrbits(t_max=1e5))
    assert not autotune.equal_arms(KeplerianOrbits(t_max=1e5))


def test_size_class_and_key():
    assert autotune.size_class([2**18] * 32, 1000) == int(np.floor(np.log2(32 * (2**18 - 2000))))
    assert autotune.size_class([10, 20], 1000) == 0
    sets = [tdi_unit_tables(_combinations("2nd generation"))]
    k1 = autotune.tune_key("GB300", "mixed", 25, sets, "XYZ", True, 0.1, 23)
    k2 = autotune.tune_key("GB300", "mixed", 45, sets, "XYZ", True, 0.1, 23)
    k3 = autotune.tune_key("GB300", "fp64", 25, sets, "XYZ", True, 0.1, 23)
    k4 = autotune.tune_key("GB300", "mixed", 25,
                           [tdi_unit_tables(_combinations("1st generation"))], "XYZ", True, 0.1,
                           23)
    assert len({k1, k2, k3, k4}) == 4
    assert "order25" in k1 and "equal" in k1 and "2^23" in k1


def test_cache_roundtrip(tmp_path, monkeypatch):
    path = tmp_path / "tiles.json"
    monkeypatch.setenv("FLR_TUNE_CACHE", str(path))
    autotune._store("k", {"tile": 256, "timings": {"256": 1.0}})
    autotune._store("k2", {"tile": 1024, "timings": {"1024": 2.0}})
    data = json.loads(path.read_text())
    assert data["k"]["tile"] == 256 and data["k2"]["tile"] == 1024
    path.write_text("not json")
    assert autotune._load() == {}


def test_best_tile_picks_fastest_and_caches(tmp_path, monkeypatch):
    """best_tile with the device and the timing replaced by fakes."""
    torch = pytest.importorskip("torch")
    monkeypatch.setenv("FLR_TUNE_CACHE", str(tmp_path / "tiles.json"))
    monkeypatch.setattr(torch.cuda, "get_device_name", lambda dev=None: "FakeGPU")
    import fastlisaresponse_gb300.response as resp

    monkeypatch.setattr(resp, "_resolve_device", lambda fb: "fake")
    calls = []

    def fake_measure(make_plan, lengths, candidates, device, reps=3, seed=0):
        calls.append(tuple(candidates))
        return {c: abs(c - 512) / 512 + 1.0 for c in candidates}

    monkeypatch.setattr(autotune, "measure", fake_measure)
    autotune._memo.clear()
    orb = EqualArmlengthOrbits(t_max=1e5)
    r = autotune.best_tile(0.1, 25, "2nd generation", orb, "mixed", lengths=[2**16] * 4)
    assert r["tile"] == 512 and not r["cached"]
    autotune._memo.clear()  # the file alone answers the second query
    r2 = autotune.best_tile(0.1, 25, "2nd generation", orb, "mixed", lengths=[2**16] * 4)
    assert r2["tile"] == 512 and r2["cached"] and len(calls) == 1
    r3 = autotune.best_tile(0.1, 45, "2nd generation", orb, "mixed", lengths=[2**16] * 4,
                            t_buffer=2e4)
    assert not r3["cached"] and len(calls) == 2
