"""Shared test setup: import paths, the `gpu` marker, golden fixtures."""

import glob
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.normpath(os.path.join(os.path.dirname(__file__), ".."))
for sub in ("lisa-on-gpu_gb300", "oracle", ""):
    path = os.path.join(ROOT, sub) if sub else ROOT
    if path not in sys.path:
        sys.path.insert(0, path)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden_names():
    return sorted(os.path.splitext(os.path.basename(p))[0]
                  for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))


def load_golden(name):
    with np.load(os.path.join(GOLDEN_DIR, f"{name}.npz")) as z:
        data = {k: z[k] for k in z.files}
    data["meta"] = json.loads(str(data["meta"]))
    return data


def golden_orbit_args(g):
    return [float(g["orb_dt"]), int(g["orb_N"]), g["orb_n"], g["orb_ltt"], g["orb_x"],
            g["orb_links"], g["orb_sc_r"], g["orb_sc_e"], float(g["orb_armlength"])]


class TableOrbits:
    """Orbit object built from stored tables (the lisatools-style surface the
    response classes read)."""

    LINKS = [12, 23, 31, 13, 32, 21]

    def __init__(self, g):
        self._args = golden_orbit_args(g)
        dt, N = self._args[0], self._args[1]
        self.t_base = np.arange(N) * dt
        self.t = self.t_base
        self.x_base = g["x_base"]
        self.configured = True
        self.armlength = self._args[8]

    def configure(self, *a, **k):
        return self

    @property
    def pycppdetector_args(self):
        return list(self._args)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a - b))


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if needed) and loads the CUDA library; skips without a GPU."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import fastlisaresponse_gb300 as flr

    flr.build()
    from fastlisaresponse_gb300 import _lib

    return _lib.lib()
