"""LISA Orbits HDF5 ingestion (orbits.read_lisa_orbits) through a stand-in
for h5py's File interface: the datasets and attributes lisatools reads, the
table shapes the kernels take, and errors on bad files."""

import contextlib
import types

import numpy as np
import pytest


class _Node(dict):
    def __init__(self, data, attrs=None):
        super().__init__(data)
        self.attrs = attrs or {}


def _fake_h5py(files):
    @contextlib.contextmanager
    def File(path, mode):
        assert mode == "r"
        yield files[path]
    return types.SimpleNamespace(File=File)


def _tables(size, dt=1e4):
    import fastlisaresponse_gb300 as flr

    ref = flr.KeplerianOrbits(dt=dt, t_max=(size - 1) * dt)
    return ref, _Node({"tcb": {"x": ref.x_base.copy(), "ltt": ref.ltt_base.copy(),
                               "n": ref.n_base.copy()}}, {"dt": dt, "size": size})


def test_read_lisa_orbits_gives_the_tables():
    import fastlisaresponse_gb300 as flr

    ref, node = _tables(40)
    orb = flr.read_lisa_orbits("orbits.h5", h5py_module=_fake_h5py({"orbits.h5": node}))
    assert np.array_equal(orb.t_base, ref.t_base)
    for a, b in zip(orb.pycppdetector_args, ref.pycppdetector_args):
        assert np.array_equal(np.asarray(a), np.asarray(b))


def test_read_lisa_orbits_flat_datasets_and_errors():
    import fastlisaresponse_gb300 as flr

    ref, node = _tables(12)
    node["tcb"]["x"] = node["tcb"]["x"].reshape(12, 9)  # any row-major layout of the rows
    orb = flr.read_lisa_orbits("a.h5", h5py_module=_fake_h5py({"a.h5": node}))
    assert np.array_equal(orb.x_base, ref.x_base)
    bad = _Node(dict(node), {"dt": 1e4, "size": 13})
    with pytest.raises(ValueError, match="size"):
        flr.read_lisa_orbits("b.h5", h5py_module=_fake_h5py({"b.h5": bad}))
    bad = _Node(dict(node), {"dt": 0.0, "size": 12})
    with pytest.raises(ValueError, match="time grid"):
        flr.read_lisa_orbits("c.h5", h5py_module=_fake_h5py({"c.h5": bad}))


def test_read_lisa_orbits_names_the_missing_reader():
    import fastlisaresponse_gb300 as flr

    try:
        import h5py  # noqa: F401
        pytest.skip("h5py is installed")
    except ImportError:
        pass
    with pytest.raises(ImportError, match="h5py"):
        flr.read_lisa_orbits("missing.h5")
