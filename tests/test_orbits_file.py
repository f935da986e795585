"""LISA Orbits HDF5 ingestion (orbits.read_lisa_orbits): through a stand-in
for h5py's File interface (the datasets and attributes lisatools reads, the
table shapes the kernels take, errors on bad files) and through the built-in
HDF5 reader (h5lite) on real HDF5 files: one the HDF5 library wrote, and
LISA Orbits-layout files in both of the library's format styles."""

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


def _scipy_matlab_data(name):
    import os

    scipy = pytest.importorskip("scipy")
    path = os.path.join(os.path.dirname(scipy.__file__), "io", "matlab", "tests", "data", name)
    if not os.path.exists(path):
        pytest.skip(f"scipy's test file {name} is not installed")
    return path


def test_h5lite_reads_a_file_written_by_the_hdf5_library():
    """scipy's MATLAB 7.3 test file was written by the HDF5 library (512-byte
    user block, superblock 0, symbol-table groups); scipy ships the same
    variable as a version-5 MAT-file, read here with scipy.io.loadmat."""
    from scipy.io import loadmat

    from fastlisaresponse_gb300 import h5lite

    want = loadmat(_scipy_matlab_data("testdouble_7.4_GLNX86.mat"))["testdouble"]
    with h5lite.File(_scipy_matlab_data("testhdf5_7.4_GLNX86.mat")) as f:
        assert list(f.keys()) == ["testdouble"]
        ds = f["testdouble"]
        assert ds.shape == (9, 1) and ds.dtype == np.float64
        assert ds.attrs["MATLAB_class"] == b"double"
        got = np.asarray(ds)
        assert np.array_equal(got.T, want)  # MATLAB stores column-major
        assert np.array_equal(ds[3:5, 0], want[0, 3:5])


def _orbits_file(path, style, chunks, ref, big_endian=False, user_block=0):
    from _h5write import Writer

    w = Writer(style, user_block=user_block)
    w.root["attrs"].update({"generator": "lisaorbits (test layout)", "dt": float(ref.t_base[1] - ref.t_base[0]),
                            "size": np.int64(ref.t_base.size), "t0": 0.0,
                            "L": np.array([2.5e9] * 6)})
    size = ref.t_base.size
    x = ref.x_base.astype(">f8") if big_endian else ref.x_base
    w.dataset("tcb/x", x, chunks=(7, 3, 3) if chunks else None)
    w.dataset("tcb/ltt", ref.ltt_base, chunks=(5, 6) if chunks else None, attrs={"units": "s"})
    w.dataset("tcb/n", ref.n_base, chunks=(size, 6, 3) if chunks else None)
    w.dataset("tps/ltt", ref.ltt_base * 0.5)
    w.save(path)


@pytest.mark.parametrize("style,chunks,big_endian,user_block", [
    ("v0", False, False, 0), ("v0", True, True, 512), ("v2", False, True, 0),
    ("v2", True, False, 1024)])
def test_read_lisa_orbits_from_an_hdf5_file(tmp_path, style, chunks, big_endian, user_block):
    """LISA Orbits layout in the two HDF5 styles the library writes (h5py's
    default and libver="latest"), contiguous and chunked (shuffle + deflate)
    datasets; read through read_lisa_orbits' built-in reader."""
    import fastlisaresponse_gb300 as flr
    from fastlisaresponse_gb300 import h5lite

    ref = flr.KeplerianOrbits(dt=1e4, t_max=22 * 1e4)
    path = tmp_path / f"orbits_{style}.h5"
    _orbits_file(path, style, chunks, ref, big_endian, user_block)
    orb = flr.read_lisa_orbits(path, h5py_module=h5lite)
    assert np.array_equal(orb.t_base, ref.t_base)
    for a, b in zip(orb.pycppdetector_args, ref.pycppdetector_args):
        assert np.array_equal(np.asarray(a), np.asarray(b))
    with h5lite.File(path) as f:
        assert set(f.keys()) == {"tcb", "tps"} and set(f["tcb"].keys()) == {"x", "ltt", "n"}
        assert f.attrs["generator"] == "lisaorbits (test layout)"
        assert f.attrs["size"] == ref.t_base.size and isinstance(f.attrs["dt"], np.floating)
        assert np.array_equal(f.attrs["L"], [2.5e9] * 6)
        assert f["tcb/ltt"].attrs["units"] == "s"
        assert np.array_equal(f["tps"]["ltt"][()], ref.ltt_base * 0.5)
        assert "tcb/v" not in f and "tcb/x" in f
        with pytest.raises(KeyError):
            f["tcb/v"]


def test_read_lisa_orbits_without_h5py(tmp_path):
    """With h5py absent, read_lisa_orbits falls back to the built-in reader."""
    import fastlisaresponse_gb300 as flr

    try:
        import h5py  # noqa: F401
        pytest.skip("h5py is installed")
    except ImportError:
        pass
    ref = flr.EqualArmlengthOrbits(dt=1e4, t_max=30 * 1e4)
    path = tmp_path / "equal.h5"
    _orbits_file(path, "v0", False, ref)
    orb = flr.read_lisa_orbits(path)
    assert np.array_equal(orb.ltt_base, ref.ltt_base) and np.array_equal(orb.x_base, ref.x_base)
    with pytest.raises(FileNotFoundError):
        flr.read_lisa_orbits(tmp_path / "missing.h5")


def test_h5lite_rejects_other_files(tmp_path):
    from fastlisaresponse_gb300 import h5lite

    bad = tmp_path / "not.h5"
    bad.write_bytes(b"x" * 4096)
    with pytest.raises(h5lite.HDF5FormatError, match="signature"):
        h5lite.File(bad)
    empty = tmp_path / "empty.h5"
    empty.write_bytes(b"")
    with pytest.raises(ValueError):
        h5lite.File(empty)
    with pytest.raises(ValueError, match="reads files only"):
        h5lite.File(bad, "w")


def test_writer_checksum_known_answers():
    """The test writer's lookup3 against the published hashlittle values."""
    from _h5write import lookup3

    assert lookup3(b"") == 0xDEADBEEF
    assert lookup3(b"Four score and seven years ago") == 0x17770551
    assert lookup3(b"Four score and seven years ago", 1) == 0xCD628161


@pytest.mark.parametrize("style", ["v0", "v2"])
def test_h5lite_dataset_forms(tmp_path, style):
    """Compact and scalar datasets, integers of every width and byte order,
    fixed-length strings, and attribute arrays."""
    from _h5write import Writer

    from fastlisaresponse_gb300 import h5lite

    rng = np.random.default_rng(4)
    w = Writer(style)
    forms = {
        "i1": rng.integers(-100, 100, 7).astype("i1"),
        "u2be": rng.integers(0, 60000, (3, 4)).astype(">u2"),
        "i4": rng.integers(-2**30, 2**30, 9).astype("<i4"),
        "u8": rng.integers(0, 2**62, 5).astype("<u8"),
        "f4be": rng.normal(size=6).astype(">f4"),
        "scalar": np.array(2.5),
        "names": np.array([b"tcb", b"tps", b"x"], dtype="S4"),
    }
    for name, arr in forms.items():
        w.dataset(f"forms/{name}", arr, compact=name in ("i1", "scalar", "names"))
    w.dataset("forms/chunked_i4", forms["i4"], chunks=(4,))
    w.root["attrs"].update({"label": np.array(b"LISA", dtype="S8"), "ints": np.arange(4),
                            "dt": 10.0})
    path = tmp_path / f"forms_{style}.h5"
    w.save(path)
    with h5lite.File(path) as f:
        for name, arr in forms.items():
            ds = f["forms"][name]
            got = ds[()]
            assert ds.shape == arr.shape
            assert np.array_equal(got, arr) and got.dtype == arr.dtype.newbyteorder("=")
        assert np.array_equal(f["forms/chunked_i4"][()], forms["i4"])
        assert f.attrs["label"] == b"LISA" and np.array_equal(f.attrs["ints"], np.arange(4))
        assert sorted(f["forms"].keys()) == sorted(list(forms) + ["chunked_i4"])
        assert len(f["forms"]) == len(forms) + 1 and "dt" in f.attrs
