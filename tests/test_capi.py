"""The C-ABI library builds, loads and exports every symbol its header
declares (no GPU needed: no kernel is launched)."""

import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "flr_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(flr_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    import fastlisaresponse_gb300 as flr

    flr.build()
    return ctypes.CDLL(flr.library_path())


def test_header_declares_the_reference_replacements():
    syms = declared_symbols()
    for name in ("flr_orbits_create", "flr_orbits_destroy", "flr_get_response",
                 "flr_get_tdi_delays", "flr_last_error", "flr_version"):
        assert name in syms


def test_library_exports_all_declared_symbols(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_version_and_error_strings(lib):
    lib.flr_version.restype = ctypes.c_char_p
    assert lib.flr_version().decode().startswith("flr_gb300")
    lib.flr_last_error.restype = ctypes.c_char_p
    assert isinstance(lib.flr_last_error(), bytes)


def test_argument_errors_before_any_device_work(lib):
    """Invalid arguments are rejected on the host, before CUDA is touched."""
    out = ctypes.c_void_p()
    lib.flr_orbits_create.argtypes = [ctypes.c_double, ctypes.c_int] + [ctypes.c_void_p] * 6 + \
        [ctypes.c_double, ctypes.POINTER(ctypes.c_void_p)]
    rc = lib.flr_orbits_create(1e4, 1, None, None, None, None, None, None, 2.5e9,
                               ctypes.byref(out))
    assert rc == -1
    lib.flr_last_error.restype = ctypes.c_char_p
    assert b"N >= 2" in lib.flr_last_error()
    rc = lib.flr_orbits_create(-1.0, 10, None, None, None, None, None, None, 2.5e9,
                               ctypes.byref(out))
    assert rc == -1 and b"dt" in lib.flr_last_error()


def test_no_oracle_in_the_product():
    """The product library links nothing from oracle/ (no CPU fallback)."""
    import fastlisaresponse_gb300 as flr

    with open(flr.library_path(), "rb") as fh:
        blob = fh.read()
    assert b"orc_get_response" not in blob and b"flr_ref_get_response" not in blob
    pkg = os.path.join(ROOT, "lisa-on-gpu_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h")):
                text = open(os.path.join(dirpath, f)).read()
                assert "import oracle" not in text and "from oracle" not in text, f
                assert "refdrive" not in text, f


def test_probe_is_not_in_the_product_library(lib):
    """The benchmark's pipe probe is built into its own library."""
    from fastlisaresponse_gb300 import _build

    assert not hasattr(lib, "flr_probe_pipe_rate")
    probe = ctypes.CDLL(_build.PROBE_LIB_PATH)
    assert hasattr(probe, "flr_probe_pipe_rate")
