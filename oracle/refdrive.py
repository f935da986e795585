"""Drive the reference's own code on the CPU -- TEST INFRASTRUCTURE ONLY.

Two pieces, both usable only where the reference checkout exists (this build
container; not the GPU host):

* :func:`ref_lib` -- ctypes handle on ``oracle/_ref/libflr_ref.so``, the
  reference's ``LISAResponse.cu`` compiled as C++ (its CPU branch) by
  ``make -C oracle ref`` against the shim headers in ``oracle/ref_shim``.
* :func:`import_reference_response` -- the reference's
  ``src/fastlisaresponse/response.py`` imported from its source file, with
  stand-ins registered for the modules it imports but that are absent here:
  ``h5py`` (imported, unused), ``lisatools.detector`` (``Orbits``,
  ``EqualArmlengthOrbits``), ``lisatools.utils.utility.AET`` and
  ``fastlisaresponse.utils.parallelbase`` (the gpubackendtools backend
  registry).  The stand-in backend's ``OrbitsWrap``/``LISAResponseWrap``
  forward to :func:`ref_lib` with the CPU binding's length checks
  (``binding_flr.hpp:61-76``).  Everything else -- A/E tables, TDI tables,
  buffers, sky basis, the calls and their arguments -- is the reference's code.

Used by ``tests/golden/make_golden.py`` and ``tests/test_oracle.py``.
"""

from __future__ import annotations

import ctypes
import importlib.util
import os
import subprocess
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _reference_root() -> str:
    """The reference checkout: FLR_REFERENCE_ROOT, else the location the
    oracle's Makefile (the recipe that compiles the checkout) names."""
    env = os.environ.get("FLR_REFERENCE_ROOT")
    if env:
        return env
    try:
        res = subprocess.run(["make", "-s", "-C", HERE, "print-ref-root"], capture_output=True,
                             text=True, check=True)
        return res.stdout.strip()
    except (OSError, subprocess.CalledProcessError):
        return ""


REF_ROOT = _reference_root()
REF_PKG = os.path.join(REF_ROOT, "src", "fastlisaresponse")
REF_LIB = os.path.join(HERE, "_ref", "libflr_ref.so")
# build of the reference's code ref_lib() loads: "parity" (-O2
# -ffp-contract=off, the pinning build) or the timing builds "o3" / "native"
REF_VARIANTS = {"parity": ("ref", "libflr_ref.so"), "o3": ("timing", "libflr_ref_o3.so"),
                "native": ("timing", "libflr_ref_native.so")}


def available() -> bool:
    return os.path.exists(os.path.join(REF_PKG, "cutils", "LISAResponse.cu"))


_lib = None
_variant = "parity"


def use_variant(name: str) -> None:
    """Select the build of the reference's code that later calls use."""
    global _lib, _variant
    if name not in REF_VARIANTS:
        raise ValueError(f"variant must be one of {sorted(REF_VARIANTS)}")
    if name != _variant:
        _variant, _lib = name, None


def ref_lib() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not available():
        raise RuntimeError("the reference sources are not available here")
    target, fname = REF_VARIANTS[_variant]
    subprocess.run(["make", "-s", "-C", HERE, target,
                    f"REF_DIR={os.path.join(REF_PKG, 'cutils')}"], check=True)
    lib = ctypes.CDLL(os.path.join(HERE, "_ref", fname))
    d, i, p = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
    orb = [d, i, p, p, p, p, p, p, d]
    lib.flr_ref_get_response.argtypes = orb + [p, p, p, p, p, d, i, p, i, i, d, i, p, d, i, p, i]
    lib.flr_ref_get_response.restype = i
    lib.flr_ref_get_tdi_delays.argtypes = orb + [p, p, i, i, p, p, p, p, p, p, p, i, i, i, d, i,
                                                 p, d, i, p, i]
    lib.flr_ref_get_tdi_delays.restype = i
    _lib = lib
    return lib


def _checked(arr, dtype, name, n=None, mult=1):
    arr = np.asarray(arr)
    if arr.dtype != dtype or not arr.flags.c_contiguous:
        raise TypeError(f"{name}: expected contiguous {np.dtype(dtype)}")
    if n is not None and arr.size != n * mult:
        raise ValueError(f"{name}: input arrays have the incorrect length. Should be {n * mult}. "
                         f"It's length is {arr.size}.")
    return arr


class RefOrbitsWrap:
    """Stand-in for ``OrbitsWrapCPU_responselisa`` (binding_flr.hpp:32-59)."""

    def __init__(self, dt, N, n_arr, ltt_arr, x_arr, links, sc_r, sc_e, armlength):
        self.dt, self.N, self.armlength = float(dt), int(N), float(armlength)
        self.n_arr = _checked(n_arr, np.float64, "n_arr", N, 18)
        self.ltt_arr = _checked(ltt_arr, np.float64, "ltt_arr", N, 6)
        self.x_arr = _checked(x_arr, np.float64, "x_arr", N, 9)
        self.links = _checked(np.asarray(links, dtype=np.int32), np.int32, "links", 6)
        self.sc_r = _checked(np.asarray(sc_r, dtype=np.int32), np.int32, "sc_r", 6)
        self.sc_e = _checked(np.asarray(sc_e, dtype=np.int32), np.int32, "sc_e", 6)

    def args(self):
        return [self.dt, self.N, self.n_arr.ctypes.data, self.ltt_arr.ctypes.data,
                self.x_arr.ctypes.data, self.links.ctypes.data, self.sc_r.ctypes.data,
                self.sc_e.ctypes.data, self.armlength]


class RefResponseWrap:
    """Stand-in for ``LISAResponseWrapCPU`` (binding_flr.hpp:78-142,
    binding_flr.cxx:16-58) calling the reference's compiled CPU code."""

    def __init__(self, orbits: RefOrbitsWrap):
        self.orbits = orbits

    def get_response_wrap(self, y_gw, t_data, k_in, u_in, v_in, dt, num_delays, input_in,
                          num_inputs, order, sampling_frequency, buffer_integer, A_in, deps,
                          num_A, E_in, projections_start_ind):
        y = _checked(y_gw, np.float64, "y_gw", num_delays, 6)
        t = _checked(t_data, np.float64, "t_data", num_delays)
        k = _checked(k_in, np.float64, "k_in", 3)
        u = _checked(u_in, np.float64, "u_in", 3)
        v = _checked(v_in, np.float64, "v_in", 3)
        h = _checked(input_in, np.complex128, "input_in")
        A = _checked(A_in, np.float64, "A_in", num_A)
        E = _checked(E_in, np.float64, "E_in")
        ref_lib().flr_ref_get_response(*self.orbits.args(), y.ctypes.data, t.ctypes.data,
                                       k.ctypes.data, u.ctypes.data, v.ctypes.data, float(dt),
                                       int(num_delays), h.ctypes.data, int(num_inputs),
                                       int(order), float(sampling_frequency),
                                       int(buffer_integer), A.ctypes.data, float(deps),
                                       int(num_A), E.ctypes.data, int(projections_start_ind))

    def get_tdi_delays_wrap(self, delayed_links, input_links, num_inputs, num_delays, t_arr,
                            unit_starts, unit_lengths, tdi_base_link, tdi_link_combinations,
                            tdi_signs_in, channels, num_units, num_channels, order,
                            sampling_frequency, buffer_integer, A_in, deps, num_A, E_in,
                            tdi_start_ind):
        out = _checked(delayed_links, np.float64, "delayed_links", num_delays, 3)
        y = _checked(input_links, np.float64, "input_links", num_inputs, 6)
        t = _checked(t_arr, np.float64, "t_arr", num_delays)
        us = _checked(np.asarray(unit_starts), np.int32, "unit_starts", num_units)
        ul = _checked(np.asarray(unit_lengths), np.int32, "unit_lengths", num_units)
        bl = _checked(tdi_base_link, np.int32, "tdi_base_link")
        lc = _checked(tdi_link_combinations, np.int32, "tdi_link_combinations")
        sg = _checked(tdi_signs_in, np.float64, "tdi_signs_in")
        ch = _checked(channels, np.int32, "channels")
        A = _checked(A_in, np.float64, "A_in", num_A)
        E = _checked(E_in, np.float64, "E_in")
        ref_lib().flr_ref_get_tdi_delays(*self.orbits.args(), out.ctypes.data, y.ctypes.data,
                                         int(num_inputs), int(num_delays), t.ctypes.data,
                                         us.ctypes.data, ul.ctypes.data, bl.ctypes.data,
                                         lc.ctypes.data, sg.ctypes.data, ch.ctypes.data,
                                         int(num_units), int(num_channels), int(order),
                                         float(sampling_frequency), int(buffer_integer),
                                         A.ctypes.data, float(deps), int(num_A), E.ctypes.data,
                                         int(tdi_start_ind))


class StubOrbits:
    """``lisatools.detector.Orbits`` stand-in wrapping precomputed tables.

    ``tables`` is any object with ``t_base``, ``x_base``, ``t`` and
    ``pycppdetector_args`` (e.g. an orbit object of the product package)."""

    LINKS = [12, 23, 31, 13, 32, 21]

    def __init__(self, tables=None):
        self._tables = tables
        self.backend = types.SimpleNamespace(name="lisatools_cpu")

    @property
    def configured(self):
        return True

    def configure(self, *args, **kwargs):
        return self

    def __getattr__(self, name):
        if name.startswith("_"):
            raise AttributeError(name)
        return getattr(self._tables, name)


def _lisatools_aet(X, Y, Z):
    return ((Z - X) / np.sqrt(2.0), (X - 2.0 * Y + Z) / np.sqrt(6.0), (X + Y + Z) / np.sqrt(3.0))


_module = None


def import_reference_response():
    """The reference's ``fastlisaresponse.response`` module, imported from its
    source with stand-ins for the absent third-party modules."""
    global _module
    if _module is not None:
        return _module
    if not available():
        raise RuntimeError("the reference sources are not available here")

    backend = types.SimpleNamespace(name="fastlisaresponse_cpu", xp=np,
                                    OrbitsWrap=RefOrbitsWrap, LISAResponseWrap=RefResponseWrap)

    class FastLISAResponseParallelModule:
        def __init__(self, force_backend=None):
            self.backend = backend

    stubs = {
        "h5py": types.ModuleType("h5py"),
        "lisatools": types.ModuleType("lisatools"),
        "lisatools.detector": types.ModuleType("lisatools.detector"),
        "lisatools.utils": types.ModuleType("lisatools.utils"),
        "lisatools.utils.utility": types.ModuleType("lisatools.utils.utility"),
        "fastlisaresponse": types.ModuleType("fastlisaresponse"),
        "fastlisaresponse.utils": types.ModuleType("fastlisaresponse.utils"),
        "fastlisaresponse.utils.parallelbase": types.ModuleType(
            "fastlisaresponse.utils.parallelbase"),
    }
    stubs["lisatools.detector"].Orbits = StubOrbits
    stubs["lisatools.detector"].EqualArmlengthOrbits = StubOrbits
    stubs["lisatools.utils.utility"].AET = _lisatools_aet
    stubs["fastlisaresponse"].__path__ = [REF_PKG]
    stubs["fastlisaresponse.utils"].__path__ = []
    stubs["fastlisaresponse.utils.parallelbase"].FastLISAResponseParallelModule = \
        FastLISAResponseParallelModule
    saved = {name: sys.modules.get(name) for name in stubs}
    sys.modules.update(stubs)
    try:
        spec = importlib.util.spec_from_file_location("fastlisaresponse.response",
                                                      os.path.join(REF_PKG, "response.py"))
        module = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(module)
    finally:
        for name, old in saved.items():
            if old is None:
                sys.modules.pop(name, None)
            else:
                sys.modules[name] = old
    module.StubOrbits = StubOrbits
    _module = module
    return module
