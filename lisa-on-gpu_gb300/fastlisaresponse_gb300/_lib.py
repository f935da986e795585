"""ctypes loader of ``libflr_gb300.so`` and the argument types of its C ABI.

There is no fallback: if the library is missing or cannot be loaded, every
entry point raises.  Build it with ``fastlisaresponse_gb300.build()``.
"""

from __future__ import annotations

import ctypes
import threading

from . import _build

FLR_OK = 0
FLR_E_INVALID_ARGUMENT = -1
FLR_E_CUDA = -2
FLR_E_NO_ORBITS = -3
FLR_E_UNSUPPORTED = -4

STATUS_BITS = {
    0x1: "tap window outside the input",
    0x2: "A-table index out of range",
    0x4: "unknown link number",
    0x8: "TDI channel out of range",
    0x10: "a staging copy completed late (its work item's outputs are NaN)",
    0x20: "a staging copy never completed (discard every output of the batch)",
}


class FLRError(RuntimeError):
    """A CUDA-side failure reported by libflr_gb300."""


_lib = None
_lock = threading.Lock()

_d = ctypes.c_double
_i = ctypes.c_int
_p = ctypes.c_void_p

_SIGNATURES = {
    "flr_version": (ctypes.c_char_p, []),
    "flr_host_alloc": (_i, [ctypes.c_size_t, ctypes.POINTER(_p)]),
    "flr_host_free": (_i, [_p]),
    "flr_last_error": (ctypes.c_char_p, []),
    "flr_orbits_create": (_i, [_d, _i, _p, _p, _p, _p, _p, _p, _d, ctypes.POINTER(_p)]),
    "flr_orbits_destroy": (_i, [_p]),
    "flr_orbits_status": (_i, [_p, ctypes.POINTER(ctypes.c_uint32), _i, _p]),
    "flr_get_response": (_i, [_p, _p, _p, _p, _p, _p, _d, _i, _p, _i, _i, _d, _i, _p, _d, _i, _p,
                              _i, _p]),
    "flr_get_tdi_delays": (_i, [_p, _p, _p, _i, _i, _p, _p, _p, _p, _p, _p, _p, _i, _i, _i, _d,
                                _i, _p, _d, _i, _p, _i, _p]),
    "flr_response_delay_indices": (_i, [_p, _p, _p, _p, _p, _i, _d, _i, _p]),
    "flr_tdi_delay_indices": (_i, [_p, _p, _i, _p, _p, _p, _p, _i, _d, _i, _p]),
    "flr_get_tdi_delays_aet": (_i, [_p, _p, _p, _i, _i, _p, _p, _p, _p, _p, _p, _p, _i, _i, _i,
                                    _d, _i, _p, _d, _i, _p, _i, _p, _i, _p]),
    "flr_xyz_to_aet": (_i, [_p, _p, _i, _i, _i, _p]),
}


def library_path() -> str:
    return _build.LIB_PATH


def lib() -> ctypes.CDLL:
    """The loaded library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            import os

            if not os.path.exists(_build.LIB_PATH):
                raise ImportError(
                    f"{_build.LIB_PATH} is not built; run fastlisaresponse_gb300.build() "
                    "(nvcc, sm_103a). There is no CPU fallback.")
            handle = ctypes.CDLL(_build.LIB_PATH)
            for name, (res, args) in _SIGNATURES.items():
                fn = getattr(handle, name)
                fn.restype = res
                fn.argtypes = args
            _lib = handle
    return _lib


def check(rc: int) -> None:
    """Turn a non-zero return code into ValueError (argument errors, as the
    reference's binding raises) or FLRError (CUDA errors)."""
    if rc == FLR_OK:
        return
    msg = lib().flr_last_error().decode(errors="replace")
    if rc in (FLR_E_INVALID_ARGUMENT, FLR_E_NO_ORBITS, FLR_E_UNSUPPORTED):
        raise ValueError(msg)
    raise FLRError(msg)


class nvtx_range:
    """NVTX range around a library call (visible in Nsight Systems); a no-op
    where NVTX is unavailable."""

    def __init__(self, name: str):
        self.name = name
        self.pushed = False

    def __enter__(self):
        try:
            import torch

            torch.cuda.nvtx.range_push(self.name)
            self.pushed = True
        except Exception:
            self.pushed = False
        return self

    def __exit__(self, *exc):
        if self.pushed:
            try:
                import torch

                torch.cuda.nvtx.range_pop()
            except Exception:
                pass
        return False


def describe_status(bits: int) -> str:
    return ", ".join(text for bit, text in STATUS_BITS.items() if bits & bit) or "ok"
