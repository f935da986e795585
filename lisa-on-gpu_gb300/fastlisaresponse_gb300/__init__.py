"""fastlisaresponse_gb300 -- the LISA time-domain response and TDI on GB300.

Drop-in for the reference package ``fastlisaresponse``'s response path:
``pyResponseTDI`` and ``ResponseWrapper`` keep the reference's constructor and
call signatures and run hand-written sm_103a CUDA kernels (``libflr_gb300.so``,
C ABI in ``include/flr_gb300.h``) through ctypes.  There is no CPU backend.
"""

from ._build import build, needs_build
from ._lib import FLRError, describe_status, library_path
from . import autotune
from .batch import BatchedResponseTDI, BatchGraph
from .binding import LISAResponseWrap, LISAResponseWrapGPU, OrbitsWrap, OrbitsWrapGPU_responselisa
from .orbits import EqualArmlengthOrbits, KeplerianOrbits, Orbits, read_lisa_orbits
from .serve import Request, ResponseServer
from .serve_device import DeviceLoopServer, DeviceTicket
from .response import (ResponseWrapper, lagrange_tables, pyResponseTDI, sky_basis,
                       tdi_unit_tables)
from .utils import AET, HostArray, get_overlap
from .waveforms import GBWave, gb_waveform, time_grid

__version__ = "0.1.0"

__all__ = [
    "AET", "BatchGraph", "DeviceLoopServer", "DeviceTicket", "HostArray", "BatchedResponseTDI", "EqualArmlengthOrbits", "FLRError", "GBWave", "KeplerianOrbits",
    "LISAResponseWrap", "LISAResponseWrapGPU", "Orbits", "OrbitsWrap",
    "OrbitsWrapGPU_responselisa", "ResponseWrapper", "autotune", "build", "describe_status",
    "gb_waveform", "get_overlap", "lagrange_tables", "library_path", "needs_build",
    "pyResponseTDI", "read_lisa_orbits", "Request", "ResponseServer", "sky_basis",
    "tdi_unit_tables", "time_grid",
]
