"""Helpers of the response path: XYZ -> AET, the overlap metric the
reference's tests use, and page-locked NumPy host arrays for asynchronous
host-device copies."""

from __future__ import annotations

import ctypes
import math
import weakref

import numpy as np

try:
    import torch
except ImportError:  # pragma: no cover
    torch = None


def AET(X, Y, Z):
    """A, E, T from X, Y, Z as lisaanalysistools defines them (the reference
    calls ``lisatools.utils.utility.AET`` at response.py:665):
    A = (Z - X)/sqrt(2), E = (X - 2Y + Z)/sqrt(6), T = (X + Y + Z)/sqrt(3).

    Works on numpy arrays and torch tensors.  For CUDA tensors the constants
    are 0-d device tensors: torch divides by a host scalar as a multiplication
    by its reciprocal, which is not the correctly rounded quotient numpy
    computes."""
    if torch is not None and isinstance(X, torch.Tensor) and X.is_cuda:
        def c(v):
            return torch.tensor(v, dtype=X.dtype, device=X.device)
        two, r2, r6, r3 = c(2.0), c(math.sqrt(2.0)), c(math.sqrt(6.0)), c(math.sqrt(3.0))
        return ((Z - X) / r2, (X - two * Y + Z) / r6, (X + Y + Z) / r3)
    return ((Z - X) / math.sqrt(2.0), (X - 2.0 * Y + Z) / math.sqrt(6.0),
            (X + Y + Z) / math.sqrt(3.0))


def get_overlap(sig1, sig2, phase_maximize=False, use_gpu=False):
    """Normalised time-domain overlap averaged over channels
    (``src/fastlisaresponse/utils/utility.py:16-82``).

    ``sig1``/``sig2`` are a list of channels or a single 1-D array (numpy or
    torch).  Returns the real part of the mean complex overlap, or its modulus
    with ``phase_maximize``."""
    def as_list(sig):
        if isinstance(sig, (list, tuple)):
            return list(sig)
        if torch is not None and isinstance(sig, torch.Tensor):
            return [sig] if sig.ndim < 2 else list(sig)
        if isinstance(sig, np.ndarray):
            return [sig] if sig.ndim < 2 else list(sig)
        raise ValueError("sig1 must be list of or single xp.ndarray.")

    s1, s2 = as_list(sig1), as_list(sig2)
    assert len(s1) == len(s2)
    assert len(s1[0]) == len(s2[0])
    overlap = 0.0 + 0.0j
    for a, b in zip(s1, s2):
        if torch is not None and (isinstance(a, torch.Tensor) or isinstance(b, torch.Tensor)):
            a = torch.as_tensor(a, dtype=torch.float64)
            b = torch.as_tensor(b, dtype=torch.float64, device=a.device)
            fa, fb = torch.fft.rfft(a), torch.fft.rfft(b)
            num = torch.dot(fa.conj(), fb)
            den = torch.sqrt(torch.dot(fa.conj(), fa) * torch.dot(fb.conj(), fb))
            overlap += complex((num / den).item())
        else:
            fa, fb = np.fft.rfft(np.asarray(a)), np.fft.rfft(np.asarray(b))
            overlap += np.dot(fa.conj(), fb) / np.sqrt(np.dot(fa.conj(), fa) * np.dot(fb.conj(), fb))
    overlap /= len(s1)
    if phase_maximize:
        return float(abs(overlap))
    return float(np.real(overlap))


class HostArray:
    """A NumPy array in page-locked host memory of exactly its size
    (cudaHostAlloc through ``flr_host_alloc``; a caching allocator would round
    it up to a power of two): copies between it and the GPU run
    asynchronously on the copy engines (``BatchedResponseTDI.run_host``).
    The memory is freed when the last view of it (``.array``, ``.tensor`` or
    anything made from them) is gone; :meth:`release` (or leaving a ``with``
    block) drops this object's own references.

    ``HostArray(shape, dtype).array`` is the NumPy view;
    ``.tensor`` a CPU torch tensor on the same memory."""

    def __init__(self, shape, dtype=np.float64):
        from . import _lib

        self.shape = tuple(np.atleast_1d(shape).tolist())
        self.dtype = np.dtype(dtype)
        count = int(np.prod(self.shape))
        nbytes = count * self.dtype.itemsize
        lib = _lib.lib()
        ptr = ctypes.c_void_p()
        _lib.check(lib.flr_host_alloc(max(nbytes, 1), ctypes.byref(ptr)))
        raw = (ctypes.c_char * max(nbytes, 1)).from_address(ptr.value)
        # freed with the ctypes block, which every NumPy/torch view keeps alive
        weakref.finalize(raw, lib.flr_host_free, ptr.value)
        self.array = np.frombuffer(raw, dtype=self.dtype, count=count).reshape(self.shape)
        self.tensor = torch.from_numpy(self.array)

    def release(self):
        self.array = None
        self.tensor = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.release()
        return False
