"""In-tree build of the CUDA library ``_lib/libflr_gb300.so`` (sm_103a only).

Each translation unit is compiled by its own ``nvcc`` process (in parallel),
then linked into one shared library with the C ABI of ``include/flr_gb300.h``.
``flr_plain.cu`` is built with ``--fmad=false``: the plain FP64 kernels must
not contract multiply-adds (their results are bit-identical to the
reference's CPU arithmetic).
"""

from __future__ import annotations

import os
import shutil
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.normpath(os.path.join(PKG_DIR, "..", "csrc"))
INCLUDE = os.path.normpath(os.path.join(PKG_DIR, "..", "..", "include"))
LIB_DIR = os.path.join(PKG_DIR, "_lib")
OBJ_DIR = os.path.join(LIB_DIR, "obj")
LIB_PATH = os.path.join(LIB_DIR, "libflr_gb300.so")
# the benchmark's arithmetic-pipe probe: a library of its own, not the product's
PROBE_SRC = os.path.join(CSRC, "probe", "flr_probe.cu")
PROBE_LIB_PATH = os.path.join(LIB_DIR, "libflr_probe.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", CSRC, "-I", INCLUDE]

# translation unit -> extra nvcc flags
SOURCES = {
    "flr_plain.cu": ["--fmad=false"],
    "flr_capi.cu": [],
    "flr_noalloc.cu": ["--fmad=false"],
    "flr_fused.cu": ["--fmad=false"],
    "flr_fused_d2.cu": ["--fmad=false"],
    "flr_fused_server.cu": ["--fmad=false"],
    "flr_fused_t0.cu": ["--fmad=false"],
    "flr_batch.cu": [],
    "flr_waveform.cu": ["--fmad=false"],
}

_lock = threading.Lock()


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libflr_gb300.so")
    return cand


def _inputs() -> list:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)
             if f.endswith((".cu", ".cuh", ".h"))]
    files += [PROBE_SRC, os.path.join(CSRC, "probe", "flr_probe.h")]
    files += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return files


def needs_build() -> bool:
    if not os.path.exists(LIB_PATH) or not os.path.exists(PROBE_LIB_PATH):
        return True
    built = min(os.path.getmtime(LIB_PATH), os.path.getmtime(PROBE_LIB_PATH))
    return any(os.path.getmtime(f) > built for f in _inputs()) or \
        os.path.getmtime(__file__) > built


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile the library if any source is newer than it; returns its path."""
    with _lock:
        if not force and not needs_build():
            return LIB_PATH
        os.makedirs(OBJ_DIR, exist_ok=True)
        nvcc = _nvcc()

        def compile_one(item):
            src, extra = item
            obj = os.path.join(OBJ_DIR, src.replace(".cu", ".o"))
            cmd = [nvcc, *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            res = subprocess.run(cmd, capture_output=True, text=True)
            if res.returncode != 0:
                raise RuntimeError(f"nvcc failed on {src}:\n{res.stdout}\n{res.stderr}")
            if verbose and (res.stdout or res.stderr):
                print(res.stdout + res.stderr)
            return obj

        def build_probe():
            tmp = PROBE_LIB_PATH + ".tmp"
            cmd = [nvcc, *ARCH, *COMMON, "-shared", PROBE_SRC, "-o", tmp]
            res = subprocess.run(cmd, capture_output=True, text=True)
            if res.returncode != 0:
                raise RuntimeError(f"nvcc failed on the probe:\n{res.stdout}\n{res.stderr}")
            os.replace(tmp, PROBE_LIB_PATH)

        with ThreadPoolExecutor(max_workers=len(SOURCES) + 1) as pool:
            probe = pool.submit(build_probe)
            objs = list(pool.map(compile_one, SOURCES.items()))
            probe.result()
        tmp = LIB_PATH + ".tmp"
        cmd = [nvcc, *ARCH, "-shared", *objs, "-o", tmp]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB_PATH)
        return LIB_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
