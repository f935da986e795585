"""Time the reference's own CPU path against the C restatement -- TEST INFRASTRUCTURE.

Run where the reference checkout exists (FLR_REFERENCE_ROOT, or the location
``oracle/Makefile`` names):

    python oracle/time_reference.py [--samples N] [--repeats R]

Both evaluate the same work on one core: one galactic binary of the batching
configuration's kind (dt = 10 s, equal-arm orbits, 2nd-generation TDI XYZ,
Lagrange order 25), N output samples plus the edge zones, get_projections then
get_tdi_delays:

* reference: the reference's ``pyResponseTDI`` imported from its source
  (``refdrive.import_reference_response``; its host tables and calls as they
  are) on its ``LISAResponse.cu`` CPU branch compiled by ``make -C oracle
  timing`` at -O3 and at -O3 -march=native (the flags of its CMake build);
* port: ``oracle.OracleResponseTDI`` on ``flr_oracle.c`` at -O3 (the build the
  benchmark's CPU baseline and reference arm time) and -O3 -march=native.

Prints one JSON line: output samples/s of each, best of R, and the
reference/port ratios.  The outputs of the two are compared as well (the
parity builds are bit-identical; the timing builds may contract FMAs).
"""

from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(HERE, "..", "lisa-on-gpu_gb300"))

import oracle  # noqa: E402
import refdrive  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--samples", type=int, default=2**17)
    ap.add_argument("--repeats", type=int, default=3)
    args = ap.parse_args()
    from fastlisaresponse_gb300 import orbits as om
    from fastlisaresponse_gb300 import waveforms as wf

    dt, order, tdi = 10.0, 25, "2nd generation"
    n = args.samples + 2 * int(1e4 / dt)
    orb = om.EqualArmlengthOrbits(t_max=(np.floor(n * dt / 1e4) + 3) * 1e4)
    h = np.ascontiguousarray(wf.gb_waveform(3e-22, 3e-3, 1e-15, 0.6, 1.2, 0.4,
                                            np.arange(n) * dt))
    lam, beta = 1.1, 0.4

    def best(fn):
        ts = []
        for _ in range(args.repeats):
            t0 = time.perf_counter()
            out = fn()
            ts.append(time.perf_counter() - t0)
        return args.samples / min(ts), out

    res, outs = {}, {}
    ref = refdrive.import_reference_response()
    for variant in ("o3", "native"):
        refdrive.use_variant(variant)
        resp = ref.pyResponseTDI(1.0 / dt, n, order=order, tdi=tdi,
                                 orbits=refdrive.StubOrbits(orb))

        def run_ref():
            resp.get_projections(h, lam, beta, t0=0.0, t_buffer=1e4)
            return np.stack(resp.get_tdi_delays())

        res[f"reference_{variant}"], outs[f"reference_{variant}"] = best(run_ref)
    for variant in ("o3", "native"):
        o = oracle.OracleResponseTDI(1.0 / dt, n, orb.pycppdetector_args, orb.x_base,
                                     order=order, tdi=tdi, variant=variant)

        def run_port():
            o.get_projections(h, lam, beta, t0=0.0, t_buffer=1e4)
            return np.stack(o.get_tdi_delays())

        res[f"port_{variant}"], outs[f"port_{variant}"] = best(run_port)
    ts = int(1e4 / dt)
    sl = slice(ts, n - ts)
    for v in ("o3", "native"):
        a, b = outs[f"reference_{v}"][:, sl], outs[f"port_{v}"][:, sl]
        res[f"rel_l2_{v}"] = float(np.linalg.norm(a - b) / np.linalg.norm(b))
        res[f"reference_over_port_{v}"] = res[f"reference_{v}"] / res[f"port_{v}"]
    res["samples"] = args.samples
    res["host"] = os.uname().machine
    print(json.dumps(res))


if __name__ == "__main__":
    main()
