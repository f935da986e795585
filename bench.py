#!/usr/bin/env python3
"""Benchmark of the LISA time-domain response + TDI on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload NAME] [--no-cpu-baseline] [--batch-sources S]
                    [--precision-sources P] [--serve-requests R]

One step = one pass of the hot path over one source: the six link projections
and the TDI channels.  The default workload is one galactic binary observed
for 1 yr at dt = 5 s (6,311,629 samples) with flexing Keplerian orbits,
2nd-generation TDI XYZ and Lagrange order 25.  The headline runs it through
the mixed-precision fused kernel (BatchedResponseTDI, autotuned tile, 8
tile-aligned launches over two streams per step; FP64 delays and bit-exact
indices, double-float taps); the plain FP64 drop-in path
(pyResponseTDI, bit-identical to the reference's CPU arithmetic) is timed on
the same source beside it.

Printed on rank 0, one JSON line:
  value       output samples/s with the input resident in HBM (CUDA events
              around each step, L2 flushed before each, max over ranks);
  e2e         the same metric through BatchedResponseTDI.run_host with the
              input in pinned host memory and X/Y/Z copied back to pinned host
              memory, the copies overlapped with the launches;
  roofline    the fused kernel's FP64 index-path operations per second
              against the FP64 FMA peak measured at start-up (and its HBM
              fraction against MEASURED_PEAKS.json); plain_fp64.roofline the
              same for the plain path's dominant kernel;
  cpu_baseline  the C oracle on one host core, on a bounded slice;
  batched / precision / serving  the batching, precision and serving
              configurations (see their sections).
With --impl reference the CPU implementation is timed instead (all host
cores, one independent source per process) and printed with "impl":
"reference".  Under torchrun every rank runs its own source and its share of
the batch (weak scaling); the reference arm runs on rank 0 only.
"""

from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "lisa-on-gpu_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

YRSID_SI = 31558149.763545603
T_BUFFER = 1e4
METRIC = "response+TDI output samples/s"
UNIT = "samples/s"
SOURCE = dict(A=1e-22, f=2e-3, fdot=1e-14)

WORKLOADS = {
    "1yr_dt5_gen2": dict(
        desc="one galactic binary, 1 yr at dt = 5 s (6,311,629 samples), flexing Keplerian "
             "orbits (arms +-1 %), 2nd-generation TDI XYZ, Lagrange order 25, float64",
        dt=5.0, n=int(YRSID_SI / 5.0), orbits="kepler", tdi="2nd generation", order=25),
    "2p21_dt5_gen2": dict(
        desc="one galactic binary, 2^21 samples at dt = 5 s, flexing Keplerian orbits, "
             "2nd-generation TDI XYZ, Lagrange order 25, float64 (profiling size)",
        dt=5.0, n=2**21, orbits="kepler", tdi="2nd generation", order=25),
    "2p18_dt10_gen1": dict(
        desc="one galactic binary, 2^18 samples at dt = 10 s, rigid equal-arm orbits, "
             "1st-generation TDI XYZ, Lagrange order 25, float64",
        dt=10.0, n=2**18, orbits="equal", tdi="1st generation", order=25),
}
DEFAULT_WORKLOAD = "1yr_dt5_gen2"
CPU_SLICE = 2**20  # samples per source in the CPU measurements (~3 s per pass on one core)
HEADLINE_CHUNKS = 8  # launches per headline step (two streams: last waves overlap)
E2E_CHUNKS = 8       # pieces of the end-to-end step's source (copy/compute overlap)
SERVE_BATCH_SAMPLES = 2**23  # samples per serving batch at most (the server's default)


# ----------------------------------------------------------------------------- setup

def make_source(w: dict, n: int, seed: int):
    from fastlisaresponse_gb300 import orbits as om
    from fastlisaresponse_gb300 import waveforms as wf

    t_max = (math.floor(n * w["dt"] / 1e4) + 3) * 1e4
    orb = om.KeplerianOrbits(t_max=t_max) if w["orbits"] == "kepler" else \
        om.EqualArmlengthOrbits(t_max=t_max)
    rng = np.random.default_rng(seed)
    iota, phi0, psi = math.acos(rng.uniform(-1, 1)), rng.uniform(0, 2 * math.pi), \
        rng.uniform(0, math.pi)
    lam, beta = rng.uniform(0, 2 * math.pi), math.asin(rng.uniform(-1, 1))
    h = wf.gb_waveform(SOURCE["A"], SOURCE["f"], SOURCE["fdot"], iota, phi0, psi,
                       np.arange(n) * w["dt"])
    return orb, np.ascontiguousarray(h), lam, beta


def output_samples(n: int, dt: float) -> int:
    return n - 2 * int(T_BUFFER / dt)


# ------------------------------------------------------------------------ CPU side

_worker_state = {}


def _cpu_worker_init(wname, n, variant):
    import oracle

    w = WORKLOADS[wname]
    orb, h, lam, beta = make_source(w, n, seed=12345)
    o = oracle.OracleResponseTDI(1.0 / w["dt"], n, orb.pycppdetector_args, orb.x_base,
                                 order=w["order"], tdi=w["tdi"], variant=variant)
    _worker_state.update(o=o, h=h, lam=lam, beta=beta)


def _cpu_worker_run(_):
    s = _worker_state
    t0 = time.perf_counter()
    s["o"].get_projections(s["h"], s["lam"], s["beta"], t0=0.0, t_buffer=T_BUFFER)
    s["o"].get_tdi_delays()
    return time.perf_counter() - t0


def cpu_rate(wname: str, cores: int, steps: int, warmup: int, variant: str = "o3"):
    """Samples/s of the CPU oracle over CPU_SLICE-sample sources of the workload's
    configuration, `cores` processes each computing its own source per step."""
    w = WORKLOADS[wname]
    n = CPU_SLICE
    per = output_samples(n, w["dt"])
    ctx = mp.get_context("spawn")
    walls = []
    with ctx.Pool(cores, initializer=_cpu_worker_init, initargs=(wname, n, variant)) as pool:
        for i in range(warmup + steps):
            t0 = time.perf_counter()
            pool.map(_cpu_worker_run, range(cores), chunksize=1)
            if i >= warmup:
                walls.append(time.perf_counter() - t0)
    total = sum(walls)
    return dict(value=per * cores * len(walls) / total, seconds=total,
                ms_per_step=1e3 * total / len(walls), samples_per_step=per * cores)


# ------------------------------------------------------------------------ GPU side

class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str):
        self.gpu_id = gpu_id
        self.lines = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", self.gpu_id], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=5)
        sms, maxes, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sms.append(float(parts[0]))
                maxes.append(float(parts[1]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[4:8]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        if not sms:
            return None
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": max(maxes),
                "reasons": sorted(reasons), "samples": len(sms)}


def measure_fp64_peak(device) -> dict:
    """FP64 FMA, FP64 division and FP32 FMA rates of this GPU from the probe
    kernels of libflr_probe.so (best of 3)."""
    import ctypes

    import torch

    from fastlisaresponse_gb300 import _build

    lib = ctypes.CDLL(_build.PROBE_LIB_PATH)
    lib.flr_probe_pipe_rate.restype = ctypes.c_int
    lib.flr_probe_pipe_rate.argtypes = [ctypes.c_int, ctypes.c_long, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_void_p, ctypes.POINTER(ctypes.c_float),
                                        ctypes.c_void_p]

    sms = torch.cuda.get_device_properties(device).multi_processor_count
    blocks, threads = sms * 8, 256
    sink = torch.zeros(blocks, dtype=torch.float64, device=device)
    stream = ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)
    out = {}
    for kind, name, iters in ((0, "fp64_fma", 4000), (1, "fp64_div", 400), (2, "fp32_fma", 40000)):
        best = None
        for _ in range(3):
            ms = ctypes.c_float()
            rc = lib.flr_probe_pipe_rate(kind, iters, blocks, threads, sink.data_ptr(),
                                         ctypes.byref(ms), stream)
            if rc != 0:
                raise RuntimeError(f"probe kind {kind} failed ({rc})")
            rate = blocks * threads * iters * 8 / (ms.value * 1e-3)
            best = rate if best is None else max(best, rate)
        out[name] = best
    out["sms"] = sms
    return out


def gpu_uuid(device) -> str:
    import torch

    props = torch.cuda.get_device_properties(device)
    uuid = getattr(props, "uuid", None)
    if uuid is not None:
        s = str(uuid)
        return s if s.startswith("GPU-") else "GPU-" + s
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
    first = vis.split(",")[device.index] if vis else str(device.index)
    return first


def load_traffic(kernel: str, workload: str):
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as fh:
        table = json.load(fh)
    entry = table.get(f"{kernel}@{workload}")
    return None if entry is None else entry.get("bytes_per_launch")


def _events():
    import torch

    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


_FLUSH = {}


def _flush_l2(device):
    """Write 256 MB (twice the L2) so that a step starts with a cold L2."""
    import torch

    buf = _FLUSH.get(device)
    if buf is None:
        buf = _FLUSH[device] = torch.empty(2**25, dtype=torch.float64, device=device)
    buf.fill_(1.0)


def _timed(fn, steps, warmup, device, kernel_events=None):
    """Run fn warmup + steps times; CUDA-event time of the steps [s].

    Before each timed step the L2 is flushed and the stream is held for ~1 ms
    (torch.cuda._sleep) while the host queues the step, so the events bracket
    device work only; the step times are summed."""
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize(device)
    if kernel_events is not None:
        kernel_events["on"] = True
    pairs = []
    for _ in range(steps):
        _flush_l2(device)
        torch.cuda._sleep(2_000_000)
        e0, e1 = _events()
        e0.record()
        fn()
        e1.record()
        pairs.append((e0, e1))
    torch.cuda.synchronize(device)
    if kernel_events is not None:
        kernel_events["on"] = False
    return sum(a.elapsed_time(b) for a, b in pairs) * 1e-3


def _rel_l2_rows(got, want):
    import torch

    worst = 0.0
    for r in range(want.shape[0]):
        den = torch.linalg.vector_norm(want[r]).item()
        num = torch.linalg.vector_norm(got[r] - want[r]).item()
        worst = max(worst, num / den if den > 0 else num)
    return worst


def _config3_sources(count, seed, dt, device, rank=0, world=1):
    """Sources drawn like the batching configuration: lengths log-uniform in
    2^15..2^22 samples, f log-U 1e-4..1e-2 Hz, fdot log-U 1e-18..1e-13,
    A log-U 1e-23..1e-21, isotropic angles; waveforms generated on the device
    for this rank's shard only (sources balanced over ranks by samples)."""
    import torch

    from fastlisaresponse_gb300 import waveforms as wf
    from fastlisaresponse_gb300.dist import shard_by_samples

    rng = np.random.default_rng(seed)
    lengths = np.exp(rng.uniform(np.log(2**15), np.log(2**22), count)).astype(np.int64)
    p = wf.draw_gb_parameters(rng, count)
    mine = shard_by_samples(lengths, rank, world)
    hs = []
    for i in mine:
        t = torch.arange(int(lengths[i]), dtype=torch.float64, device=device) * dt
        hs.append(wf.gb_waveform(p["A"][i], p["f"][i], p["fdot"][i], p["iota"][i],
                                 p["phi0"][i], p["psi"][i], t))
    return lengths, mine, hs, p["lam"][mine], p["beta"][mine]


def run_batch_section(args, device, peaks, rank=0, world=1):
    """The batching configuration: all sources (2048 by default) in one
    persistent launch of the mixed kernel, replayed from the CUDA graph of its
    size bucket, against the FP64 fused kernel on the first 256 sources (whose
    rate does not depend on the batch size; timing all 2048 in FP64 would take
    about a minute).  Under torchrun the sources are sharded over the ranks
    (no collective on the data path; the job time is the slowest rank's)."""
    import torch

    import fastlisaresponse_gb300 as flr
    from fastlisaresponse_gb300.dist import max_over_ranks

    dt = 10.0
    lengths, mine, hs, lam, beta = _config3_sources(args.batch_sources, seed=3, dt=dt,
                                                    device=device, rank=rank, world=world)
    orb = flr.EqualArmlengthOrbits(t_max=(math.floor(lengths.max() * dt / 1e4) + 3) * 1e4)
    ts = int(T_BUFFER / dt)
    n_out = int(sum(int(n) - 2 * ts for n in lengths))
    sub = list(range(min(256, len(mine))))
    n_sub = int(sum(int(lengths[mine[i]]) - 2 * ts for i in sub))
    res = {"sources": int(args.batch_sources), "samples": int(lengths.sum()),
           "output_samples": n_out, "sources_per_rank": len(mine),
           "workload": "batching configuration: lengths log-uniform 2^15..2^22 at dt = 10 s, "
                       "f log-U 1e-4..1e-2 Hz, fdot log-U 1e-18..1e-13, A log-U 1e-23..1e-21, "
                       "equal-arm orbits, 2nd-gen TDI XYZ, order 25",
           "hbm_bytes_inputs_outputs": int(lengths.sum()) * 40}
    tune = [int(lengths[i]) for i in mine[:32]]
    # mixed: every source of this rank in one launch, through its graph bucket
    bat = flr.BatchedResponseTDI(1 / dt, order=25, tdi="2nd generation", orbits=orb,
                                 precision="mixed", tile="auto", tune_lengths=tune)
    out_m = [torch.empty((3, int(lengths[i])), dtype=torch.float64, device=device) for i in mine]
    steps = max(1, min(args.steps, 3))
    secs = max_over_ranks([_timed(lambda: bat(hs, lam, beta, out=out_m, use_graph=True),
                                  steps, 1, device)], device=device)[0]
    assert bat.status() == 0, flr.describe_status(bat.status())
    res["mixed"] = {"value": n_out * steps / secs, "ms_per_step": 1e3 * secs / steps,
                    "steps": steps, "plan": bat.plan_info, "tune": bat.tune,
                    "path": "BatchedResponseTDI(precision='mixed', use_graph=True): one graph "
                            "replay (staging copy + fused kernel) per step"}
    del bat
    # fp64 on the first sources
    bat = flr.BatchedResponseTDI(1 / dt, order=25, tdi="2nd generation", orbits=orb,
                                 precision="fp64", tile="auto", tune_lengths=tune)
    holder = {}

    def step():
        holder["o"] = bat([hs[i] for i in sub], lam[sub], beta[sub])

    secs = max_over_ranks([_timed(step, 1, 1, device)], device=device)[0]
    assert bat.status() == 0, flr.describe_status(bat.status())
    res["fp64"] = {"value": n_sub / secs, "ms_per_step": 1e3 * secs, "steps": 1,
                   "sources": len(sub), "plan": bat.plan_info, "tune": bat.tune}
    del bat
    res["speedup_mixed_over_fp64"] = res["mixed"]["value"] / res["fp64"]["value"]
    res["max_rel_l2_mixed_vs_fp64"] = max_over_ranks(
        [max(_rel_l2_rows(out_m[i], holder["o"][k]) for k, i in enumerate(sub))],
        device=device)[0]
    res["accuracy_sources"] = len(sub)
    del holder
    # the sampler's form: <h|d> and <h|h> per source formed in the kernel, the
    # channels never stored (data = the mixed outputs themselves)
    bat = flr.BatchedResponseTDI(1 / dt, order=25, tdi="2nd generation", orbits=orb,
                                 precision="mixed", tile="auto", tune_lengths=tune)
    box = {}

    def inner_step():
        box["i"] = bat.inner_products(hs, lam, beta, out_m)

    secs = max_over_ranks([_timed(inner_step, steps, 1, device)], device=device)[0]
    assert bat.status() == 0, flr.describe_status(bat.status())
    hh = box["i"][:, 1, :]
    hh_ref = torch.stack([(o[:, ts:o.shape[1] - ts] ** 2).sum(dim=1) for o in out_m])
    res["inner_products"] = {
        "value": n_out * steps / secs, "ms_per_step": 1e3 * secs / steps, "steps": steps,
        "path": "BatchedResponseTDI.inner_products: per-source <h|d>, <h|h> per channel from "
                "the fused kernel, no channel stored (24 B/sample of HBM writes saved)",
        "max_rel_diff_hh_vs_stored": float(((hh - hh_ref).abs() / hh_ref.abs()).max().item())}
    del bat, out_m, hs, box
    torch.cuda.empty_cache()
    return res


def _err_stats(got, want):
    """Per-row relative L2 and max error (max |got - want| / max |want|)."""
    import torch

    d = got - want
    num = torch.linalg.vector_norm(d, dim=1)
    den = torch.linalg.vector_norm(want, dim=1)
    mx = d.abs().amax(dim=1) / want.abs().amax(dim=1).clamp_min(1e-300)
    return (num / den.clamp_min(1e-300)).cpu().numpy(), mx.cpu().numpy()


def run_precision_section(args, device):
    """Precision configuration: sources of 2^20 samples at dt = 10 s drawn as
    in the batching configuration, Lagrange orders 25 and 45.  The mixed path
    is compared with the FP64 fused path (bit-identical to the oracle and the
    plain path) per link and per X/Y/Z channel, and its integer delay indices
    (receiver, emitter, every TDI unit) with the FP64 path's, bit for bit."""
    import torch

    import fastlisaresponse_gb300 as flr

    dt, n = 10.0, 2**20
    count = args.precision_sources
    rng = np.random.default_rng(4)
    p = flr.waveforms.draw_gb_parameters(rng, count)
    orb = flr.EqualArmlengthOrbits(t_max=(math.floor(n * dt / 1e4) + 3) * 1e4)
    t = torch.arange(n, dtype=torch.float64, device=device) * dt
    chunk = 16
    res = {"workload": f"{count} galactic binaries x 2^20 samples at dt = 10 s drawn as in the "
                       "batching configuration, equal-arm orbits, 2nd-gen TDI XYZ",
           "sources": count, "reference": "FP64 fused path (bit-identical to the oracle)"}
    for order in (25, 45):
        tb = 1e4 if order <= 25 else 2e4  # order 45 needs the longer garbage margin
        plans = {prec: flr.BatchedResponseTDI(1 / dt, order=order, tdi="2nd generation",
                                              orbits=orb, precision=prec, t_buffer=tb,
                                              force_backend=device)
                 for prec in ("fp64", "mixed")}
        ts = plans["fp64"].tdi_start_ind
        sl = slice(ts, n - ts)
        link_l2, link_max, chan_l2, chan_max = [], [], [], []
        mism = {"d_rec": 0, "d_em": 0, "d_tdi": 0}
        secs = {"fp64": 0.0, "mixed": 0.0}
        for c0 in range(0, count, chunk):
            idx = range(c0, min(count, c0 + chunk))
            hs = [flr.gb_waveform(p["A"][i], p["f"][i], p["fdot"][i], p["iota"][i],
                                  p["phi0"][i], p["psi"][i], t) for i in idx]
            lam, beta = p["lam"][list(idx)], p["beta"][list(idx)]
            runs = {}
            for prec, bat in plans.items():
                bat(hs[:1], lam[:1], beta[:1])  # warm-up
                holder = {}

                def step():
                    holder["o"] = bat(hs, lam, beta)

                secs[prec] += _timed(step, 1, 0, device)
                runs[prec] = (holder["o"], bat(hs, lam, beta, diagnostics=True)[1])
                assert bat.status() == 0, flr.describe_status(bat.status())
            for j in range(len(hs)):
                (o64, d64), (omx, dmx) = [(runs[k][0][j], runs[k][1][j])
                                          for k in ("fp64", "mixed")]
                for key in mism:
                    mism[key] += int((dmx[key][:, sl] != d64[key][:, sl]).sum().item())
                a, b = _err_stats(dmx["y"][:, sl], d64["y"][:, sl])
                link_l2.append(a)
                link_max.append(b)
                a, b = _err_stats(omx[:, sl], o64[:, sl])
                chan_l2.append(a)
                chan_max.append(b)
            del runs, hs
        link_l2, link_max = np.asarray(link_l2), np.asarray(link_max)
        chan_l2, chan_max = np.asarray(chan_l2), np.asarray(chan_max)
        n_out = count * (n - 2 * ts)
        res[f"order_{order}"] = {
            "t_buffer_s": tb,
            "per_link": {str(k): {"rel_l2_max": float(link_l2[:, k].max()),
                                  "rel_l2_median": float(np.median(link_l2[:, k])),
                                  "max_err_max": float(link_max[:, k].max())}
                         for k in range(6)},
            "per_channel": {ch: {"rel_l2_max": float(chan_l2[:, k].max()),
                                 "rel_l2_median": float(np.median(chan_l2[:, k])),
                                 "max_err_max": float(chan_max[:, k].max())}
                            for k, ch in enumerate("XYZ")},
            "index_mismatches": mism,
            "samples_per_s": {prec: n_out / s for prec, s in secs.items()},
            "speedup_mixed_over_fp64": secs["fp64"] / secs["mixed"],
        }
        del plans
        torch.cuda.empty_cache()
    res["max_err_definition"] = "max |mixed - fp64| / max |fp64| per row"
    return res


def run_serving_section(args, device):
    """Open-loop Poisson request streams against ResponseServer: saturation
    throughput, then p50/p99 latency at rates below it."""
    import threading

    import torch

    import fastlisaresponse_gb300 as flr

    dt = 10.0
    count = args.serve_requests
    rng = np.random.default_rng(5)
    lengths = np.exp(rng.uniform(np.log(2**14), np.log(2**22), count)).astype(np.int64)
    p = flr.waveforms.draw_gb_parameters(rng, count)
    params = [(p["A"][i], p["f"][i], p["fdot"][i], p["iota"][i], p["phi0"][i], p["psi"][i],
               p["lam"][i], p["beta"][i]) for i in range(count)]
    sets = rng.integers(0, 2, count)
    orb = flr.EqualArmlengthOrbits(t_max=(math.floor(lengths.max() * dt / 1e4) + 3) * 1e4)
    out = {"workload": "open-loop Poisson requests: lengths log-uniform 2^14..2^22 at dt = 10 s, "
                       "1st/2nd-gen TDI 50/50, galactic-binary parameters drawn as in the "
                       "batching configuration, waveforms generated on the device, mixed "
                       "precision, 160 GB admission budget, 2 streams",
           "requests_per_rate": count, "mean_samples": float(lengths.mean())}

    # batched throughput of the same requests (the first 2000 at most: ~60 GB)
    # in one launch pair (reference point)
    bat = flr.BatchedResponseTDI(1 / dt, tdi=["1st generation", "2nd generation"], orbits=orb,
                                 precision="mixed", force_backend=device)
    nb = min(count, 2000)
    prm = np.asarray([q[:6] for q in params[:nb]])
    lam = [q[6] for q in params[:nb]]
    beta = [q[7] for q in params[:nb]]
    bat.run_gb(prm[:4], lengths[:4], lam[:4], beta[:4], tdi_set=sets[:4])  # warm-up
    torch.cuda.synchronize(device)
    e0, e1 = _events()
    e0.record()
    outs, hs = bat.run_gb(prm, lengths[:nb], lam, beta, tdi_set=sets[:nb])
    e1.record()
    torch.cuda.synchronize(device)
    del outs, hs
    secs = e0.elapsed_time(e1) * 1e-3
    n_out = int(sum(int(n) - 2000 for n in lengths[:nb]))
    out["batched_throughput_samples_per_s"] = n_out / secs
    out["batched_reference_requests"] = nb
    del bat
    torch.cuda.empty_cache()

    def run(rate):
        with flr.ResponseServer(1 / dt, orbits=orb, num_streams=2, force_backend=device,
                                keep_results=False,
                                max_batch_samples=SERVE_BATCH_SAMPLES) as srv:
            srv.submit(params[0], int(lengths[0]), int(sets[0])).result(timeout=60)  # warm-up
            srv.completed.clear()
            arrivals = (np.cumsum(rng.exponential(1.0 / rate, count)) if rate
                        else np.zeros(count))

            def client():
                t_start = time.perf_counter()
                for i in range(count):
                    delay = t_start + arrivals[i] - time.perf_counter()
                    if delay > 0:
                        time.sleep(delay)
                    srv.submit(params[i], int(lengths[i]), int(sets[i]))

            th = threading.Thread(target=client)
            th.start()
            th.join()
            while len(srv.completed) < count:
                time.sleep(0.005)
            st = srv.stats()
        return st

    sat = run(None)
    out["saturation"] = sat
    cap = sat["throughput_requests_per_s"]
    out["rates"] = []
    for frac in (0.5, 0.8, 0.9):
        st = run(frac * cap)
        st["offered_requests_per_s"] = frac * cap
        st["fraction_of_batched_throughput"] = (st["throughput_samples_per_s"] /
                                                out["batched_throughput_samples_per_s"])
        out["rates"].append(st)
    return out


def run_ours(args, rank, world, device):
    import torch

    import fastlisaresponse_gb300 as flr
    from fastlisaresponse_gb300 import _lib, perfmodel

    w = WORKLOADS[args.workload]
    n, dt = w["n"], w["dt"]
    orb, h, lam, beta = make_source(w, n, seed=1 + rank)
    n_out = output_samples(n, dt)
    h_dev = torch.as_tensor(h, device=device)
    lib = _lib.lib()
    peaks = measure_fp64_peak(device)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # --- headline: mixed-precision fused path (BatchedResponseTDI, one source,
    # HEADLINE_CHUNKS tile-aligned launches over two streams; same bits as one)
    bat = flr.BatchedResponseTDI(1.0 / dt, order=w["order"], tdi=w["tdi"], orbits=orb,
                                 precision="mixed", force_backend=device, tile="auto",
                                 tune_lengths=[n])
    out_dev = torch.empty((3, n), dtype=torch.float64, device=device)
    held = {}

    def mixed_step():
        held["mixed"] = bat([h_dev], lam, beta, out=[out_dev], chunks=HEADLINE_CHUNKS)[0]

    for _ in range(args.warmup):
        mixed_step()
    torch.cuda.synchronize(device)
    clocks = ClockSampler(gpu_uuid(device))
    clocks.start()
    time.sleep(0.4)
    barrier()
    elapsed = _timed(mixed_step, args.steps, 0, device)
    barrier()
    clock_info = clocks.stop()
    assert bat.status() == 0, flr.describe_status(bat.status())

    # --- the fused kernel alone: single launches, CUDA events around each on
    # its stream (the roofline's per-launch duration)
    ev = {"on": False, "fused": []}
    run_fn = lib.flr_batch_run

    def timed_run(*a):
        if not ev["on"]:
            return run_fn(*a)
        e0, e1 = _events()
        e0.record()
        rc = run_fn(*a)
        e1.record()
        ev["fused"].append((e0, e1))
        return rc

    lib.flr_batch_run = timed_run
    one = {}

    def single_step():
        one["o"] = bat([h_dev], lam, beta)[0]

    single_elapsed = _timed(single_step, max(1, min(args.steps, 5)), 1, device, kernel_events=ev)
    lib.flr_batch_run = run_fn
    assert torch.equal(one["o"], held["mixed"])  # chunked launches: the same bits

    # --- the plain FP64 drop-in path on the same source
    resp = flr.pyResponseTDI(1.0 / dt, n, order=w["order"], tdi=w["tdi"], orbits=orb,
                             force_backend=device)
    pev = {"on": False, "response": [], "tdi": []}

    def wrap(name, fn):
        def inner(*a, **k):
            if not pev["on"]:
                return fn(*a, **k)
            e0, e1 = _events()
            e0.record()
            fn(*a, **k)
            e1.record()
            pev[name].append((e0, e1))
        return inner

    resp.cpp_response.get_response_wrap = wrap("response", resp.cpp_response.get_response_wrap)
    resp.cpp_response.get_tdi_delays_wrap = wrap("tdi", resp.cpp_response.get_tdi_delays_wrap)

    def plain_step():
        resp.get_projections(h_dev, lam, beta, t0=0.0, t_buffer=T_BUFFER)
        resp.get_tdi_delays()

    plain_steps = max(1, min(args.steps, 5))
    plain_elapsed = _timed(plain_step, plain_steps, 1, device, kernel_events=pev)
    assert resp.status() == 0
    max_rel = _rel_l2_rows(held["mixed"], resp.XYZ)

    # --- end to end through BatchedResponseTDI.run_host: pinned host in, pinned
    # host out, copies overlapped with the computation (4 chunks)
    h_pin = torch.from_numpy(h).pin_memory()
    out_pin = torch.empty((3, n), dtype=torch.float64).pin_memory()

    def e2e_step():
        bat.run_host([h_pin], lam, beta, out=[out_pin], chunks=E2E_CHUNKS)

    barrier()
    e2e_elapsed = _timed(e2e_step, args.steps, args.warmup, device)
    barrier()

    from fastlisaresponse_gb300.dist import max_over_ranks

    elapsed, e2e_elapsed = max_over_ranks([elapsed, e2e_elapsed], device=device)

    # --- rooflines
    tables = resp.tdi_tables_host
    lists = []
    for u in range(tables["num_units"]):
        st, ln = tables["unit_starts"][u], tables["unit_lengths"][u]
        lists.append([x for x in tables["tdi_link_combinations"][st:st + ln] if x != -11])
    n_delay_links = sum(len(x) for x in lists)
    measured = {}
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        with open(peaks_path) as fh:
            measured = json.load(fh)
    hbm_peak = measured.get("hbm_gbs")
    peak = peaks["fp64_fma"]
    div_cost = peaks["fp64_fma"] / peaks["fp64_div"]

    fused_ms = 1e3 * statistics.mean(a.elapsed_time(b) * 1e-3 for a, b in ev["fused"])
    idx_ops = perfmodel.mixed_index_ops(tables["num_units"],
                                        perfmodel.prefix_shared_subtractions(lists))
    fused_secs = fused_ms * 1e-3
    fused_bytes = 40 * n_out  # complex input in, three channels out
    roofline = {
        "bound": "fp64",
        "kernel": "fused_kernel<mixed> (flr_fused.cu)",
        "achieved": idx_ops["total"] * n_out / fused_secs / 1e9,
        "peak": peak / 1e9,
        "unit": "G FP64-ops/s",
        "frac": idx_ops["total"] * n_out / fused_secs / peak,
        "definition": "FP64 operations the bit-exact delay/index path needs per output "
                      f"sample (perfmodel.mixed_index_ops: {idx_ops['total']}), over the "
                      "launch's CUDA-event time; the double-float taps run on the FP32 pipe "
                      "and are not counted",
        "peak_source": "measured in this run: FP64 FMA probe kernel (flr_probe_pipe_rate), "
                       "best of 3; MEASURED_PEAKS.json has no FP64 figure",
        "launch_ms": fused_ms,
        "algorithmic_bytes": fused_bytes,
        "traffic": load_traffic("fused_kernel_mixed", args.workload),
        "hbm": {"achieved_gbs": fused_bytes / fused_secs / 1e9, "peak_gbs": hbm_peak,
                "frac": (fused_bytes / fused_secs / 1e9 / hbm_peak) if hbm_peak else None,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if hbm_peak else None},
        "pipe_peaks_g_per_s": {k: v / 1e9 for k, v in peaks.items() if k != "sms"},
    }
    kern = {k: 1e3 * statistics.mean(a.elapsed_time(b) * 1e-3 for a, b in pev[k])
            for k in ("response", "tdi")}
    counts = perfmodel.counts_per_sample(w["order"], tables["num_units"], n_delay_links)
    computed = {"response": n - 2 * resp.projections_start_ind,
                "tdi": n - 2 * resp.tdi_start_ind}
    dominant = max(kern, key=kern.get)
    c = counts[dominant]
    slots = perfmodel.fp64_slots(c, div_cost) * computed[dominant]
    psecs = kern[dominant] * 1e-3
    plain = {
        "value": n_out * plain_steps / plain_elapsed,
        "ms_per_step": 1e3 * plain_elapsed / plain_steps,
        "steps": plain_steps,
        "path": "pyResponseTDI.get_projections + get_tdi_delays (two plain FP64 kernels, "
                "bit-identical to the reference's CPU arithmetic)",
        "kernels_ms": kern,
        "roofline": {
            "bound": "fp64", "kernel": f"{dominant}_plain_kernel",
            "achieved": slots / psecs / 1e9, "peak": peak / 1e9, "unit": "G FP64-slots/s",
            "frac": slots / psecs / peak,
            "frac_division_as_one_op": (c["ops"] + c["divs"]) * computed[dominant] / psecs / peak,
            "definition": "reference-arithmetic FP64 work (perfmodel.counts_per_sample: "
                          f"{c['ops']} ops + {c['divs']} divisions per sample for {dominant}), "
                          f"divisions weighted by their measured cost ({div_cost:.2f} FMA "
                          "slots)",
            "traffic": load_traffic(f"{dominant}_plain_kernel", args.workload),
        },
    }
    result = {
        "metric": METRIC,
        "value": n_out * args.steps * world / elapsed,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * elapsed / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64 delays/indices + double-float (2xf32) taps; outputs f64",
        "data": "synthetic (seeded galactic-binary waveform, analytic orbits)",
        "config": {"workload": w["desc"], "name": args.workload, "samples_per_step": n_out,
                   "input_samples": n,
                   "path": "mixed-precision fused kernel (BatchedResponseTDI, one source, "
                           f"{HEADLINE_CHUNKS} tile-aligned launches over two streams per step, "
                           "the same bits as one launch); integer delay indices bit-exact",
                   "single_launch_samples_per_s": n_out * max(1, min(args.steps, 5))
                   / single_elapsed,
                   "tile": bat.plan_info["tile"], "tile_tuning": bat.tune,
                   "l2": "flushed before every timed step (256 MB write); h 16 B + XYZ "
                         f"24 B per sample = {40 * n / 1e6:.0f} MB per step"},
        "accuracy": {"max_rel_l2_vs_plain_fp64": max_rel, "bound": 1e-6,
                     "per": "TDI channel, this run's outputs"},
        "plain_fp64": plain,
        "speedup_vs_plain_fp64": (n_out * args.steps / elapsed) / plain["value"],
        "e2e": {"value": n_out * args.steps * world / e2e_elapsed, "unit": UNIT,
                "h2d_bytes_per_step": 16 * n, "d2h_bytes_per_step": 24 * n,
                "api": "BatchedResponseTDI.run_host: the input in pinned host memory, X/Y/Z "
                       "returned to pinned host memory, copies overlapped with the chunks' "
                       f"launches ({E2E_CHUNKS} chunks, 2 compute streams)"},
        "gpu_launches": args.steps * HEADLINE_CHUNKS,
        "roofline": roofline,
        "clocks": clock_info,
    }
    if args.batch_sources > 0:
        result["batched"] = run_batch_section(args, device, peaks, rank, world)
    if args.precision_sources > 0 and world == 1:
        result["precision"] = run_precision_section(args, device)
    if args.serve_requests > 0 and world == 1:
        result["serving"] = run_serving_section(args, device)
    return result


def cpu_baseline_line(args, cores: int, variant: str = "o3"):
    steps = max(1, min(args.steps, 3))
    r = cpu_rate(args.workload, cores, steps=steps, warmup=1, variant=variant)
    w = WORKLOADS[args.workload]
    return {"value": r["value"], "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{cores} independent source(s) of {CPU_SLICE} samples "
                      f"({output_samples(CPU_SLICE, w['dt'])} output samples each) in the "
                      f"workload's configuration, {steps} timed passes; C oracle "
                      f"(oracle/flr_oracle.c, gcc -O3), one process per core",
            "seconds": r["seconds"]}


def run_reference(args):
    cores = os.cpu_count() or 1
    w = WORKLOADS[args.workload]
    r = cpu_rate(args.workload, cores, steps=args.steps, warmup=args.warmup, variant="o3")
    line = {
        "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded galactic-binary waveform, analytic orbits)",
        "config": {"workload": w["desc"], "name": args.workload,
                   "samples_per_step": r["samples_per_step"],
                   "cpu_slice": f"{CPU_SLICE} samples per source, one source per core"},
        "impl": "reference",
        "cpu_baseline": {"value": r["value"], "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{cores} sources x {CPU_SLICE} samples per step"},
        "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "the reference's CPU path, restated in C (oracle/flr_oracle.c) and pinned "
                "bit for bit to the reference's own compiled CPU code; the port is timed "
                "because the reference's code cannot be built without its sources and "
                "lisaanalysistools, which the GPU host does not have",
    }
    return line


def run_profile_batch(spec: str) -> None:
    """Small batched case for ncu captures: 16 galactic binaries x 2^18
    samples at dt = 10 s, 2nd-gen TDI, order 25; spec = "<fp64|mixed>:<equal|kepler>".
    Two calls of the batch (the capture takes the first)."""
    import torch

    import fastlisaresponse_gb300 as flr

    prec, kind = spec.split(":")
    dev = torch.device("cuda", 0)
    dt, ns, n = 10.0, 16, 2**18
    rng = np.random.default_rng(5)
    t_max = (n * dt // 1e4 + 3) * 1e4
    orb = flr.EqualArmlengthOrbits(t_max=t_max) if kind == "equal" else \
        flr.KeplerianOrbits(t_max=t_max)
    p = flr.waveforms.draw_gb_parameters(rng, ns)
    t = torch.arange(n, dtype=torch.float64, device=dev) * dt
    hs = [flr.gb_waveform(p["A"][i], p["f"][i], p["fdot"][i], p["iota"][i], p["phi0"][i],
                          p["psi"][i], t) for i in range(ns)]
    bat = flr.BatchedResponseTDI(1 / dt, order=25, tdi="2nd generation", orbits=orb,
                                 precision=prec)
    for _ in range(2):
        bat(hs, p["lam"], p["beta"])
    torch.cuda.synchronize()
    assert bat.status() == 0
    print(json.dumps({"profile_batch": spec, "plan": bat.plan_info}))


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default=DEFAULT_WORKLOAD)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch-sources", type=int, default=2048,
                    help="sources in the batching section (0 = skip)")
    ap.add_argument("--serve-requests", type=int, default=1000,
                    help="requests per arrival rate in the serving section (0 = skip)")
    ap.add_argument("--precision-sources", type=int, default=32,
                    help="sources of 2^20 samples in the precision section (0 = skip)")
    ap.add_argument("--profile-batch", default=None, metavar="PREC:ORBIT",
                    help="run only the small batched profiling case (fp64|mixed:equal|kepler)")
    args = ap.parse_args()
    if args.profile_batch:
        import fastlisaresponse_gb300 as flr

        flr.build()
        run_profile_batch(args.profile_batch)
        return
    args.warmup = max(args.warmup, 0)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)), flush=True)
        return

    # CPU processes are spawned before the first CUDA call
    cpu_line = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu_line = cpu_baseline_line(args, cores=1)

    import torch

    import fastlisaresponse_gb300 as flr

    flr.build()
    device = torch.device("cuda", local)
    torch.cuda.set_device(device)
    if world > 1:
        torch.distributed.init_process_group("nccl", device_id=device)
    result = run_ours(args, rank, world, device)
    if cpu_line is not None:
        result["cpu_baseline"] = cpu_line
    if rank == 0:
        print(json.dumps(result), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
