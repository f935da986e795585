#!/usr/bin/env python3
"""Benchmark of the LISA time-domain response + TDI on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--batch-sources S] [--no-cpu-baseline] [--precision-sources P]
                    [--serve-requests R] [--details FILE]

Headline workload (one step = one pass of the hot path over it): the batching
configuration -- 2048 galactic binaries with lengths log-uniform in
2^15..2^22 samples at dt = 10 s (1.76e9 samples), f log-uniform 1e-4..1e-2 Hz,
fdot 1e-18..1e-13, A 1e-23..1e-21, isotropic angles (seed 3), equal-arm
orbits, 2nd-generation TDI XYZ, Lagrange order 25.  Our arm evaluates it in
mixed precision (FP64 delays and bit-exact integer indices, double-float
taps), all sources in one persistent launch replayed from a CUDA graph per
step.  Printed on rank 0, one JSON line:
  value         output samples/s with the inputs resident in HBM (28 GB, larger
                than L2; L2 also flushed before each step), CUDA events around
                each step, max over ranks;
  e2e           the same through BatchedResponseTDI.run_host: waveforms in
                page-locked host memory, channels returned to page-locked host
                memory, copies inside the timed region;
  roofline      the fused kernel's FP64 index-path operations per second against
                the FP64 FMA rate measured at start-up, its HBM bytes against
                MEASURED_PEAKS.json;
  cpu_baseline  the C restatement of the reference's CPU path on one host core,
                on slices of the same source list;
  plain_fp64    the plain FP64 drop-in path (pyResponseTDI, bit-identical to the
                reference's CPU arithmetic) on a length-matched subset of the
                same sources, and speedup_vs_plain_fp64 = value / its rate;
  fp64_fused    the fused kernel in its FP64 flavour on that subset;
  accuracy      mixed vs plain FP64 on that subset (relative L2 per channel);
  single_source the 1 yr / dt = 5 s source with flexing Keplerian orbits
                (mixed, single launch, plain FP64, the drop-in ResponseWrapper
                end to end with NumPy in and out);
  precision / serving  compact summaries of those configurations (--details
                writes the serving section's full statistics to FILE).
With --impl reference the reference's CPU path (the C restatement) is timed
on all host cores over slices of the same source list, printed with "impl":
"reference" and the same "config".  Under torchrun every rank takes a share of
the sources balanced by samples (weak scaling); the reference arm runs on rank
0 only.
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

BATCH = dict(sources=2048, seed=3, dt=10.0, log2_min=15, log2_max=22, order=25,
             tdi="2nd generation")
SINGLE = dict(desc="one galactic binary (A 1e-22, f 2e-3 Hz, fdot 1e-14), 1 yr at dt = 5 s "
                   "(6,311,629 samples), flexing Keplerian orbits (arms +-1 %), 2nd-generation "
                   "TDI XYZ, Lagrange order 25",
              dt=5.0, n=int(YRSID_SI / 5.0), order=25, tdi="2nd generation",
              A=1e-22, f=2e-3, fdot=1e-14)
CPU_SLICE = 2**17         # output samples per CPU task (a slice of one source)
SUBSET_STRIDE = 16        # plain FP64 leg: every 16th source by length (128 of 2048)
E2E_GROUP_SAMPLES = 2**24  # samples per launch of the host pipeline
SINGLE_CHUNKS = 8          # launches per 1 yr step (two streams: last waves overlap)
SERVE_BATCH_SAMPLES = 2**23


def batch_config(sources: int) -> dict:
    """The `config` of both arms' JSON lines (identical, so the two measure
    the same workload)."""
    return {"workload": f"batching configuration: {sources} galactic binaries, lengths "
                        "log-uniform 2^15..2^22 samples at dt = 10 s, f log-U 1e-4..1e-2 Hz, "
                        "fdot log-U 1e-18..1e-13, A log-U 1e-23..1e-21, isotropic angles "
                        f"(seed {BATCH['seed']}), equal-arm orbits, 2nd-generation TDI XYZ, "
                        "Lagrange order 25",
            "sources": sources, "order": BATCH["order"], "tdi": BATCH["tdi"],
            "dt": BATCH["dt"], "t_buffer_s": T_BUFFER,
            "l2": "inputs (16 B/sample, 28 GB) far larger than the 129 MB L2; L2 also "
                  "flushed before each timed step"}


def batch_sources(count: int, seed: int = BATCH["seed"]):
    """Lengths and galactic-binary parameters of the batching configuration."""
    from fastlisaresponse_gb300 import waveforms as wf

    rng = np.random.default_rng(seed)
    lengths = np.exp(rng.uniform(np.log(2**BATCH["log2_min"]), np.log(2**BATCH["log2_max"]),
                                 count)).astype(np.int64)
    return lengths, wf.draw_gb_parameters(rng, count)


def output_samples(n, dt=BATCH["dt"]) -> int:
    return int(n) - 2 * int(T_BUFFER / dt)


def orbit_t_max(n_max: int, dt: float) -> float:
    return (math.floor(n_max * dt / 1e4) + 3) * 1e4


# ----------------------------------------------------------------------------- CPU side

_worker = {}


def _cpu_init(count, variant):
    import oracle
    from fastlisaresponse_gb300 import orbits as om

    lengths, p = batch_sources(count)
    dt = BATCH["dt"]
    orb = om.EqualArmlengthOrbits(t_max=orbit_t_max(int(lengths.max()), dt))
    ts = int(T_BUFFER / dt)
    o = oracle.OracleResponseTDI(1.0 / dt, CPU_SLICE + 2 * ts, orb.pycppdetector_args,
                                 orb.x_base, order=BATCH["order"], tdi=BATCH["tdi"],
                                 variant=variant)
    _worker.update(o=o, lengths=lengths, p=p)


def _cpu_task(task):
    """Output samples [a, a + CPU_SLICE) of source i (the whole source if it is
    shorter), computed as the reference's CPU path does: the slice's input
    with its edge zones, get_projections then get_tdi_delays."""
    from fastlisaresponse_gb300 import waveforms as wf

    i, a = task
    s = _worker
    p, dt = s["p"], BATCH["dt"]
    ts = int(T_BUFFER / dt)
    n = int(s["lengths"][i])
    n_slice = min(n, CPU_SLICE + 2 * ts)
    start = min(a, n - n_slice)
    t = (start + np.arange(n_slice)) * dt
    h = wf.gb_waveform(p["A"][i], p["f"][i], p["fdot"][i], p["iota"][i], p["phi0"][i],
                       p["psi"][i], t)
    t0 = time.perf_counter()
    s["o"].get_projections(h, p["lam"][i], p["beta"][i], t0=float(t[0]), t_buffer=T_BUFFER)
    s["o"].get_tdi_delays()
    return n_slice - 2 * ts, time.perf_counter() - t0


def _cpu_schedule(count: int, tasks: int, offset: int):
    """`tasks` slices spread over the source list: source (offset + k) * 797
    mod count (797 is prime to the count: every source in turn), at a start
    that walks through the source."""
    lengths, _ = batch_sources(count)
    out = []
    for k in range(offset, offset + tasks):
        i = (k * 797) % count
        n = int(lengths[i])
        out.append((i, ((k * 104729) % max(1, n - CPU_SLICE)) if n > CPU_SLICE else 0))
    return out


def cpu_rate(count: int, cores: int, steps: int, warmup: int, tasks_per_core: int,
             variant: str = "o3"):
    """Output samples/s of the CPU path over slices of the batch's sources,
    `cores` processes, `cores * tasks_per_core` slices per step."""
    ctx = mp.get_context("spawn")
    walls, samples = [], 0
    per_step = cores * tasks_per_core
    with ctx.Pool(cores, initializer=_cpu_init, initargs=(count, variant)) as pool:
        for st in range(warmup + steps):
            tasks = _cpu_schedule(count, per_step, st * per_step)
            t0 = time.perf_counter()
            res = pool.map(_cpu_task, tasks, chunksize=1)
            wall = time.perf_counter() - t0
            if st >= warmup:
                walls.append(wall)
                samples += sum(r[0] for r in res)
    total = sum(walls)
    return dict(value=samples / total, seconds=total, ms_per_step=1e3 * total / len(walls),
                samples_per_step=samples / len(walls), steps=len(walls))


# ----------------------------------------------------------------------------- GPU side

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
    return vis.split(",")[device.index] if vis else str(device.index)


def load_traffic(kernel: str):
    """DRAM bytes per computed output sample of a kernel from an ncu capture
    (profiles/ncu_traffic.json), or None."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    if not os.path.exists(path):
        return None
    with open(path) as fh:
        entry = json.load(fh).get(kernel)
    return entry if isinstance(entry, dict) and "bytes_per_output_sample" in entry else None


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
    device work; the step times are summed."""
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


def _device_waveforms(lengths, p, idx, dt, device):
    import torch

    from fastlisaresponse_gb300 import waveforms as wf

    hs = []
    for i in idx:
        t = torch.arange(int(lengths[i]), dtype=torch.float64, device=device) * dt
        hs.append(wf.gb_waveform(p["A"][i], p["f"][i], p["fdot"][i], p["iota"][i],
                                 p["phi0"][i], p["psi"][i], t))
    return hs


def _timed_wrapped(lib_obj, names, holder):
    """Wrap the named methods of lib_obj so that, while holder["on"], CUDA
    events bracket each call on the current stream (holder[name] collects
    them); returns a function that restores the originals."""
    saved = {n: getattr(lib_obj, n) for n in names}

    def make(name, fn):
        def inner(*a, **k):
            if not holder["on"]:
                return fn(*a, **k)
            e0, e1 = _events()
            e0.record()
            rc = fn(*a, **k)
            e1.record()
            holder[name].append((e0, e1))
            return rc
        return inner

    for n, fn in saved.items():
        holder.setdefault(n, [])
        setattr(lib_obj, n, make(n, fn))

    def restore():
        for n, fn in saved.items():
            setattr(lib_obj, n, fn)
    return restore


def _mean_ms(pairs):
    return statistics.mean(a.elapsed_time(b) for a, b in pairs)


def _unit_lists(tb):
    lists = []
    for u in range(tb["num_units"]):
        st, ln = tb["unit_starts"][u], tb["unit_lengths"][u]
        lists.append([x for x in tb["tdi_link_combinations"][st:st + ln] if x != -11])
    return lists


def run_headline(args, device, peaks, rank, world):
    """The batching configuration in mixed precision (value, e2e, roofline),
    with the plain FP64 drop-in path, the FP64 fused kernel and the mixed
    kernel on a length-matched subset beside it."""
    import torch

    import fastlisaresponse_gb300 as flr
    from fastlisaresponse_gb300 import _lib, perfmodel
    from fastlisaresponse_gb300.dist import max_over_ranks, shard_by_samples

    dt = BATCH["dt"]
    lengths, p = batch_sources(args.batch_sources)
    mine = list(shard_by_samples(lengths, rank, world))
    orb = flr.EqualArmlengthOrbits(t_max=orbit_t_max(int(lengths.max()), dt))
    hs = _device_waveforms(lengths, p, mine, dt, device)
    lam, beta = p["lam"][mine], p["beta"][mine]
    n_out = sum(output_samples(lengths[i]) for i in mine)
    res = {}

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # --- value: every source of this rank in one launch, through its graph bucket
    tune = [int(lengths[i]) for i in mine[:32]]
    bat = flr.BatchedResponseTDI(1 / dt, order=BATCH["order"], tdi=BATCH["tdi"], orbits=orb,
                                 precision="mixed", tile="auto", tune_lengths=tune,
                                 force_backend=device)
    outs = [torch.empty((3, int(lengths[i])), dtype=torch.float64, device=device) for i in mine]

    def step():
        bat(hs, lam, beta, out=outs, use_graph=True)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(device)
    clocks = ClockSampler(gpu_uuid(device))
    clocks.start()
    time.sleep(0.4)
    barrier()
    secs = _timed(step, args.steps, 0, device)
    barrier()
    res["clocks"] = clocks.stop()
    assert bat.status() == 0, flr.describe_status(bat.status())
    launch_secs = secs / args.steps  # one graph replay = staging copy + one fused launch
    job_secs = max_over_ranks([secs], device=device)[0]
    res["value"] = n_out * world * args.steps / job_secs
    res["ms_per_step"] = 1e3 * job_secs / args.steps
    res["plan"] = {k: bat.plan_info[k] for k in ("tile", "grid", "smem_bytes", "grouped")}

    # --- roofline of the fused kernel (one launch per step)
    tb = bat.tdi_sets[0]
    lists = _unit_lists(tb)
    idx_ops = perfmodel.mixed_index_ops_grouped(num_groups=len({len(x) for x in lists}),
                                                max_len=max(len(x) for x in lists))
    measured = {}
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        with open(peaks_path) as fh:
            measured = json.load(fh)
    hbm_peak = measured.get("hbm_gbs")
    fused_bytes = 40 * n_out  # complex input in, three channels out
    traffic = load_traffic("fused_kernel_mixed_grouped")
    res["roofline"] = {
        "bound": "fp64",
        "kernel": "fused_kernel<mixed, grouped> (flr_fused.cu), equal arms",
        "achieved": idx_ops["total"] * n_out / launch_secs / 1e9,
        "peak": peaks["fp64_fma"] / 1e9,
        "unit": "G FP64-ops/s",
        "frac": idx_ops["total"] * n_out / launch_secs / peaks["fp64_fma"],
        "definition": "FP64 operations of the bit-exact delay/index path per output sample "
                      f"(perfmodel.mixed_index_ops_grouped: {idx_ops['total']}) x output "
                      "samples / one launch's CUDA-event time; the double-float taps run on "
                      "the FP32 pipe, not counted; peak = FP64 FMA probe of this run "
                      "(MEASURED_PEAKS.json has no FP64 figure); the count is the reference "
                      "formula's, part of which the kernel does as integer work (index "
                      "splits and sample times from the bits, no t0 operations at t0 = 0), "
                      "so the fraction can reach 1 below FP64-pipe saturation",
        "launch_ms": 1e3 * launch_secs,
        "traffic": (traffic["bytes_per_output_sample"] * n_out) if traffic else None,
        "traffic_source": traffic["source"] if traffic else None,
        "hbm": {"algorithmic_bytes": fused_bytes,
                "achieved_gbs": fused_bytes / launch_secs / 1e9, "peak_gbs": hbm_peak,
                "frac": (fused_bytes / launch_secs / 1e9 / hbm_peak) if hbm_peak else None},
    }
    if traffic and traffic.get("warp_instructions_per_output_sample"):
        # issue slots: the kernel's warp instructions per sample (ncu, the
        # first 64 sources) x samples / launch time against 4 schedulers x SMs
        # x the SM clock sampled during the timed steps
        sms = torch.cuda.get_device_properties(device).multi_processor_count
        mhz = res["clocks"].get("sm_mhz") or res["clocks"].get("sm_max_mhz")
        wips = traffic["warp_instructions_per_output_sample"]
        if mhz:
            res["roofline"]["issue"] = {
                "warp_instructions_per_sample": wips,
                "achieved_g_per_s": wips * n_out / launch_secs / 1e9,
                "peak_g_per_s": 4 * sms * mhz * 1e6 / 1e9,
                "frac": wips * n_out / launch_secs / (4 * sms * mhz * 1e6),
                "ncu_fp64_pipe_active": traffic.get("fp64_pipe_active"),
                "ncu_issue_active": traffic.get("issue_active")}

    # --- e2e: host memory in and out through run_host (grouped launches)
    # (two page-locked regions, one view per source: the inputs and the channels)
    barrier()
    n_in = sum(int(lengths[i]) for i in mine)
    h_all = flr.HostArray(n_in, np.complex128)
    o_all = flr.HostArray(3 * n_in)
    h_host, o_host, off = [], [], 0
    for i, h in zip(mine, hs):
        n = int(lengths[i])
        h_host.append(h_all.tensor[off:off + n])
        o_host.append(o_all.tensor[3 * off:3 * (off + n)].view(3, n))
        h_host[-1].copy_(h)
        off += n
    bat_h = flr.BatchedResponseTDI(1 / dt, order=BATCH["order"], tdi=BATCH["tdi"], orbits=orb,
                                   precision="mixed", tile=bat.plan_info["tile"],
                                   force_backend=device)

    def e2e_step():
        bat_h.run_host(h_host, lam, beta, out=o_host, group_samples=E2E_GROUP_SAMPLES)

    e2e_secs = max_over_ranks([_timed(e2e_step, args.steps, args.warmup, device)],
                              device=device)[0]
    torch.cuda.synchronize(device)
    assert bat_h.status() == 0
    e2e_same = all(torch.equal(o, d.cpu()) for o, d in zip(o_host[:16], outs[:16]))
    del h_host, o_host, bat_h
    h_all.release()
    o_all.release()
    del h_all, o_all
    res["e2e"] = {"value": n_out * world * args.steps / e2e_secs, "unit": UNIT,
                  "h2d_bytes_per_step": 16 * n_in, "d2h_bytes_per_step": 24 * n_in,
                  "api": "BatchedResponseTDI.run_host: waveforms in page-locked host memory "
                         "(HostArray), channels back to page-locked host memory, "
                         f"~2^{int(math.log2(E2E_GROUP_SAMPLES))} samples per launch, copies "
                         "overlapped with the launches",
                  "same_bits_as_device_run": bool(e2e_same)}

    # --- the plain FP64 drop-in path, the FP64 fused kernel and the mixed kernel on a
    # length-matched subset: every SUBSET_STRIDE-th source in length order
    order = sorted(range(len(mine)), key=lambda k: int(lengths[mine[k]]))
    sub = order[SUBSET_STRIDE // 2::SUBSET_STRIDE]
    sub_out = sum(output_samples(lengths[mine[k]]) for k in sub)
    sub_len = [int(lengths[mine[k]]) for k in sub]
    resp = {}
    for k in sub:  # one drop-in instance per source length (the API's num_pts)
        resp[k] = flr.pyResponseTDI(1 / dt, int(lengths[mine[k]]), order=BATCH["order"],
                                    tdi=BATCH["tdi"], orbits=orb, force_backend=device)
    pev = {"on": False}
    lib = _lib.lib()
    restore = _timed_wrapped(lib, ["flr_get_response", "flr_get_tdi_delays"], pev)

    def plain_step():
        for k in sub:
            resp[k].get_projections(hs[k], float(lam[k]), float(beta[k]), t0=0.0,
                                    t_buffer=T_BUFFER)
            resp[k].get_tdi_delays()

    plain_steps = max(1, min(args.steps, 2))
    plain_secs = _timed(plain_step, plain_steps, 1, device, kernel_events=pev)
    restore()
    assert all(r.status() == 0 for r in resp.values())
    plain_rate = sub_out * plain_steps / plain_secs
    kern = {"response": _mean_ms(pev["flr_get_response"]),
            "tdi": _mean_ms(pev["flr_get_tdi_delays"])}
    # mixed on the subset (same sources), and its accuracy against the plain path
    sub_outs = [outs[k] for k in sub]
    acc = max(_rel_l2_rows(o, resp[k].XYZ) for o, k in zip(sub_outs, sub))
    mixed_sub_secs = _timed(lambda: bat([hs[k] for k in sub], lam[sub], beta[sub],
                                        out=sub_outs), 2, 1, device)
    # FP64 fused on the subset: bit-identical to the plain path
    bat64 = flr.BatchedResponseTDI(1 / dt, order=BATCH["order"], tdi=BATCH["tdi"], orbits=orb,
                                   precision="fp64", tile="auto", tune_lengths=sub_len[:32],
                                   force_backend=device)
    box = {}

    def fp64_step():
        box["o"] = bat64([hs[k] for k in sub], lam[sub], beta[sub])

    fp64_secs = _timed(fp64_step, 1, 1, device)
    assert bat64.status() == 0
    fp64_same = all(torch.equal(o, resp[k].XYZ) for o, k in zip(box["o"], sub))
    del box, bat64
    # plain path roofline: its dominant kernel, reference-arithmetic FP64 work
    counts = perfmodel.counts_per_sample(BATCH["order"], tb["num_units"],
                                         sum(len(x) for x in lists))
    div_cost = peaks["fp64_fma"] / peaks["fp64_div"]
    dom = max(kern, key=kern.get)
    c = counts[dom]
    r0 = resp[sub[-1]]
    start = {"response": r0.projections_start_ind, "tdi": r0.tdi_start_ind}[dom]
    computed = sum(int(lengths[mine[k]]) - 2 * start for k in sub) / len(sub)
    psecs = kern[dom] * 1e-3
    res["plain_fp64"] = {
        "value": plain_rate, "sources": len(sub), "output_samples": sub_out,
        "ms_per_step": 1e3 * plain_secs / plain_steps,
        "path": "pyResponseTDI.get_projections + get_tdi_delays per source (drop-in API, "
                f"device inputs), every {SUBSET_STRIDE}th source of the batch in length order",
        "roofline_frac": perfmodel.fp64_slots(c, div_cost) * computed / psecs
        / peaks["fp64_fma"],
        "roofline_frac_division_as_one_op": (c["ops"] + c["divs"]) * computed / psecs
        / peaks["fp64_fma"],
        "roofline_kernel": f"{dom}_plain_kernel (mean launch {kern[dom]:.2f} ms)"}
    res["fp64_fused"] = {"value": sub_out / fp64_secs, "sources": len(sub),
                         "bit_identical_to_plain": bool(fp64_same)}
    res["mixed_on_subset"] = sub_out * 2 / mixed_sub_secs
    res["accuracy"] = {"max_rel_l2_vs_plain_fp64": acc, "bound": 1e-6,
                       "per": "TDI channel, the subset's sources"}
    res["gpu_launches"] = args.steps  # one fused kernel per graph replay
    del outs, hs, resp
    torch.cuda.empty_cache()
    return res


def run_single_source(args, device, peaks):
    """The 1 yr source: mixed (chunked and one launch), plain FP64, and the
    drop-in ResponseWrapper end to end with NumPy in and out."""
    import torch

    import fastlisaresponse_gb300 as flr
    from fastlisaresponse_gb300 import batch as bm
    from fastlisaresponse_gb300 import perfmodel
    from fastlisaresponse_gb300 import waveforms as wf

    w = SINGLE
    n, dt = w["n"], w["dt"]
    orb = flr.KeplerianOrbits(t_max=orbit_t_max(n, dt))
    rng = np.random.default_rng(1)
    iota, phi0, psi = math.acos(rng.uniform(-1, 1)), rng.uniform(0, 2 * math.pi), \
        rng.uniform(0, math.pi)
    lam, beta = rng.uniform(0, 2 * math.pi), math.asin(rng.uniform(-1, 1))
    h = np.ascontiguousarray(wf.gb_waveform(w["A"], w["f"], w["fdot"], iota, phi0, psi,
                                            np.arange(n) * dt))
    h_dev = torch.as_tensor(h, device=device)
    n_out = output_samples(n, dt)
    steps = max(1, min(args.steps, 5))
    bat = flr.BatchedResponseTDI(1 / dt, order=w["order"], tdi=w["tdi"], orbits=orb,
                                 precision="mixed", tile="auto", tune_lengths=[n],
                                 force_backend=device)
    out = torch.empty((3, n), dtype=torch.float64, device=device)
    chunked = _timed(lambda: bat([h_dev], lam, beta, out=[out], chunks=SINGLE_CHUNKS), steps,
                     2, device)
    ev = {"on": False}
    lib = bm._plan_fns()
    restore = _timed_wrapped(lib, ["flr_batch_run"], ev)
    one = _timed(lambda: bat([h_dev], lam, beta, out=[out]), steps, 1, device, kernel_events=ev)
    restore()
    assert bat.status() == 0
    launch_s = _mean_ms(ev["flr_batch_run"]) * 1e-3
    tb = bat.tdi_sets[0]
    idx_ops = perfmodel.mixed_index_ops(
        tb["num_units"], perfmodel.prefix_shared_subtractions(_unit_lists(tb)))
    # plain FP64 drop-in path
    resp = flr.pyResponseTDI(1 / dt, n, order=w["order"], tdi=w["tdi"], orbits=orb,
                             force_backend=device)

    def plain_step():
        resp.get_projections(h_dev, lam, beta, t0=0.0, t_buffer=T_BUFFER)
        resp.get_tdi_delays()

    plain_steps = max(1, min(args.steps, 3))
    plain = _timed(plain_step, plain_steps, 1, device)
    acc = _rel_l2_rows(out, resp.XYZ)
    # the drop-in wrapper end to end: NumPy waveform in, NumPy channels out
    wrapped = {}
    prm = [w["A"], w["f"], w["fdot"], iota, phi0, psi, lam, beta]
    for prec, k in (("mixed", 5), (None, 3)):
        rw = flr.ResponseWrapper(lambda *a, **kw: h, n * dt / YRSID_SI, dt, 6, 7, orbits=orb,
                                 order=w["order"], tdi=w["tdi"], n_overide=n, precision=prec,
                                 remove_garbage=False, force_backend=device)
        holder = {}

        def e2e_step():
            holder["x"] = [c.cpu().numpy() for c in rw(*prm)]

        k = max(1, min(args.steps, k))
        wrapped["mixed" if prec else "plain_fp64"] = n_out * k / _timed(e2e_step, k, 1, device)
    return {
        "workload": w["desc"],
        "mixed": n_out * steps / chunked,
        "mixed_single_launch": n_out * steps / one,
        "plain_fp64": n_out * plain_steps / plain,
        "speedup_vs_plain_fp64": (n_out * steps / chunked) / (n_out * plain_steps / plain),
        "fp64_index_roofline_frac": idx_ops["total"] * n_out / launch_s / peaks["fp64_fma"],
        "launch_ms": 1e3 * launch_s,
        "max_rel_l2_vs_plain_fp64": acc,
        "e2e_dropin_numpy": wrapped,
        "e2e_api": "ResponseWrapper (waveform_gen returning a NumPy array; precision='mixed' "
                   "or the plain path) and .cpu().numpy() of the channels, per step",
    }


def run_precision_section(args, device):
    """Precision configuration: sources of 2^20 samples at dt = 10 s drawn as
    in the batching configuration, Lagrange orders 25 and 45; mixed against the
    FP64 fused path (bit-identical to the oracle) per link and per channel, and
    integer delay indices bit for bit."""
    import torch

    import fastlisaresponse_gb300 as flr

    def err_stats(got, want):
        d = got - want
        num = torch.linalg.vector_norm(d, dim=1)
        den = torch.linalg.vector_norm(want, dim=1)
        mx = d.abs().amax(dim=1) / want.abs().amax(dim=1).clamp_min(1e-300)
        return (num / den.clamp_min(1e-300)).cpu().numpy(), mx.cpu().numpy()

    dt, n = 10.0, 2**20
    count = args.precision_sources
    rng = np.random.default_rng(4)
    p = flr.waveforms.draw_gb_parameters(rng, count)
    orb = flr.EqualArmlengthOrbits(t_max=orbit_t_max(n, dt))
    t = torch.arange(n, dtype=torch.float64, device=device) * dt
    chunk = 16
    res = {"sources": count, "samples_per_source": n}
    for order in (25, 45):
        tb = 1e4 if order <= 25 else 2e4  # order 45 needs the longer garbage margin
        plans = {prec: flr.BatchedResponseTDI(1 / dt, order=order, tdi="2nd generation",
                                              orbits=orb, precision=prec, t_buffer=tb,
                                              force_backend=device)
                 for prec in ("fp64", "mixed")}
        ts = plans["fp64"].tdi_start_ind
        sl = slice(ts, n - ts)
        link_l2, chan_l2, chan_max = [], [], []
        mism = 0
        secs = {"fp64": 0.0, "mixed": 0.0}
        for c0 in range(0, count, chunk):
            idx = list(range(c0, min(count, c0 + chunk)))
            hs = [flr.gb_waveform(p["A"][i], p["f"][i], p["fdot"][i], p["iota"][i],
                                  p["phi0"][i], p["psi"][i], t) for i in idx]
            lam, beta = p["lam"][idx], p["beta"][idx]
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
                for key in ("d_rec", "d_em", "d_tdi"):
                    mism += int((dmx[key][:, sl] != d64[key][:, sl]).sum().item())
                link_l2.append(err_stats(dmx["y"][:, sl], d64["y"][:, sl])[0])
                a, b = err_stats(omx[:, sl], o64[:, sl])
                chan_l2.append(a)
                chan_max.append(b)
            del runs, hs
        link_l2, chan_l2 = np.asarray(link_l2), np.asarray(chan_l2)
        n_out = count * (n - 2 * ts)
        res[f"order_{order}"] = {
            "link_rel_l2_max": float(link_l2.max()),
            "channel_rel_l2_max": float(chan_l2.max()),
            "channel_rel_l2_median": float(np.median(chan_l2)),
            "channel_max_err_max": float(np.max(chan_max)),
            "index_mismatches": mism,
            "mixed_samples_per_s": n_out / secs["mixed"],
            "fp64_samples_per_s": n_out / secs["fp64"],
        }
        del plans
        torch.cuda.empty_cache()
    return res


def run_serving_section(args, device):
    """Open-loop Poisson request streams against ResponseServer: saturation
    throughput, then p50/p99 latency at rates below it."""
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
    orb = flr.EqualArmlengthOrbits(t_max=orbit_t_max(int(lengths.max()), dt))
    out = {"requests_per_rate": count}
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
    batched = sum(output_samples(nn) for nn in lengths[:nb]) / (e0.elapsed_time(e1) * 1e-3)
    out["batched_samples_per_s"] = batched
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
            return srv.stats()

    sat = run(None)
    out["saturation_samples_per_s"] = sat["throughput_samples_per_s"]
    cap = sat["throughput_requests_per_s"]
    out["rates"] = []
    full = {"saturation": sat, "rates": []}
    for frac in (0.5, 0.8, 0.9):
        st = run(frac * cap)
        full["rates"].append(st)
        out["rates"].append({"of_saturation": frac, "p50_ms": st["p50_ms"],
                             "p99_ms": st["p99_ms"],
                             "of_batched": st["throughput_samples_per_s"] / batched})

    # the device-resident loop on the same request streams (outputs allocated
    # before the clock starts; a poller records each request's completion)
    samples = np.asarray([output_samples(nn) for nn in lengths], dtype=np.float64)

    def run_device(rate):
        outs = [torch.empty((3, int(nn)), dtype=torch.float64, device=device) for nn in lengths]
        with flr.DeviceLoopServer(1 / dt, orbits=orb, capacity=count + 1, idle_seconds=0.02,
                                  force_backend=device) as srv:
            srv.submit(params[0], int(lengths[0]), int(sets[0])).result(timeout=60)  # warm-up
            arrivals = (np.cumsum(rng.exponential(1.0 / rate, count)) if rate
                        else np.zeros(count))
            tickets = [None] * count

            def client():
                t_start = time.perf_counter()
                for i in range(count):
                    delay = t_start + arrivals[i] - time.perf_counter()
                    if delay > 0:
                        time.sleep(delay)
                    tickets[i] = srv.submit(params[i], int(lengths[i]), int(sets[i]),
                                            out=outs[i])

            th = threading.Thread(target=client)
            th.start()
            pending = set(range(count))
            while pending:
                for i in [j for j in pending if tickets[j] is not None and tickets[j].done()]:
                    pending.discard(i)
                time.sleep(2e-5)
            th.join()
            assert srv.status() == 0
            lat = np.asarray([t.latency for t in tickets]) * 1e3
            span = max(t.t_done for t in tickets) - min(t.t_submit for t in tickets)
            info = srv.info()
        del outs
        return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "throughput_samples_per_s": float(samples.sum() / span),
                "launches": int(info["launches"])}

    dsat = run_device(None)
    dl = {"saturation_samples_per_s": dsat["throughput_samples_per_s"], "rates": []}
    for frac in (0.5, 0.8, 0.9):
        st = run_device(frac * cap)
        dl["rates"].append({"of_response_server_saturation": frac, "p50_ms": st["p50_ms"],
                            "p99_ms": st["p99_ms"], "launches": st["launches"],
                            "of_batched": st["throughput_samples_per_s"] / batched})
    out["device_loop"] = dl
    full["device_loop"] = dl
    return out, full


def run_ours(args, rank, world, device, cpu_line):
    peaks = measure_fp64_peak(device)
    head = run_headline(args, device, peaks, rank, world)
    result = {
        "metric": METRIC,
        "value": head["value"],
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": head["ms_per_step"],
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64 delays/indices + double-float (2xf32) taps; outputs f64",
        "data": "synthetic (seeded galactic binaries generated on the device; analytic "
                "equal-arm orbits)",
        "config": batch_config(args.batch_sources),
        "gpu_launches": head["gpu_launches"],
        "roofline": head["roofline"],
        "clocks": head["clocks"],
        "e2e": head["e2e"],
    }
    if cpu_line is not None:
        result["cpu_baseline"] = cpu_line
    details = {}
    if world == 1:
        result["single_source"] = run_single_source(args, device, peaks)
        if args.precision_sources > 0:
            result["precision"] = run_precision_section(args, device)
        if args.serve_requests > 0:
            result["serving"], details["serving"] = run_serving_section(args, device)
    # the line ends with the comparison on the same sources
    result["pipe_peaks_g_per_s"] = {k: v / 1e9 for k, v in peaks.items() if k != "sms"}
    result["plan"] = head["plan"]
    result["fp64_fused"] = head["fp64_fused"]
    result["mixed_on_subset"] = head["mixed_on_subset"]
    result["accuracy"] = head["accuracy"]
    result["plain_fp64"] = head["plain_fp64"]
    result["speedup_vs_plain_fp64"] = head["value"] / world / head["plain_fp64"]["value"]
    return result, details


def cpu_baseline_line(args, cores: int):
    steps, per_core = 2, 20
    r = cpu_rate(args.batch_sources, cores, steps=steps, warmup=0, tasks_per_core=per_core)
    return {"value": r["value"], "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{steps} x {cores * per_core} slices of {CPU_SLICE} output samples "
                      "(whole source when shorter) spread over the batch's sources, each with "
                      "its edge zones; C restatement of the reference's CPU path "
                      "(oracle/flr_oracle.c, gcc -O3), one process per core",
            "seconds": r["seconds"]}


def run_reference(args):
    cores = os.cpu_count() or 1
    r = cpu_rate(args.batch_sources, cores, steps=args.steps, warmup=args.warmup,
                 tasks_per_core=2)
    sample = (f"per step {2 * cores} slices of {CPU_SLICE} output samples (whole source when "
              "shorter) spread over the batch's sources, each with its edge zones")
    return {
        "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded galactic binaries; analytic equal-arm orbits)",
        "config": batch_config(args.batch_sources),
        "impl": "reference",
        "cpu_baseline": {"value": r["value"], "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "the reference's CPU path restated in C (oracle/flr_oracle.c, gcc -O3), pinned "
                "bit for bit to the reference's own compiled CPU code; the reference's sources "
                "and lisaanalysistools are not on the GPU host",
    }


def run_profile_batch(spec: str) -> None:
    """Small cases for ncu captures, spec = "<fp64|mixed|plain>:<kind>":
    kind equal|kepler: 16 galactic binaries x 2^18 samples at dt = 10 s with
    equal-arm or Keplerian orbits; kind batch64: the first 64 sources of the
    batching configuration (49.3 M samples, 2.0 GB of inputs and outputs).
    2nd-gen TDI XYZ, order 25; plain:<equal|kepler>: the plain FP64 drop-in
    path (pyResponseTDI) on one source of 2^21 samples at dt = 5 s.  An
    optional third field sets the tile of the batched cases (default: the
    library's).  Two calls (the capture takes the first)."""
    import torch

    import fastlisaresponse_gb300 as flr

    prec, kind, *rest = spec.split(":")
    tile = int(rest[0]) if rest else 0
    dev = torch.device("cuda", 0)
    if prec == "plain":
        # the plain FP64 drop-in path on one source of 2^21 samples at dt = 5 s
        dt, n = 5.0, 2**21
        orb = flr.EqualArmlengthOrbits(t_max=orbit_t_max(n, dt)) if kind == "equal" else \
            flr.KeplerianOrbits(t_max=orbit_t_max(n, dt))
        h = flr.gb_waveform(SINGLE["A"], SINGLE["f"], SINGLE["fdot"], 0.7, 0.3, 0.2,
                            torch.arange(n, dtype=torch.float64, device=dev) * dt)
        resp = flr.pyResponseTDI(1 / dt, n, order=25, tdi="2nd generation", orbits=orb,
                                 force_backend=dev)
        for _ in range(2):
            resp.get_projections(h, 1.0, 0.3, t_buffer=T_BUFFER)
            resp.get_tdi_delays()
        torch.cuda.synchronize()
        assert resp.status() == 0
        print(json.dumps({"profile_batch": spec, "computed_samples": n - 2 * resp.tdi_start_ind}))
        return
    dt = 10.0
    if kind == "batch64":
        lengths, p = batch_sources(BATCH["sources"])
        idx = list(range(64))
        lengths = lengths[:64]
        hs = _device_waveforms(lengths, p, idx, dt, dev)
        lam, beta = p["lam"][idx], p["beta"][idx]
        orb = flr.EqualArmlengthOrbits(t_max=orbit_t_max(int(lengths.max()), dt))
    else:
        ns, n = 16, 2**18
        rng = np.random.default_rng(5)
        t_max = orbit_t_max(n, dt)
        orb = flr.EqualArmlengthOrbits(t_max=t_max) if kind == "equal" else \
            flr.KeplerianOrbits(t_max=t_max)
        p = flr.waveforms.draw_gb_parameters(rng, ns)
        t = torch.arange(n, dtype=torch.float64, device=dev) * dt
        hs = [flr.gb_waveform(p["A"][i], p["f"][i], p["fdot"][i], p["iota"][i], p["phi0"][i],
                              p["psi"][i], t) for i in range(ns)]
        lam, beta = p["lam"], p["beta"]
    bat = flr.BatchedResponseTDI(1 / dt, order=25, tdi="2nd generation", orbits=orb,
                                 precision=prec, tile=tile)
    for _ in range(2):
        bat(hs, lam, beta)
    torch.cuda.synchronize()
    assert bat.status() == 0
    samples = sum(len(h) - 2 * bat.tdi_start_ind for h in hs)
    print(json.dumps({"profile_batch": spec, "computed_samples": samples,
                      "plan": bat.plan_info}))


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batch-sources", type=int, default=BATCH["sources"],
                    help="sources of the headline batch (default 2048)")
    ap.add_argument("--serve-requests", type=int, default=1000,
                    help="requests per arrival rate in the serving section (0 = skip)")
    ap.add_argument("--precision-sources", type=int, default=32,
                    help="sources of 2^20 samples in the precision section (0 = skip)")
    ap.add_argument("--details", default=None, metavar="FILE",
                    help="also write the serving section's full statistics to FILE")
    ap.add_argument("--profile-batch", default=None, metavar="PREC:ORBIT",
                    help="run only a small profiling case (fp64|mixed:equal|kepler|batch64, plain:equal|kepler)")
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
    result, details = run_ours(args, rank, world, device, cpu_line)
    if rank == 0:
        if args.details:
            with open(args.details, "w") as fh:
                json.dump(details, fh, indent=1)
        print(json.dumps(result), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
