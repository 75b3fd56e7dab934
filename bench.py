#!/usr/bin/env python
"""Benchmark of the labelled-reduction + fill workload on GB300.

Workload (numbagg's grouped / fill hot path): float64 values of shape
64 x 16,777,216, N(0,1) with 5% NaN; int32 labels along the last axis, uniform in
[0, K) for K in {16, 4096, 1,000,000}; group_nansum / nanmean / nanvar / nancount /
nanargmax for each K; ffill / bfill with limit=None and limit=5 on the same values
re-masked with NaN runs of geometric length (p = 0.3).  One step = those 19 calls.

Metric: algorithmic HBM bytes per second (GB/s) over the step, per function and in
aggregate, as a fraction of the measured copy bandwidth.  Algorithmic bytes per
call: grouped 8*R*M (values) + 4*M (labels, shared by the rows) + 8*R*K (output);
fill 16*R*M (read + write).

    python bench.py [--gpus N --steps K --warmup W] [--impl reference]

N > 1 runs one replica per GPU (launched with torchrun); the path has no exchange
step, so ranks only synchronise around the timed region.  `--impl reference` times
numbagg's algorithm on the host cores (the C restatement of its loops, OpenMP over
rows like numba's parallel target) on a bounded sample of the same workload.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

ROWS = 64
COLS = 16_777_216
NAN_P = 0.05
KS = (16, 4096, 1_000_000)
GROUP_FUNCS = ("nansum", "nanmean", "nanvar", "nancount", "nanargmax")
FILL_LIMITS = (None, 5)
RUN_START_P = 0.015  # NaN-run starts per position for the fill input (runs ~Geometric(0.3))
RUN_P = 0.3
SAMPLE_COLS_CPU = 2_097_152  # bounded sample for the host-core timings (1/8 of the columns)
METRIC = "HBM GB/s & % of peak per func; FP32-compensated vs FP64 speedup at stated err"


def parse_args(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=("ours", "reference"), default="ours")
    # the end-to-end pipeline starts empty and drains at the end (about 0.8 s of fill and
    # drain measured on a GB300); 32 steps keep that within about 10% of the steady state
    p.add_argument("--e2e-steps", type=int, default=32)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--cols", type=int, default=COLS, help="columns (smaller for quick runs)")
    p.add_argument("--only", default=None, help="regex: time only the calls whose key matches (profiling)")
    p.add_argument(
        "--suite",
        choices=("group_fill", "scan", "ragged", "link", "aggregate", "columns"),
        default="group_fill",
        help="group_fill: the headline workload; scan: the moving-window, EWM and matrix shapes; "
        "ragged: the batched mix of series of uneven length; link: pinned host<->device copy "
        "bandwidth (the bound of the end-to-end number); aggregate: the static aggregations; "
        "columns: a non-last axis in place against moving it last with a copy",
    )
    p.add_argument("--ragged-series", type=int, default=100_000, help="series in the ragged batch")
    p.add_argument(
        "--no-configs",
        action="store_true",
        help="skip the other workloads (moving windows / EWM on the precision-stress data with their fp32c "
        "speed-up and errors, the small graph-replayed move_mean, the matrices, the ragged mix) that the "
        "default run reports beside the headline",
    )
    return p.parse_args(argv)


# ---- multi-process helpers (replicas) ---------------------------------------------------


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reduce_max(value: float, device=None) -> float:
    """Maximum of `value` over all ranks (identity without a process group)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return value
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier():
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized():
        dist.barrier()


# ---- workload ---------------------------------------------------------------------------


def calls_and_bytes(rows: int, cols: int):
    """(key, kind, args) for the 19 calls of one step, with algorithmic bytes."""
    out = []
    for K in KS:
        for f in GROUP_FUNCS:
            out.append((f"group_{f}_K{K}", ("group", f, K), 8 * rows * cols + 4 * cols + 8 * rows * K))
    for lim in FILL_LIMITS:
        for f in ("ffill", "bfill"):
            out.append((f"{f}_limit{lim}", ("fill", f, lim), 16 * rows * cols))
    return out


def make_inputs(rows: int, cols: int, device):
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(1)
    values = torch.randn((rows, cols), generator=g, dtype=torch.float64, device=device)
    values[torch.rand((rows, cols), generator=g, device=device) < NAN_P] = float("nan")
    labels = {}
    for K in KS:
        gk = torch.Generator(device=device)
        gk.manual_seed(1000 + K)
        labels[K] = torch.randint(0, K, (cols,), generator=gk, dtype=torch.int32, device=device)
    # fill input: the same values re-masked with NaN runs of geometric length
    fill = values.clone()
    starts = torch.rand((rows, cols), generator=g, device=device) < RUN_START_P
    r_idx, c_idx = torch.nonzero(starts, as_tuple=True)
    del starts
    u = torch.rand(r_idx.shape, generator=g, dtype=torch.float64, device=device).clamp_min(1e-300)
    lengths = (torch.floor(torch.log(u) / math.log(1.0 - RUN_P)) + 1).to(torch.int64)  # Geometric(RUN_P)
    ends = torch.clamp(c_idx + lengths, max=cols)
    delta = torch.zeros((rows, cols + 1), dtype=torch.int32, device=device)
    delta.index_put_((r_idx, c_idx), torch.ones_like(c_idx, dtype=torch.int32), accumulate=True)
    delta.index_put_((r_idx, ends), -torch.ones_like(c_idx, dtype=torch.int32), accumulate=True)
    covered = torch.cumsum(delta[:, :cols], dim=1) > 0
    del delta
    fill[covered] = float("nan")
    del covered
    return values, labels, fill


def run_call(nb, spec, values, labels, fill):
    kind, f, arg = spec
    if kind == "group":
        return getattr(nb, f"group_{f}")(values, labels[arg], num_labels=arg, axis=-1)
    return getattr(nb, f)(fill, limit=arg)


# ---- clocks ------------------------------------------------------------------------------


class ClockSampler:
    FIELDS = (
        "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
        "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
        "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"
    )

    def __init__(self, gpu_index: int):
        self.gpu_index = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self._thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu_index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL,
                text=True,
            )
        except (OSError, ValueError):
            self.proc = None
            return
        self._thread = threading.Thread(target=self._read, daemon=True)
        self._thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self._thread:
            self._thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names[1:], parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(smax) if smax else None,
            "reasons": sorted(reasons),
            "samples": len(sm),
        }


def measured_peak() -> tuple[float, str]:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def traffic_for(key: str):
    """DRAM bytes per launch of the dominant call, from a committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as fh:
            data = json.load(fh)
        return data.get(key)
    except (OSError, ValueError):
        return None


# ---- CPU timing (oracle = numbagg's loops restated in C, OpenMP over rows) ---------------


def cpu_step(values_np, labels_np, fill_np):
    import oracle

    t0 = time.perf_counter()
    for K in KS:
        lab = labels_np[K]
        for f in GROUP_FUNCS:
            oracle.group(f"group_{f}", values_np, lab, num_labels=K, axis=-1)
    for lim in FILL_LIMITS:
        for f in ("ffill", "bfill"):
            oracle.fill(f, fill_np, limit=lim)
    return time.perf_counter() - t0


def cpu_sample(values, labels, fill, cols):
    sc = min(cols, SAMPLE_COLS_CPU)
    v = values[:, :sc].cpu().numpy()
    fl = fill[:, :sc].cpu().numpy()
    lab = {K: labels[K][:sc].cpu().numpy() for K in KS}
    return v, lab, fl, sc


def sample_bytes(rows, sc):
    return sum(b for _, _, b in calls_and_bytes(rows, sc))


def sample_desc(rows, sc):
    return (
        f"{rows} x {sc} columns (first {sc} of {COLS}) of the same inputs, the 19 calls once; "
        "numbagg's loops restated in C (oracle), OpenMP schedule(static) over rows; the sample keeps every "
        "call's full output (rows x K), so with K = 10^6 the per-element cost includes 8x more output per "
        "input element than the full workload"
    )


# ---- the reference arm --------------------------------------------------------------------


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    import numpy as np

    import oracle

    oracle.lib()
    rng = np.random.default_rng(1)
    sc = min(args.cols, SAMPLE_COLS_CPU)
    values = rng.standard_normal((ROWS, sc))
    values[rng.random(values.shape) < NAN_P] = np.nan
    fill = values.copy()
    rr, cc = np.nonzero(rng.random(values.shape) < RUN_START_P)
    ends = np.minimum(cc + rng.geometric(RUN_P, size=cc.shape), sc)
    delta = np.zeros((ROWS, sc + 1), dtype=np.int32)
    np.add.at(delta, (rr, cc), 1)
    np.add.at(delta, (rr, ends), -1)
    fill[np.cumsum(delta[:, :sc], axis=1) > 0] = np.nan
    labels = {K: rng.integers(0, K, size=sc).astype(np.int32) for K in KS}
    for _ in range(args.warmup):
        cpu_step(values, labels, fill)
    t = 0.0
    for _ in range(args.steps):
        t += cpu_step(values, labels, fill)
    ms = 1000.0 * t / max(args.steps, 1)
    gbs = sample_bytes(ROWS, sc) / (ms / 1000.0) / 1e9
    cores = os.cpu_count()
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": gbs,
        "unit": "GB/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": workload_config(ROWS, args.cols),
        "cpu_baseline": {"value": gbs, "unit": "GB/s", "cores": cores, "kind": "port", "sample": sample_desc(ROWS, sc)},
        "e2e": {"value": gbs, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def workload_config(rows, cols):
    return {
        "workload": f"group_nan{{sum,mean,var,count,argmax}} x K in {list(KS)} + ffill/bfill limit in [None, 5]; "
        f"float64 values {rows}x{cols}, 5% NaN; int32 labels",
        "rows": rows,
        "cols": cols,
        "num_labels": list(KS),
        "fill_nan_runs": f"starts Bernoulli({RUN_START_P}) per position, length Geometric({RUN_P})",
        "l2": "inputs larger than L2 (each float64 array is 8.6 GB, L2 is 129 MB)",
        "parallelism": "replicas",
    }


# ---- our arm --------------------------------------------------------------------------------


def run_ours(args):
    import torch
    import torch.distributed as dist

    world, rank, local = dist_env()
    if world > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    device = torch.device("cuda", local if world > 1 else torch.cuda.current_device())
    torch.cuda.set_device(device)
    import numbagg_gb300 as nb
    from numbagg_gb300 import _lib

    rows, cols = ROWS, args.cols
    values, labels, fill = make_inputs(rows, cols, device)
    calls = calls_and_bytes(rows, cols)
    if args.only:
        import re

        calls = [c for c in calls if re.search(args.only, c[0])]
    torch.cuda.synchronize(device)

    for _ in range(args.warmup):
        for _, spec, _ in calls:
            run_call(nb, spec, values, labels, fill)
    torch.cuda.synchronize(device)

    stream = torch.cuda.current_stream(device)
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(len(calls) + 1)] for _ in range(args.steps)]
    sampler = ClockSampler(device.index or 0)
    sampler.start()
    time.sleep(0.3)
    barrier()
    torch.cuda.synchronize(device)
    launches0 = _lib.launch_count()
    for s in range(args.steps):
        ev[s][0].record(stream)
        for i, (_, spec, _) in enumerate(calls):
            run_call(nb, spec, values, labels, fill)
            ev[s][i + 1].record(stream)
    torch.cuda.synchronize(device)
    barrier()
    launches = _lib.launch_count() - launches0
    clocks = sampler.stop()

    per_call_ms = [0.0] * len(calls)
    total_ms = 0.0
    for s in range(args.steps):
        total_ms += ev[s][0].elapsed_time(ev[s][-1])
        for i in range(len(calls)):
            per_call_ms[i] += ev[s][i].elapsed_time(ev[s][i + 1])
    ms_step = total_ms / args.steps
    ms_step = reduce_max(ms_step, device)
    step_bytes = sum(b for _, _, b in calls)
    value = world * step_bytes / (ms_step / 1000.0) / 1e9

    peak, peak_kind = measured_peak()
    per_func = {}
    for (key, _, b), t in zip(calls, per_call_ms):
        avg = t / args.steps
        gbs = b / (avg / 1000.0) / 1e9
        per_func[key] = {"ms": round(avg, 4), "GB/s": round(gbs, 1), "frac": round(gbs / peak, 4)}
    dom = max(range(len(calls)), key=lambda i: per_call_ms[i])
    dom_key, _, dom_bytes = calls[dom]
    dom_ms = per_call_ms[dom] / args.steps
    achieved = dom_bytes / (dom_ms / 1000.0) / 1e9
    roofline = {
        "bound": "hbm",
        "kernel": dom_key,
        "achieved": round(achieved, 1),
        "peak": peak,
        "peak_kind": peak_kind,
        "unit": "GB/s",
        "frac": round(achieved / peak, 4),
        "traffic": traffic_for(dom_key),
        "bytes_per_launch": dom_bytes,
    }

    e2e = None
    if not args.no_e2e and args.e2e_steps > 0:
        e2e = run_e2e(args, nb, values, labels, fill, calls, device, world)

    cpu = None
    if rank == 0 and not args.no_cpu and world == 1:
        v, lab, fl, sc = cpu_sample(values, labels, fill, cols)
        import oracle

        oracle.lib()
        t = cpu_step(v, lab, fl)
        cpu = {
            "value": round(sample_bytes(rows, sc) / t / 1e9, 2),
            "unit": "GB/s",
            "cores": os.cpu_count(),
            "kind": "port",
            "sample": sample_desc(rows, sc),
        }

    configs = None
    if rank == 0 and world == 1 and not args.no_configs and not args.only:
        del values, labels, fill
        configs = run_configs(nb, device, args)

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": round(value, 1),
            "unit": "GB/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": round(ms_step, 3),
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64",
            "data": "synthetic",
            "config": workload_config(rows, cols),
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": int(launches),
            "clocks": clocks,
            "per_func": per_func,
        }
        if configs is not None:
            line["configs"] = configs["configs"]
            line["fp32c"] = configs["fp32c"]
            line["gpu_launches_configs"] = configs["gpu_launches"]
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


CONFIG_STEPS, CONFIG_WARMUP = 2, 1  # the other workloads: timed steps per call, warm-up calls


def run_configs(nb, device, args):
    """The other workloads of the metric, measured after the headline (whose inputs
    are freed first), each call warmed up once and timed over CONFIG_STEPS calls:
      * the moving windows and EWM functions on the precision-stress data
        (1024 x 1,048,576 float64) in plain float64 and FP32-compensated form, with
        each form's error against the exact reference and the fp32c speed-up;
      * the 100 x 10,000 move_mean replayed from CUDA graphs;
      * move_covmatrix / move_corrmatrix on 65,536 x 256 float32;
      * the ragged batched mix."""
    import gc

    import torch

    gc.collect()
    torch.cuda.empty_cache()
    cols = min(args.cols, SCAN_COLS)
    per_func, speedup, l1 = measure_scan(nb, device, cols, CONFIG_STEPS, CONFIG_WARMUP)
    ragged, rconf, l2 = measure_ragged(nb, device, args.ragged_series, CONFIG_STEPS, CONFIG_WARMUP)
    fp32c = {}
    for base, sp in speedup.items():
        fp32c[base] = {
            "speedup": sp,
            "plain_ms": per_func[base]["ms"],
            "fp32c_ms": per_func[base + "_fp32c"]["ms"],
            "max_rel_err_plain": per_func[base].get("max_rel_err_vs_exact"),
            "max_rel_err_fp32c": per_func[base + "_fp32c"].get("max_rel_err_vs_exact"),
            "max_scaled_err_plain": per_func[base].get("max_scaled_err_vs_exact"),
            "max_scaled_err_fp32c": per_func[base + "_fp32c"].get("max_scaled_err_vs_exact"),
        }
    fp32c["ragged_mix"] = {
        "speedup": round(ragged["f64"]["ms_per_mix"] / ragged["fp32c"]["ms_per_mix"], 2),
        "plain_ms": ragged["f64"]["ms_per_mix"],
        "fp32c_ms": ragged["fp32c"]["ms_per_mix"],
    }
    configs = {
        "move_mean_100x10000_w20": per_func.pop("move_mean_small_w20"),
        "precision_stress": {"config": scan_config(cols), "per_func": {k: v for k, v in per_func.items() if "matrix" not in k}},
        "matrices_65536x256_f32_w500": {k: v for k, v in per_func.items() if "matrix" in k},
        "ragged_mix": {"config": rconf, "results": ragged},
        "timing": f"each call warmed up {CONFIG_WARMUP}x, then {CONFIG_STEPS} calls timed with CUDA events",
    }
    return {"configs": configs, "fp32c": fp32c, "gpu_launches": l1 + l2}


def run_e2e(args, nb, values, labels, fill, calls, device, world):
    """The same step through the public API with host buffers: every step copies its
    inputs from pinned host memory and reads every result back into pinned memory.
    Three streams overlap the work as a production pipeline would: host-to-device copies
    (into double-buffered device inputs, so step k+1's inputs arrive while step k
    computes), the calls, and device-to-host copies of each result as soon as its call
    has finished."""
    import torch

    h_values = torch.empty(values.shape, dtype=values.dtype, pin_memory=True)
    h_fill = torch.empty(fill.shape, dtype=fill.dtype, pin_memory=True)
    h_values.copy_(values)
    h_fill.copy_(fill)
    h_labels = {K: torch.empty(labels[K].shape, dtype=labels[K].dtype, pin_memory=True).copy_(labels[K]) for K in KS}
    h_out_fill = torch.empty(fill.shape, dtype=fill.dtype, pin_memory=True)
    h_out_group = {K: torch.empty((values.shape[0], K), dtype=torch.float64, pin_memory=True) for K in KS}
    comp = torch.cuda.current_stream(device)
    s_in = torch.cuda.Stream(device)
    s_out = torch.cuda.Stream(device)
    # the fill calls first: their outputs are most of the bytes read back, so the
    # device-to-host stream starts as early as possible in each step
    calls = [c for c in calls if c[1][0] == "fill"] + [c for c in calls if c[1][0] != "fill"]
    h2d = values.numel() * 8 + fill.numel() * 8 + sum(labels[K].numel() * 4 for K in KS)
    d2h = 0
    for _, (kind, f, arg), _ in calls:
        d2h += fill.numel() * 8 if kind == "fill" else values.shape[0] * arg * 8
    # two sets of device inputs (the timed values/fill tensors are reused as one of them)
    sets = [
        (values, fill, dict(labels)),
        (torch.empty_like(values), torch.empty_like(fill), {K: torch.empty_like(labels[K]) for K in KS}),
    ]
    released = [None, None]  # compute-stream event after the last use of each set
    drained = {}  # device-to-host event after each step's last read-back

    def step(k):
        d_values, d_fill, d_labels = sets[k % 2]
        # at most two steps of results waiting for the read-back (bounds device memory)
        if k - 2 in drained:
            comp.wait_event(drained.pop(k - 2))
        with torch.cuda.stream(s_in):
            if released[k % 2] is not None:
                s_in.wait_event(released[k % 2])
            d_fill.copy_(h_fill, non_blocking=True)
            ev_fill = s_in.record_event()
            d_values.copy_(h_values, non_blocking=True)
            for K in KS:
                d_labels[K].copy_(h_labels[K], non_blocking=True)
            ev_group = s_in.record_event()
        comp.wait_event(ev_fill)
        for _, spec, _ in calls:
            kind, f, arg = spec
            if kind == "group":
                comp.wait_event(ev_group)
            r = run_call(nb, spec, d_values, d_labels, d_fill)
            done = comp.record_event()
            with torch.cuda.stream(s_out):
                s_out.wait_event(done)
                (h_out_fill if kind == "fill" else h_out_group[arg]).copy_(r, non_blocking=True)
                r.record_stream(s_out)
        released[k % 2] = comp.record_event()
        drained[k] = s_out.record_event()

    step(0)
    torch.cuda.synchronize(device)
    barrier()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(comp)
    s_in.wait_event(t0)
    for k in range(args.e2e_steps):
        step(k + 1)
    comp.wait_stream(s_in)
    comp.wait_stream(s_out)
    t1.record(comp)
    torch.cuda.synchronize(device)
    barrier()
    ms = reduce_max(t0.elapsed_time(t1) / args.e2e_steps, device)
    step_bytes = sum(b for _, _, b in calls)
    return {
        "value": round(world * step_bytes / (ms / 1000.0) / 1e9, 1),
        "unit": "GB/s",
        "h2d_bytes_per_step": int(h2d),
        "d2h_bytes_per_step": int(d2h),
        "ms_per_step": round(ms, 3),
        "steps": args.e2e_steps,
        "streams": "host-to-device, compute, device-to-host (overlapped; inputs double-buffered)",
    }


# ---- the scan suite: moving windows, EWM, matrices -----------------------------------------

SCAN_ROWS, SCAN_COLS = 1024, 1_048_576  # precision-stress shape
SCAN_WINDOWS = (5, 252, 10_000)
SCAN_ALPHAS = (0.5, 0.01, 1e-4)
SMALL_ROWS, SMALL_COLS = 100, 10_000  # the reference's CPU-runnable move_mean case
MATRIX_T, MATRIX_V = 65_536, 256


def scan_inputs(device, cols):
    """a = 1e6 + z1, b = 1e6 + 0.7 z1 + sqrt(0.51) z2 (correlation 0.7), 2% NaN each."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(3)
    z1 = torch.randn((SCAN_ROWS, cols), generator=g, dtype=torch.float64, device=device)
    b = torch.randn((SCAN_ROWS, cols), generator=g, dtype=torch.float64, device=device)
    b.mul_(math.sqrt(0.51)).add_(z1, alpha=0.7).add_(1e6)
    a = z1.add_(1e6)
    a[torch.rand(a.shape, generator=g, device=device) < 0.02] = float("nan")
    b[torch.rand(b.shape, generator=g, device=device) < 0.02] = float("nan")
    g.manual_seed(0)
    small = torch.randn((SMALL_ROWS, SMALL_COLS), generator=g, dtype=torch.float64, device=device)
    small[torch.rand(small.shape, generator=g, device=device) < 0.10] = float("nan")
    g.manual_seed(4)
    A = torch.randn((MATRIX_V, MATRIX_V), generator=g, dtype=torch.float64, device=device) / 16.0
    Z = torch.randn((MATRIX_T, MATRIX_V), generator=g, dtype=torch.float64, device=device)
    X = (Z @ A.T).to(torch.float32)
    X[torch.rand(X.shape, generator=g, device=device) < 0.01] = float("nan")
    return a, b, small, X


class _Fp32c:
    """The package with precision="fp32c" added to every call."""

    def __init__(self, nb):
        self._nb = nb

    def __getattr__(self, name):
        f = getattr(self._nb, name)
        return lambda *args, **kw: f(*args, precision="fp32c", **kw)


def scan_calls(cols):
    """(key, callable(nb, a, b, small, X), algorithmic bytes, elements) of the scan suite.
    min_count = window // 2: with 2% NaN the default (= window) leaves almost every
    output NaN at the two larger windows."""
    R, N = SCAN_ROWS, cols
    out = []
    for w in SCAN_WINDOWS:
        out.append((f"move_std_w{w}", lambda nb, a, b, s, X, w=w: nb.move_std(a, window=w, min_count=w // 2), 16 * R * N, R * N))
    for w in SCAN_WINDOWS:
        out.append(
            (f"move_corr_w{w}", lambda nb, a, b, s, X, w=w: nb.move_corr(a, b, window=w, min_count=w // 2), 24 * R * N, R * N)
        )
    for al in SCAN_ALPHAS:
        out.append((f"move_exp_nanmean_a{al:g}", lambda nb, a, b, s, X, al=al: nb.move_exp_nanmean(a, alpha=al), 16 * R * N, R * N))
        out.append((f"move_exp_nanvar_a{al:g}", lambda nb, a, b, s, X, al=al: nb.move_exp_nanvar(a, alpha=al), 16 * R * N, R * N))
        out.append(
            (f"move_exp_nancorr_a{al:g}", lambda nb, a, b, s, X, al=al: nb.move_exp_nancorr(a, b, alpha=al), 24 * R * N, R * N)
        )
    # the FP32-compensated forms of the same calls
    for key, fn, nbytes, elems in list(out):
        out.append((key + "_fp32c", lambda nb, a, b, s, X, fn=fn: fn(_Fp32c(nb), a, b, s, X), nbytes, elems))
    T, V = MATRIX_T, MATRIX_V
    for f in ("move_covmatrix", "move_corrmatrix"):
        out.append((f"{f}_w500", lambda nb, a, b, s, X, f=f: getattr(nb, f)(X, window=500, min_count=400), 4 * T * V + 4 * T * V * V, T * V))
    return out


def measure_scan(nb, device, cols, steps, warmup, only=None, errors=True, error_rows=2, error_positions=2048):
    """Time every call of the scan suite (each warmed up, then `steps` back to back) and,
    with `errors`, measure each moving / EWM result's error in both forms against
    the exact reference at sampled positions of the first rows."""
    import re

    import torch

    from numbagg_gb300 import _lib

    a, b, small, X = scan_inputs(device, cols)
    calls = scan_calls(cols)
    if only:
        calls = [c for c in calls if re.search(only, c[0])]
    peak, _ = measured_peak()
    stream = torch.cuda.current_stream(device)
    per_func = {}
    launches0 = _lib.launch_count()
    for key, fn, nbytes, elems in calls:
        for _ in range(warmup):
            fn(nb, a, b, small, X)
        torch.cuda.synchronize(device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn(nb, a, b, small, X)
        e1.record(stream)
        torch.cuda.synchronize(device)
        ms = e0.elapsed_time(e1) / steps
        gbs = nbytes / (ms / 1000.0) / 1e9
        entry = {"ms": round(ms, 4), "GB/s": round(gbs, 1), "frac": round(gbs / peak, 4), "Gelem/s": round(elems / ms / 1e6, 2)}
        if errors and not key.startswith(("move_covmatrix", "move_corrmatrix")):
            res = fn(nb, a[:error_rows], b[:error_rows], small, X)
            errs, serrs = [], []
            for r in range(min(error_rows, res.shape[0])):
                pos = _sample_positions(cols, error_positions, device)
                base = key[: -len("_fp32c")] if key.endswith("_fp32c") else key
                if base.startswith("move_exp_"):
                    fname, al = base.rsplit("_a", 1)
                    exact, scale = exact_move_exp(fname, a[r], b[r] if "corr" in fname else None, float(al), pos)
                else:
                    fname, w = base.rsplit("_w", 1)
                    w = int(w)
                    exact, scale = exact_move(fname, a[r], b[r] if fname == "move_corr" else None, w, w // 2, pos)
                e, se = max_errors(res[r][pos], exact, scale)
                if e is not None:
                    errs.append(e)
                    serrs.append(se)
            entry["max_rel_err_vs_exact"] = float(f"{max(errs):.3g}") if errs else None
            entry["max_scaled_err_vs_exact"] = float(f"{max(serrs):.3g}") if serrs else None
        per_func[key] = entry
    # the 100 x 10,000 move_mean (16 MB, resident in L2): replayed from a CUDA graph
    if not only or re.search(only, "move_mean_small"):
        fn = lambda: nb.move_mean(small, window=20, min_count=20)  # noqa: E731
        s2 = torch.cuda.Stream(device)
        s2.wait_stream(stream)
        with torch.cuda.stream(s2):
            for _ in range(3):
                fn()
        stream.wait_stream(s2)
        torch.cuda.synchronize(device)
        graph = torch.cuda.CUDAGraph()
        reps = 100
        with torch.cuda.graph(graph, stream=s2):
            for _ in range(reps):
                fn()
        graph.replay()
        torch.cuda.synchronize(device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(10):
            graph.replay()
        e1.record(stream)
        torch.cuda.synchronize(device)
        us = e0.elapsed_time(e1) * 1000.0 / (10 * reps)
        nbytes = 16 * SMALL_ROWS * SMALL_COLS
        per_func["move_mean_small_w20"] = {
            "us": round(us, 2),
            "GB/s": round(nbytes / (us / 1e6) / 1e9, 1),
            "note": "16 MB, L2-resident; 1000 launches replayed from CUDA graphs",
        }
    speedup = {
        k[: -len("_fp32c")]: round(per_func[k[: -len("_fp32c")]]["ms"] / v["ms"], 2)
        for k, v in per_func.items()
        if k.endswith("_fp32c") and k[: -len("_fp32c")] in per_func
    }
    del a, b, small, X
    torch.cuda.empty_cache()
    return per_func, speedup, int(_lib.launch_count() - launches0)


def scan_config(cols):
    return {
        "scan": f"{SCAN_ROWS}x{cols} float64, a = 1e6 + z1, b = 1e6 + 0.7 z1 + sqrt(0.51) z2, 2% NaN; min_count = window // 2",
        "matrix": f"{MATRIX_T}x{MATRIX_V} float32 from N(0, A A^T / 256), 1% NaN, window 500, min_count 400",
        "small": f"{SMALL_ROWS}x{SMALL_COLS} float64 N(0,1), 10% NaN, window 20, min_count 20",
        "errors": "at 2048 evenly spaced positions of each of the first 2 rows: max |got - exact| / |exact| "
        "(relative) and max |got - exact| / max(|exact|, S) (scaled; S = 1 for correlations, the mean square of "
        "the data minus 1e6 for variances, its root for standard deviations); exact = two-pass float64 sums of "
        "the data minus 1e6 (exact by Sterbenz) over each window, or over the weights (1 - alpha)^k down to 1e-20",
    }


def run_scan_suite(args):
    import torch

    import numbagg_gb300 as nb

    world, rank, local = dist_env()
    device = torch.device("cuda", local if world > 1 else torch.cuda.current_device())
    torch.cuda.set_device(device)
    cols = min(args.cols, SCAN_COLS)
    per_func, speedup, launches = measure_scan(nb, device, cols, args.steps, args.warmup, args.only)
    peak, peak_kind = measured_peak()
    line = {
        "suite": "scan",
        "fp32c_speedup": speedup,
        "unit": "GB/s",
        "peak": peak,
        "peak_kind": peak_kind,
        "dtype": "f64 (matrices: f32 in, f32 out)",
        "config": scan_config(cols),
        "steps": args.steps,
        "warmup": args.warmup,
        "gpu_launches": launches,
        "per_func": per_func,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


# ---- error against an exact float64 reference (precision-stress data) ----------------------
#
# The data are a = 1e6 + z1, b = 1e6 + 0.7 z1 + sqrt(0.51) z2: subtracting 1e6 is exact
# (Sterbenz), and every statistic here is shift invariant (the means shift back), so
# the reference statistics are computed on z with two-pass float64 sums, directly
# over each sampled position's window (or, for the exponential forms, over the
# weights (1 - alpha)^(t - s) down to 1e-20), on the GPU with torch.
PIVOT = 1e6


def _sample_positions(n, count, device, lo=0):
    import torch

    count = max(1, min(count, n - lo))
    return torch.linspace(lo, n - 1, count, device=device).round().to(torch.int64).unique()


def exact_move(fname, a_row, b_row, window, min_count, pos):
    """numbagg's move_std / move_corr at positions `pos` of one row, exactly enough to
    measure float64 errors (numbagg/moving.py:123-151, :223-275)."""
    import torch

    k = torch.arange(window, device=pos.device)
    idx = pos[:, None] - k[None, :]
    inside = idx >= 0
    idx = idx.clamp_min(0)
    za = a_row[idx] - PIVOT
    valid = inside & ~torch.isnan(za)
    if b_row is not None:
        zb = b_row[idx] - PIVOT
        valid &= ~torch.isnan(zb)
    n = valid.sum(1).to(torch.float64)
    za = torch.where(valid, za, 0.0)
    ma = za.sum(1) / n
    da = torch.where(valid, za - ma[:, None], 0.0)
    if b_row is None:
        var = (da * da).sum(1) / (n - 1)
        res = torch.sqrt(var)
        scale = torch.sqrt((za * za).sum(1) / n)  # the root mean square of the window
        return torch.where(n >= max(min_count, 2), res, float("nan")), scale
    zb = torch.where(valid, zb, 0.0)
    mb = zb.sum(1) / n
    db = torch.where(valid, zb - mb[:, None], 0.0)
    res = (da * db).sum(1) / torch.sqrt((da * da).sum(1) * (db * db).sum(1))
    return torch.where(n >= max(min_count, 1), res, float("nan")), torch.ones_like(res)


def exact_move_exp(fname, a_row, b_row, alpha, pos):
    """move_exp_nanmean / nanvar / nancorr at positions `pos` of one row with a scalar
    alpha and min_weight 0 (numbagg/moving_exp.py:41-156, :275-335)."""
    import torch

    L = int(min(math.ceil(math.log(1e-20) / math.log1p(-alpha)), 1 << 22)) if alpha < 1 else 1
    out = torch.empty(pos.shape, dtype=torch.float64, device=pos.device)
    scale = torch.empty(pos.shape, dtype=torch.float64, device=pos.device)
    step = max(1, (1 << 24) // L)
    k = torch.arange(L, device=pos.device)
    w_all = torch.exp(k.to(torch.float64) * math.log1p(-alpha))
    for s0 in range(0, pos.numel(), step):
        p = pos[s0 : s0 + step]
        idx = p[:, None] - k[None, :]
        inside = idx >= 0
        idx = idx.clamp_min(0)
        za = a_row[idx] - PIVOT
        valid = inside & ~torch.isnan(za)
        if b_row is not None:
            zb = b_row[idx] - PIVOT
            valid &= ~torch.isnan(zb)
        w = torch.where(valid, w_all[None, :], 0.0)
        sw = w.sum(1)
        sw2 = (w * w).sum(1)
        za = torch.where(valid, za, 0.0)
        ma = (w * za).sum(1) / sw
        if fname == "move_exp_nanmean":
            r = ma + PIVOT
            sc = r.abs()
        else:
            da = torch.where(valid, za - ma[:, None], 0.0)
            bias = 1 - sw2 / (sw * sw)
            if fname == "move_exp_nanvar":
                r = torch.where(bias > 0, (w * da * da).sum(1) / sw / bias, float("nan"))
                sc = (w * za * za).sum(1) / sw  # the weighted mean square
            else:
                zb = torch.where(valid, zb, 0.0)
                mb = (w * zb).sum(1) / sw
                db = torch.where(valid, zb - mb[:, None], 0.0)
                r = (w * da * db).sum(1) / torch.sqrt((w * da * da).sum(1) * (w * db * db).sum(1))
                r = torch.where(bias > 0, r, float("nan"))
                sc = torch.ones_like(r)
        out[s0 : s0 + step] = r
        scale[s0 : s0 + step] = sc
    return out, scale


def max_errors(got, exact, scale):
    """(max |got - exact| / |exact|, max |got - exact| / max(|exact|, scale)) over the
    positions where both are finite; the second divides by the statistic's natural
    magnitude where the statistic itself is near zero (1 for a correlation, the mean
    square for a variance, the root mean square for a standard deviation)."""
    import torch

    fin = torch.isfinite(got) & torch.isfinite(exact)
    if not bool(fin.any()):
        return None, None
    diff = (got[fin] - exact[fin]).abs()
    rel = diff / exact[fin].abs().clamp_min(1e-300)
    scaled = diff / torch.maximum(exact[fin].abs(), scale[fin]).clamp_min(1e-300)
    return float(rel.max()), float(scaled.max())


# ---- the ragged batched mix ---------------------------------------------------------------


RAGGED_SLICE_ELEMS = 2_500_000_000  # elements per streamed slice of series (outputs sized for one slice)


def measure_ragged(nb, device, nseries, steps, warmup, slice_elems=RAGGED_SLICE_ELEMS):
    """Series with lengths log-uniform in [16, 10^6] (seeded), N(0,1) with 3% NaN, int32
    labels uniform in [0, 64), flat float64 buffer plus int64 offsets; every series runs
    move_mean(window=20), move_exp_nanstd(alpha=0.05) and group_nanmean(64 labels).
    The batch is resident in HBM; it is cut into slices of consecutive series of at most
    `slice_elems` elements, each slice one captured CUDA graph (RaggedMix, chunk length
    autotuned) writing into one pair of output buffers sized for the largest slice, so
    the 100,000-series batch (about 9e9 values, 108 GB of inputs) streams through about
    40 GB of outputs.  A step replays every slice's graph; plain float64 and fp32c."""
    import numpy as np
    import torch

    from numbagg_gb300 import _lib

    rng = np.random.default_rng(5)
    lens = np.round(np.exp(rng.uniform(np.log(16), np.log(1e6), size=nseries))).astype(np.int64)
    offsets_np = np.concatenate([[0], np.cumsum(lens)])
    total = int(offsets_np[-1])
    g = torch.Generator(device=device)
    g.manual_seed(5)
    values = torch.empty(total, dtype=torch.float64, device=device)
    labels = torch.empty(total, dtype=torch.int32, device=device)
    piece = 1 << 28
    for p0 in range(0, total, piece):  # generated in pieces to bound the temporaries
        p1 = min(total, p0 + piece)
        v = torch.randn(p1 - p0, generator=g, dtype=torch.float64, device=device)
        v[torch.rand(p1 - p0, generator=g, device=device) < 0.03] = float("nan")
        values[p0:p1] = v
        labels[p0:p1] = torch.randint(0, 64, (p1 - p0,), generator=g, dtype=torch.int32, device=device)
        del v
    offsets = torch.from_numpy(offsets_np).to(device)
    # slices of consecutive series
    bounds, s0 = [], 0
    while s0 < nseries:
        s1 = s0 + 1
        while s1 < nseries and offsets_np[s1 + 1] - offsets_np[s0] <= slice_elems:
            s1 += 1
        bounds.append((s0, s1))
        s0 = s1
    longest = max(int(offsets_np[b] - offsets_np[a]) for a, b in bounds)
    mean_buf = torch.empty(longest, dtype=torch.float64, device=device)
    std_buf = torch.empty(longest, dtype=torch.float64, device=device)
    stream = torch.cuda.current_stream(device)
    res = {}
    launches0 = _lib.launch_count()
    for precision in ("f64", "fp32c"):
        mixes = []
        for a, b in bounds:
            e0, e1 = int(offsets_np[a]), int(offsets_np[b])
            mixes.append(
                nb.ragged.RaggedMix(values[e0:e1], labels[e0:e1], offsets[a : b + 1] - offsets[a], window=20,
                                    alpha=0.05, num_labels=64, precision=precision,
                                    outs=[mean_buf[: e1 - e0], std_buf[: e1 - e0], None])
            )
        for _ in range(warmup):
            for mix in mixes:
                mix.run()
        torch.cuda.synchronize(device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            for mix in mixes:
                mix.run()
        e1.record(stream)
        torch.cuda.synchronize(device)
        ms = e0.elapsed_time(e1) / steps
        res[precision] = {
            "ms_per_mix": round(ms, 3),
            "elements_per_s": round(total / (ms / 1e3), 1),
            "GB/s": round((8 + 4 + 8 + 8) * total / (ms / 1e3) / 1e9, 1),
            "chunk_len": sorted({m.chunk for m in mixes}),
            "graphs_per_step": len(mixes),
        }
        del mixes
    del values, labels, offsets, mean_buf, std_buf
    torch.cuda.empty_cache()
    config = {
        "series": nseries,
        "elements": total,
        "lengths": "round(exp(U(ln 16, ln 1e6))), seed 5",
        "values": "float64 N(0,1), 3% NaN; int32 labels U[0, 64)",
        "streaming": f"{len(bounds)} slices of consecutive series, at most {slice_elems} elements each, one "
        "captured graph per slice, outputs in one pair of buffers sized for the largest slice",
    }
    return res, config, int(_lib.launch_count() - launches0)


def run_ragged_suite(args):
    import torch

    import numbagg_gb300 as nb

    world, rank, local = dist_env()
    device = torch.device("cuda", local if world > 1 else torch.cuda.current_device())
    torch.cuda.set_device(device)
    res, config, launches = measure_ragged(nb, device, args.ragged_series, args.steps, args.warmup)
    line = {
        "suite": "ragged",
        "metric": "elements/s of the mix (move_mean w=20 + move_exp_nanstd a=0.05 + group_nanmean K=64 per series)",
        "config": config,
        "bytes_per_element": "8 read + 4 labels + 8 + 8 written (two scans); the group output is negligible",
        "results": res,
        "fp32c_speedup": round(res["f64"]["ms_per_mix"] / res["fp32c"]["ms_per_mix"], 2),
        "graph": "one CUDA graph per precision (RaggedMix), replayed per step",
        "gpu_launches": launches,
        "steps": args.steps,
        "warmup": args.warmup,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def run_aggregate_suite(args):
    """The static aggregations over the last axis of the headline's values: float64
    64 x cols, N(0,1) with 5% NaN; 8 algorithmic bytes per element (the reads)."""
    import torch

    import numbagg_gb300 as nb
    from numbagg_gb300 import _lib

    world, rank, local = dist_env()
    device = torch.device("cuda", local if world > 1 else torch.cuda.current_device())
    torch.cuda.set_device(device)
    g = torch.Generator(device=device)
    g.manual_seed(1)
    values = torch.randn((ROWS, args.cols), generator=g, dtype=torch.float64, device=device)
    values[torch.rand((ROWS, args.cols), generator=g, device=device) < NAN_P] = float("nan")
    calls = {
        "nansum": lambda: nb.nansum(values, axis=-1),
        "nanmean": lambda: nb.nanmean(values, axis=-1),
        "nanvar": lambda: nb.nanvar(values, axis=-1),
        "nancount": lambda: nb.nancount(values, axis=-1),
        "nanmax": lambda: nb.nanmax(values, axis=-1),
        "nanargmax": lambda: nb.nanargmax(values, axis=-1),
        "anynan": lambda: nb.anynan(values, axis=-1),
        "nansum_all_axes": lambda: nb.nansum(values),
        # the same buffer as (cols, 64) reduced over its first axis: in place through the
        # stride, no copy
        "nansum_axis0": lambda: nb.nansum(values.view(args.cols, ROWS), axis=0),
        "nanvar_axis0": lambda: nb.nanvar(values.view(args.cols, ROWS), axis=0),
    }
    peak, peak_kind = measured_peak()
    stream = torch.cuda.current_stream(device)
    nbytes = 8 * values.numel()
    res = {}
    launches0 = _lib.launch_count()
    for key, fn in calls.items():
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize(device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize(device)
        ms = e0.elapsed_time(e1) / args.steps
        gbs = nbytes / (ms / 1e3) / 1e9
        res[key] = {"ms": round(ms, 4), "GB/s": round(gbs, 1), "frac": round(gbs / peak, 4)}
    line = {
        "suite": "aggregate",
        "metric": "HBM GB/s of the static aggregations (8 bytes read per element)",
        "config": {"values": f"float64 {ROWS} x {args.cols}, N(0,1), {NAN_P:.0%} NaN",
                   "axis": "-1; *_axis0: the buffer viewed as cols x 64, axis 0"},
        "peak": peak,
        "peak_kind": peak_kind,
        "per_func": res,
        "note": "nanargmax synchronises once per call to check for all-NaN slices; nanvar is two passes",
        "gpu_launches": int(_lib.launch_count() - launches0),
        "steps": args.steps,
        "warmup": args.warmup,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def run_link_suite(args):
    """Pinned host <-> device copy bandwidth through the copy engines (4 GiB per copy):
    each direction alone, and both at once on two streams.  The end-to-end step moves
    its inputs in and its results out over this link."""
    import torch

    world, rank, local = dist_env()
    device = torch.device("cuda", local if world > 1 else torch.cuda.current_device())
    torch.cuda.set_device(device)
    n = 4 << 30
    h_a = torch.empty(n, dtype=torch.uint8, pin_memory=True)
    h_b = torch.empty(n, dtype=torch.uint8, pin_memory=True)
    h_a.fill_(1)
    h_b.fill_(2)
    d_a = torch.empty(n, dtype=torch.uint8, device=device)
    d_b = torch.empty(n, dtype=torch.uint8, device=device)
    d_a.fill_(3)
    s1, s2 = torch.cuda.Stream(device), torch.cuda.Stream(device)

    def timed(fn):
        best = None
        for _ in range(max(3, args.steps)):
            torch.cuda.synchronize(device)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s1)
            s2.wait_event(e0)
            fn()
            s1.wait_stream(s2)
            e1.record(s1)
            torch.cuda.synchronize(device)
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        return best

    def d2h():
        with torch.cuda.stream(s1):
            h_a.copy_(d_a, non_blocking=True)

    def h2d():
        with torch.cuda.stream(s1):
            d_b.copy_(h_b, non_blocking=True)

    def both():
        with torch.cuda.stream(s1):
            h_a.copy_(d_a, non_blocking=True)
        with torch.cuda.stream(s2):
            d_b.copy_(h_b, non_blocking=True)

    r_d2h, r_h2d, r_both = timed(d2h), timed(h2d), timed(both)
    line = {
        "suite": "link",
        "metric": "pinned host<->device copy GB/s (best of the repetitions)",
        "bytes_per_copy": n,
        "d2h_GB/s": round(n / (r_d2h / 1e3) / 1e9, 1),
        "h2d_GB/s": round(n / (r_h2d / 1e3) / 1e9, 1),
        "both_directions_total_GB/s": round(2 * n / (r_both / 1e3) / 1e9, 1),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def run_columns_suite(args):
    """Along axis 0 of float64 arrays (1 GiB, 5% NaN): each family through the public
    API, where the library chooses (`chosen`), forced in place through its column kernel
    (`in_place`), and with the axis moved last by a copy before the row kernel
    (`moved`).  The library's crossover between the two comes from this measurement."""
    import torch

    import numbagg_gb300 as nb
    from numbagg_gb300 import _host

    world, rank, local = dist_env()
    device = torch.device("cuda", local if world > 1 else torch.cuda.current_device())
    torch.cuda.set_device(device)
    stream = torch.cuda.current_stream(device)

    def timed(fn):
        for _ in range(max(1, args.warmup)):
            fn()
        torch.cuda.synchronize(device)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize(device)
        return round(e0.elapsed_time(e1) / args.steps, 3)

    res = {}
    for shape in ((16384, 8192), (2048, 65536)):
        g = torch.Generator(device=device)
        g.manual_seed(0)
        x = torch.randn(shape, generator=g, dtype=torch.float64, device=device)
        x[torch.rand(shape, generator=g, device=device) < NAN_P] = float("nan")
        lab = torch.randint(0, 12, (shape[0],), generator=g, device=device, dtype=torch.int32)
        families = {
            "ffill": lambda v, ax: nb.ffill(v, axis=ax),
            "move_mean_w20": lambda v, ax: nb.move_mean(v, window=20, axis=ax),
            "move_exp_nanmean_a0.1": lambda v, ax: nb.move_exp_nanmean(v, alpha=0.1, axis=ax),
            "group_nansum_K12": lambda v, ax: nb.group_nansum(v, lab, axis=ax, num_labels=12),
            "group_nanargmax_K12": lambda v, ax: nb.group_nanargmax(v, lab, axis=ax, num_labels=12),
        }
        for name, f in families.items():
            chosen = timed(lambda: f(x, 0))
            saved = _host.COLUMN_MIN_ROW_BYTES
            _host.COLUMN_MIN_ROW_BYTES = 0  # the column kernel whatever the width
            try:
                in_place = timed(lambda: f(x, 0))
            finally:
                _host.COLUMN_MIN_ROW_BYTES = saved
            moved = timed(lambda: f(x.T.contiguous(), -1))
            res[f"{name} {shape[0]}x{shape[1]}"] = {"chosen_ms": chosen, "in_place_ms": in_place, "moved_ms": moved}
        del x
        torch.cuda.empty_cache()
    line = {
        "suite": "columns",
        "metric": "ms per call along axis 0: the library's choice, the in-place column kernel, the copy + row kernel",
        "config": {"values": f"float64, N(0,1), {NAN_P:.0%} NaN, 1 GiB per array", "labels": "int32 U[0, 12) along axis 0",
                   "crossover": f"in place from {_host.COLUMN_MIN_ROW_BYTES} bytes of columns per position"},
        "per_call": res,
        "steps": args.steps,
        "warmup": args.warmup,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main(argv=None):
    args = parse_args(argv)
    if args.impl == "reference":
        return run_reference(args)
    if args.suite == "scan":
        return run_scan_suite(args)
    if args.suite == "ragged":
        return run_ragged_suite(args)
    if args.suite == "link":
        return run_link_suite(args)
    if args.suite == "aggregate":
        return run_aggregate_suite(args)
    if args.suite == "columns":
        return run_columns_suite(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
