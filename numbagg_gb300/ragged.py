"""Ragged batches: many series of uneven length in one call (an extension; numbagg
applies its functions array by array).

A batch is a flat float64 CUDA tensor ``values`` holding the series back to back and
an int64 tensor ``offsets`` of ``nseries + 1`` entries: series ``s`` is
``values[offsets[s]:offsets[s + 1]]``.  Each function computes exactly what the
numbagg function of the same name computes on every series on its own:

* ``move_sum / move_mean / move_var / move_std(values, offsets, *, window,
  min_count=None)`` return a tensor laid out like ``values``;
* ``move_exp_nanmean / nanvar / nanstd(values, offsets, *, alpha, min_weight=0)``
  likewise (``alpha`` a scalar or one value per element);
* ``group_nansum / nanmean / nancount(values, labels, offsets, *, num_labels)`` take
  per-element labels laid out like ``values`` and return ``nseries x num_labels``.

Every scan also takes ``precision="fp32c"`` (the FP32-compensated forms).  The kernels
walk the series with one persistent grid; the work items are planned on the device,
so the calls contain no host round trip and can be captured in a CUDA graph.
``RaggedPlan`` captures any list of requests (function, window / alpha / num_labels)
over one batch as a single CUDA graph and replays it, each moving-window chunk length
chosen by ``autotune_chunk`` and cached per shape and GPU model; ``RaggedMix`` is the
plan of the benchmark's pipeline (moving mean, EWM standard deviation and a grouped
mean per series).
"""

from __future__ import annotations

import json
import math
import os
import threading

import torch

from . import _host, _lib

PRECISIONS = ("f64", "fp32c")


def _check_batch(values, offsets):
    if not (isinstance(values, torch.Tensor) and values.is_cuda and values.dtype == torch.float64 and values.ndim == 1):
        raise TypeError("values must be a 1-D float64 CUDA tensor")
    if not (isinstance(offsets, torch.Tensor) and offsets.is_cuda and offsets.dtype == torch.int64 and offsets.ndim == 1):
        raise TypeError("offsets must be a 1-D int64 CUDA tensor")
    if offsets.numel() < 1:
        raise ValueError("offsets needs nseries + 1 entries")
    return values.contiguous(), offsets.contiguous()


def check_offsets(values, offsets):
    """offsets[0] == 0, nondecreasing, offsets[-1] == values.numel() (one device
    round trip; RaggedMix checks once when it is built)."""
    values, offsets = _check_batch(values, offsets)
    ok = bool(((offsets[1:] >= offsets[:-1]).all() & (offsets[0] == 0) & (offsets[-1] == values.numel())).item())
    if not ok:
        raise ValueError("offsets must start at 0, not decrease, and end at values.numel()")


def _sfx(precision):
    if precision not in PRECISIONS:
        raise ValueError(f"precision must be one of {PRECISIONS}: {precision!r}")
    return "f64_fp32c" if precision == "fp32c" else "f64"


def _move(name, values, offsets, window, min_count, precision, chunk_len, out=None):
    values, offsets = _check_batch(values, offsets)
    window = _host.check_int("window", window)
    if window <= 0:
        raise ValueError(f"window not in valid range: {window}")
    min_count = window if min_count is None else _host.check_int("min_count", min_count)
    if min_count < 0:
        raise ValueError(f"min_count must be positive: {min_count}")
    nseries = offsets.numel() - 1
    out = torch.empty_like(values) if out is None else out
    if nseries and values.numel():
        L = _lib.lib()
        ws = _lib.workspaces.scratch(L.nbg_move_ragged_workspace_bytes(nseries, values.numel()), values.device)
        fn = getattr(L, f"nbg_{name}_ragged_{_sfx(precision)}")
        _lib.check(
            fn(values.data_ptr(), offsets.data_ptr(), nseries, out.data_ptr(), window, min_count, int(chunk_len or 0),
               ws.data_ptr(), ws.numel(), _host.stream(values.device)),
            f"ragged {name}",
        )
    return out


def move_sum(values, offsets, *, window, min_count=None, precision="f64", chunk_len=None):
    return _move("move_sum", values, offsets, window, min_count, precision, chunk_len)


def move_mean(values, offsets, *, window, min_count=None, precision="f64", chunk_len=None):
    return _move("move_mean", values, offsets, window, min_count, precision, chunk_len)


def move_var(values, offsets, *, window, min_count=None, precision="f64", chunk_len=None):
    return _move("move_var", values, offsets, window, min_count, precision, chunk_len)


def move_std(values, offsets, *, window, min_count=None, precision="f64", chunk_len=None):
    return _move("move_std", values, offsets, window, min_count, precision, chunk_len)


def _move_exp(name, values, offsets, alpha, min_weight, precision, out=None):
    values, offsets = _check_batch(values, offsets)
    nseries = offsets.numel() - 1
    total = values.numel()
    if isinstance(alpha, torch.Tensor) and alpha.ndim > 0:
        if alpha.shape != values.shape:
            raise ValueError("alpha must be a scalar or laid out like values")
        alpha_t, alpha_mode, alpha_s = alpha.to(values.device, torch.float64).contiguous(), 2, 0.0
    else:
        alpha_t, alpha_mode, alpha_s = None, 0, float(alpha)
    out = torch.empty_like(values) if out is None else out
    if nseries and total:
        L = _lib.lib()
        ws = _lib.workspaces.scratch(L.nbg_move_exp_ragged_workspace_bytes(nseries, total), values.device)
        fn = getattr(L, f"nbg_{name}_ragged_{_sfx(precision)}")
        _lib.check(
            fn(values.data_ptr(), offsets.data_ptr(), nseries, total, _lib.ptr(alpha_t), alpha_s, alpha_mode,
               float(min_weight), out.data_ptr(), ws.data_ptr(), ws.numel(), _host.stream(values.device)),
            f"ragged {name}",
        )
    return out


def move_exp_nanmean(values, offsets, *, alpha, min_weight=0, precision="f64"):
    return _move_exp("move_exp_nanmean", values, offsets, alpha, min_weight, precision)


def move_exp_nanvar(values, offsets, *, alpha, min_weight=0, precision="f64"):
    return _move_exp("move_exp_nanvar", values, offsets, alpha, min_weight, precision)


def move_exp_nanstd(values, offsets, *, alpha, min_weight=0, precision="f64"):
    return _move_exp("move_exp_nanstd", values, offsets, alpha, min_weight, precision)


def _group(name, values, labels, offsets, num_labels, out=None):
    values, offsets = _check_batch(values, offsets)
    if not (isinstance(labels, torch.Tensor) and labels.shape == values.shape and not labels.dtype.is_floating_point):
        raise TypeError("labels must be an integer tensor laid out like values")
    num_labels = _host.check_int("num_labels", num_labels)
    if num_labels < 0:
        raise ValueError(f"num_labels must be non-negative: {num_labels}")
    nseries = offsets.numel() - 1
    lab = labels.to(values.device, torch.int64 if labels.dtype == torch.int64 else torch.int32).contiguous()
    out = torch.empty((nseries, num_labels), dtype=torch.float64, device=values.device) if out is None else out
    if nseries and num_labels:
        L = _lib.lib()
        ws = _lib.workspaces.scratch(L.nbg_group_ragged_workspace_bytes(nseries, values.numel(), num_labels), values.device)
        ls = "i64" if lab.dtype == torch.int64 else "i32"
        fn = getattr(L, f"nbg_group_{name}_ragged_f64_{ls}")
        _lib.check(
            fn(values.data_ptr(), lab.data_ptr(), offsets.data_ptr(), nseries, values.numel(), num_labels,
               out.data_ptr(), ws.data_ptr(), ws.numel(), _host.stream(values.device)),
            f"ragged group_{name}",
        )
    return out


def group_nansum(values, labels, offsets, *, num_labels):
    return _group("nansum", values, labels, offsets, num_labels)


def group_nanmean(values, labels, offsets, *, num_labels):
    return _group("nanmean", values, labels, offsets, num_labels)


def group_nancount(values, labels, offsets, *, num_labels):
    return _group("nancount", values, labels, offsets, num_labels)


# ---- autotuning ----------------------------------------------------------------------

_CANDIDATE_CHUNKS = (8192, 32768, 131072)
_cache: dict[str, int] = {}
_cache_lock = threading.Lock()
_CACHE_FILE = os.environ.get("NUMBAGG_GB300_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "numbagg_gb300_tune.json"))


def device_key(device) -> str:
    """The GPU a tuned choice belongs to: its name, SM count and compute capability."""
    p = torch.cuda.get_device_properties(device)
    return f"{p.name}|sm{p.multi_processor_count}|cc{p.major}{p.minor}".replace(" ", "_")


def _shape_key(op, precision, nseries, total, window, dev="any"):
    # shapes in the same power-of-two buckets share a choice, per GPU model
    return f"{dev}|{op}|{precision}|s{int(math.log2(max(nseries, 1)))}|n{int(math.log2(max(total, 1)))}|w{window}"


def _read_cache_file() -> dict[str, int]:
    try:
        with open(_CACHE_FILE) as fh:
            data = json.load(fh)
        if isinstance(data, dict):
            return {str(k): int(v) for k, v in data.items()}
    except (OSError, ValueError, TypeError):
        pass
    return {}


def _load_cache():
    _cache.update(_read_cache_file())


def _save_cache():
    """Merge this process's choices into the file and replace it atomically (a temporary
    file in the same directory, then os.replace), so concurrent processes never read a
    half-written cache."""
    try:
        d = os.path.dirname(_CACHE_FILE) or "."
        os.makedirs(d, exist_ok=True)
        merged = _read_cache_file()
        merged.update(_cache)
        tmp = f"{_CACHE_FILE}.{os.getpid()}.{threading.get_ident()}.tmp"
        with open(tmp, "w") as fh:
            json.dump(merged, fh, indent=1, sort_keys=True)
        os.replace(tmp, _CACHE_FILE)
    except OSError:
        pass


def autotune_chunk(op, values, offsets, *, window, precision="f64", reps=3):
    """Chunk length (positions per work item) of the ragged moving-window kernel for this
    shape on this GPU: each candidate is timed with CUDA events on the real batch, the
    fastest is kept in a process-wide cache (also merged into a JSON file,
    NUMBAGG_GB300_TUNE_CACHE or ~/.cache/numbagg_gb300_tune.json, keyed by the GPU
    model, and read back by later processes)."""
    key = _shape_key(op, precision, offsets.numel() - 1, values.numel(), window, device_key(values.device))
    with _cache_lock:
        if not _cache:
            _load_cache()
        if key in _cache:
            return _cache[key]
    out = torch.empty_like(values)
    best, best_ms = _CANDIDATE_CHUNKS[0], float("inf")
    stream = torch.cuda.current_stream(values.device)
    for c in _CANDIDATE_CHUNKS:
        _move(op, values, offsets, window, None, precision, c, out)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            _move(op, values, offsets, window, None, precision, c, out)
        e1.record(stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1) / reps
        if ms < best_ms:
            best, best_ms = c, ms
    with _cache_lock:
        _cache[key] = best
        _save_cache()
    return best


# ---- one graph over many requests ----------------------------------------------------

MOVE_OPS = ("move_sum", "move_mean", "move_var", "move_std")
EXP_OPS = ("move_exp_nanmean", "move_exp_nanvar", "move_exp_nanstd")
GROUP_OPS = ("group_nansum", "group_nanmean", "group_nancount")


def check_request(name, params):
    """(name, parameters) of one request; raises for unknown functions or keywords."""
    allowed = {
        **{op: {"window", "min_count"} for op in MOVE_OPS},
        **{op: {"alpha", "min_weight"} for op in EXP_OPS},
        **{op: {"num_labels"} for op in GROUP_OPS},
    }
    if name not in allowed:
        raise ValueError(f"unknown ragged function {name!r}; one of {sorted(allowed)}")
    extra = set(params) - allowed[name]
    if extra:
        raise TypeError(f"{name} got unexpected keywords {sorted(extra)}")
    needed = {"window"} if name in MOVE_OPS else ({"alpha"} if name in EXP_OPS else {"num_labels"})
    missing = needed - set(params)
    if missing:
        raise TypeError(f"{name} needs {sorted(missing)}")
    return name, dict(params)


class RaggedPlan:
    """Many requests -- any mix of the moving-window, exponentially weighted and grouped
    functions above, each with its own window / alpha / num_labels -- over one ragged
    batch, captured once as a single CUDA graph and replayed by ``run()``.

    ``requests`` is a list of ``(name, params)``, e.g. ``[("move_mean", {"window": 20}),
    ("move_exp_nanstd", {"alpha": 0.05}), ("group_nanmean", {"num_labels": 64})]``.
    Every moving-window request's chunk length is autotuned for this shape on this GPU
    (``tune=False``: the kernels' default).  Inputs are read from the tensors given here
    (refill them in place between runs).  ``outs`` may hold a preallocated output per
    request (None: allocate), so that plans over successive slices of a larger batch
    can share output buffers; ``run()`` returns the outputs in request order."""

    def __init__(self, values, offsets, requests, *, labels=None, precision="f64", tune=True, outs=None):
        check_offsets(values, offsets)
        _sfx(precision)
        self.values, self.offsets, self.labels, self.precision = values, offsets, labels, precision
        self.requests = [check_request(n, p) for n, p in requests]
        if any(n in GROUP_OPS for n, _ in self.requests) and labels is None:
            raise TypeError("grouped requests need labels laid out like values")
        dev = values.device
        nseries = offsets.numel() - 1
        outs = list(outs) if outs is not None else [None] * len(self.requests)
        if len(outs) != len(self.requests):
            raise ValueError("outs needs one entry per request")
        self.chunks, self.outs = [], []
        for (name, p), o in zip(self.requests, outs):
            if name in MOVE_OPS:
                c = autotune_chunk(name, values, offsets, window=p["window"], precision=precision) if tune else 0
                o = torch.empty_like(values) if o is None else o
            elif name in EXP_OPS:
                c = 0
                o = torch.empty_like(values) if o is None else o
            else:
                c = 0
                shape = (nseries, p["num_labels"])
                o = torch.empty(shape, dtype=torch.float64, device=dev) if o is None else o
            want = values.shape if name not in GROUP_OPS else (nseries, p["num_labels"])
            if tuple(o.shape) != tuple(want) or o.dtype != torch.float64 or o.device != dev:
                raise ValueError(f"output for {name} must be float64 {tuple(want)} on {dev}")
            self.chunks.append(c)
            self.outs.append(o)
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            self._body()  # allocates the scratch of this stream before capture
        torch.cuda.current_stream(dev).wait_stream(side)
        torch.cuda.synchronize(dev)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph, stream=side):
            self._body()

    def _body(self):
        for (name, p), c, o in zip(self.requests, self.chunks, self.outs):
            if name in MOVE_OPS:
                _move(name, self.values, self.offsets, p["window"], p.get("min_count"), self.precision, c, o)
            elif name in EXP_OPS:
                _move_exp(name, self.values, self.offsets, p["alpha"], p.get("min_weight", 0), self.precision, o)
            else:
                _group(name[len("group_"):], self.values, self.labels, self.offsets, p["num_labels"], o)

    def run(self):
        self.graph.replay()
        return self.outs


class RaggedMix(RaggedPlan):
    """The benchmark's pipeline as a RaggedPlan: move_mean(window), move_exp_nanstd(alpha)
    and group_nanmean(num_labels) of every series.  ``run()`` returns (mean, std,
    groups)."""

    def __init__(self, values, labels, offsets, *, window=20, alpha=0.05, num_labels=64, precision="f64",
                 tune=True, outs=None):
        super().__init__(
            values,
            offsets,
            [("move_mean", {"window": window}), ("move_exp_nanstd", {"alpha": alpha}),
             ("group_nanmean", {"num_labels": num_labels})],
            labels=labels,
            precision=precision,
            tune=tune,
            outs=outs,
        )
        self.window, self.alpha, self.num_labels = window, alpha, num_labels
        self.chunk = self.chunks[0]
        self.mean, self.std, self.groups = self.outs

    def run(self):
        self.graph.replay()
        return self.mean, self.std, self.groups


__all__ = [
    "RaggedMix",
    "RaggedPlan",
    "autotune_chunk",
    "check_offsets",
    "check_request",
    "device_key",
    "group_nancount",
    "group_nanmean",
    "group_nansum",
    "move_exp_nanmean",
    "move_exp_nanstd",
    "move_exp_nanvar",
    "move_mean",
    "move_std",
    "move_sum",
    "move_var",
]
