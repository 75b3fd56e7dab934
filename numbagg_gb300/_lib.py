"""Loader for ``libnbg_gb300.so`` and the host-side plumbing around its C ABI.

The library is found beside this file (built in-tree by ``numbagg_gb300._build``).
There is no fallback: if the library is missing or no CUDA device is present every
entry point raises.  Workspaces are torch device buffers kept per (device, stream):
scan workspaces are zero-filled once and then maintain themselves; grouped scratch
needs no initialisation.
"""

from __future__ import annotations

import ctypes
import os
import threading

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libnbg_gb300.so")

STATUS = {
    0: "ok",
    1: "invalid argument",
    2: "CUDA launch error",
    3: "workspace missing or too small",
    4: "look-back wait exceeded its bound",
    5: "unsupported shape or dtype",
    6: "problem larger than the fixed scratch of the allocation-free entry point",
}

_lib: ctypes.CDLL | None = None
_lock = threading.Lock()

c_ll = ctypes.c_longlong
c_vp = ctypes.c_void_p
c_sz = ctypes.c_size_t
c_d = ctypes.c_double
c_i = ctypes.c_int


UNSUPPORTED = 5


class NbgError(RuntimeError):
    """A CUDA-side failure reported by the C ABI."""


def _declare(lib: ctypes.CDLL) -> None:
    def sig(name, res, *args):
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = list(args)

    sig("nbg_version", c_i)
    sig("nbg_launch_count", ctypes.c_ulonglong)
    sig("nbg_set_deterministic", None, c_i)
    sig("nbg_get_deterministic", c_i)
    sig("nbg_status_string", ctypes.c_char_p, c_i)
    sig("nbg_workspace_header_bytes", c_sz)
    sig("nbg_workspace_error", c_i, c_vp, ctypes.POINTER(c_i), ctypes.POINTER(ctypes.c_uint), c_vp)
    sig("nbg_debug_lookback_timeout", c_i, c_vp, c_sz, c_i, c_vp)
    sig("nbg_move_workspace_bytes", c_sz, c_ll, c_ll)
    sig("nbg_move_exp_workspace_bytes", c_sz, c_ll, c_ll)
    sig("nbg_fill_workspace_bytes", c_sz, c_ll, c_ll)
    sig("nbg_ffill_noalloc_max_scratch_bytes", c_sz)
    sig("nbg_ffill_f64_noalloc", c_i, c_vp, c_vp, c_ll, c_ll, c_ll, c_vp)
    sig("nbg_ffill_noalloc_error", c_i, ctypes.POINTER(c_i), ctypes.POINTER(ctypes.c_uint), c_vp)
    sig("nbg_group_workspace_bytes", c_sz, c_i, c_ll, c_ll, c_ll)
    sig("nbg_move_exp_matrix_workspace_bytes", c_sz, c_i, c_i, c_ll, c_ll, c_ll)
    sig("nbg_pair_matrix_workspace_bytes", c_sz, c_i, c_i, c_ll, c_ll, c_ll)
    for dt in ("f64", "f32"):
        for f in ("move_sum", "move_mean", "move_var", "move_std"):
            sig(f"nbg_{f}_{dt}", c_i, c_vp, c_vp, c_ll, c_ll, c_ll, c_ll, c_vp, c_sz, c_vp)
        for f in ("move_cov", "move_corr"):
            sig(f"nbg_{f}_{dt}", c_i, c_vp, c_vp, c_vp, c_ll, c_ll, c_ll, c_ll, c_vp, c_sz, c_vp)
        for f in ("move_exp_nancount", "move_exp_nanmean", "move_exp_nansum", "move_exp_nanvar", "move_exp_nanstd"):
            sig(f"nbg_{f}_{dt}", c_i, c_vp, c_vp, c_d, c_i, c_d, c_vp, c_ll, c_ll, c_vp, c_sz, c_vp)
        for f in ("move_exp_nancov", "move_exp_nancorr"):
            sig(f"nbg_{f}_{dt}", c_i, c_vp, c_vp, c_vp, c_d, c_i, c_d, c_vp, c_ll, c_ll, c_vp, c_sz, c_vp)
        for f in ("move_covmatrix", "move_corrmatrix"):
            sig(f"nbg_{f}_{dt}", c_i, c_vp, c_vp, c_ll, c_ll, c_ll, c_ll, c_ll, c_vp)
        for f in ("move_exp_nancovmatrix", "move_exp_nancorrmatrix"):
            sig(f"nbg_{f}_{dt}", c_i, c_vp, c_vp, c_ll, c_d, c_vp, c_ll, c_ll, c_ll, c_vp, c_sz, c_vp)
        for f in ("nancovmatrix", "nancorrmatrix"):
            sig(f"nbg_{f}_{dt}", c_i, c_vp, c_vp, c_ll, c_ll, c_ll, c_vp, c_sz, c_vp)
    # FP32-compensated forms of the float64 scans
    for f in ("move_sum", "move_mean", "move_var", "move_std"):
        sig(f"nbg_{f}_f64_fp32c", c_i, c_vp, c_vp, c_ll, c_ll, c_ll, c_ll, c_vp, c_sz, c_vp)
    for f in ("move_cov", "move_corr"):
        sig(f"nbg_{f}_f64_fp32c", c_i, c_vp, c_vp, c_vp, c_ll, c_ll, c_ll, c_ll, c_vp, c_sz, c_vp)
    for f in ("move_exp_nancount", "move_exp_nanmean", "move_exp_nansum", "move_exp_nanvar", "move_exp_nanstd"):
        sig(f"nbg_{f}_f64_fp32c", c_i, c_vp, c_vp, c_d, c_i, c_d, c_vp, c_ll, c_ll, c_vp, c_sz, c_vp)
    for f in ("move_exp_nancov", "move_exp_nancorr"):
        sig(f"nbg_{f}_f64_fp32c", c_i, c_vp, c_vp, c_vp, c_d, c_i, c_d, c_vp, c_ll, c_ll, c_vp, c_sz, c_vp)
    # ragged batches
    sig("nbg_move_exp_ragged_workspace_bytes", c_sz, c_ll, c_ll)
    sig("nbg_move_ragged_workspace_bytes", c_sz, c_ll, c_ll)
    sig("nbg_group_ragged_workspace_bytes", c_sz, c_ll, c_ll, c_ll)
    for sfx in ("f64", "f64_fp32c"):
        for f in ("move_sum", "move_mean", "move_var", "move_std"):
            sig(f"nbg_{f}_ragged_{sfx}", c_i, c_vp, c_vp, c_ll, c_vp, c_ll, c_ll, c_ll, c_vp, c_sz, c_vp)
        for f in ("move_exp_nanmean", "move_exp_nanvar", "move_exp_nanstd"):
            sig(f"nbg_{f}_ragged_{sfx}", c_i, c_vp, c_vp, c_ll, c_ll, c_vp, c_d, c_i, c_d, c_vp, c_vp, c_sz, c_vp)
    for f in ("nansum", "nanmean", "nancount"):
        for ls in ("i32", "i64"):
            sig(f"nbg_group_{f}_ragged_f64_{ls}", c_i, c_vp, c_vp, c_vp, c_ll, c_ll, c_ll, c_vp, c_vp, c_sz, c_vp)
    # grouped reductions over non-last axes, in place
    sig("nbg_group_cols_max_labels", c_sz, c_i)
    for f in GROUP_FUNC_IDS:
        for vs in ("f64", "f32") if f in ("nanmean", "nanvar", "nanstd") else ("f64", "f32", "i32", "i64"):
            for ls in ("i32", "i64"):
                sig(f"nbg_group_{f}_cols_{vs}_{ls}", c_i, c_vp, c_vp, c_vp, c_ll, c_ll, c_ll, c_ll, c_ll, c_vp)
    for dt in ("f64", "f32", "i32", "i64"):
        for f in ("ffill", "bfill"):
            sig(f"nbg_{f}_{dt}", c_i, c_vp, c_vp, c_ll, c_ll, c_ll, c_vp, c_sz, c_vp)
            sig(f"nbg_{f}_cols_{dt}", c_i, c_vp, c_vp, c_ll, c_ll, c_ll, c_ll, c_vp)
    # moving windows along a non-last axis (one thread per column)
    for dt in ("f64", "f32"):
        for f in ("move_sum", "move_mean", "move_var", "move_std"):
            sig(f"nbg_{f}_cols_{dt}", c_i, c_vp, c_vp, c_ll, c_ll, c_ll, c_ll, c_ll, c_vp)
        for f in ("move_cov", "move_corr"):
            sig(f"nbg_{f}_cols_{dt}", c_i, c_vp, c_vp, c_vp, c_ll, c_ll, c_ll, c_ll, c_ll, c_vp)
    # the exponentially weighted family along a non-last axis (one thread per column)
    for sfx in ("f64", "f32", "f64_fp32c"):
        for f in ("move_exp_nancount", "move_exp_nanmean", "move_exp_nansum", "move_exp_nanvar", "move_exp_nanstd"):
            sig(f"nbg_{f}_cols_{sfx}", c_i, c_vp, c_vp, c_d, c_i, c_d, c_vp, c_ll, c_ll, c_ll, c_vp)
        for f in ("move_exp_nancov", "move_exp_nancorr"):
            sig(f"nbg_{f}_cols_{sfx}", c_i, c_vp, c_vp, c_vp, c_d, c_i, c_d, c_vp, c_ll, c_ll, c_ll, c_vp)
    # static aggregations over the last axis
    sig("nbg_aggregate_workspace_bytes", c_sz, c_ll, c_ll)
    for dt in ("f64", "f32", "i32", "i64"):
        for f in ("allnan", "anynan", "nancount", "nansum", "nanmax", "nanmin", "nanargmax", "nanargmin"):
            sig(f"nbg_{f}_{dt}", c_i, c_vp, c_vp, c_ll, c_ll, c_vp, c_sz, c_vp)
    for dt in ("f64", "f32"):
        sig(f"nbg_nanmean_{dt}", c_i, c_vp, c_vp, c_ll, c_ll, c_vp, c_sz, c_vp)
        for f in ("nanvar", "nanstd"):
            sig(f"nbg_{f}_{dt}", c_i, c_vp, c_vp, c_ll, c_ll, c_ll, c_vp, c_sz, c_vp)
    # the same over the middle axis of a contiguous (outer, m, inner) array
    sig("nbg_aggregate_cols_workspace_bytes", c_sz, c_ll, c_ll, c_ll)
    for dt in ("f64", "f32", "i32", "i64"):
        for f in ("allnan", "anynan", "nancount", "nansum", "nanmax", "nanmin", "nanargmax", "nanargmin"):
            sig(f"nbg_{f}_cols_{dt}", c_i, c_vp, c_vp, c_ll, c_ll, c_ll, c_vp, c_sz, c_vp)
    for dt in ("f64", "f32"):
        sig(f"nbg_nanmean_cols_{dt}", c_i, c_vp, c_vp, c_ll, c_ll, c_ll, c_vp, c_sz, c_vp)
        for f in ("nanvar", "nanstd"):
            sig(f"nbg_{f}_cols_{dt}", c_i, c_vp, c_vp, c_ll, c_ll, c_ll, c_ll, c_vp, c_sz, c_vp)
    for name in GROUP_FUNC_IDS:
        vdts = ("f64", "f32") if name in ("nanmean", "nanvar", "nanstd") else ("f64", "f32", "i32", "i64")
        for vd in vdts:
            for ld in ("i32", "i64"):
                sig(f"nbg_group_{name}_{vd}_{ld}", c_i, c_vp, c_vp, c_vp, c_ll, c_ll, c_ll, c_ll, c_vp, c_sz, c_vp)


GROUP_FUNC_IDS = {
    "nansum": 0,
    "nancount": 1,
    "nanmean": 2,
    "nanvar": 3,
    "nanstd": 4,
    "nansum_of_squares": 5,
    "nanargmax": 6,
    "nanargmin": 7,
    "nanmax": 8,
    "nanmin": 9,
    "nanfirst": 10,
    "nanlast": 11,
    "nanprod": 12,
    "nanany": 13,
    "nanall": 14,
}


def lib() -> ctypes.CDLL:
    """The loaded C library.  Raises if it is missing or no CUDA device is visible."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(
                    f"numbagg_gb300's CUDA library is not built ({LIB_PATH} missing); "
                    "run `python -c 'import numbagg_gb300._build as b; b.build()'`"
                )
            handle = ctypes.CDLL(LIB_PATH)
            _declare(handle)
            _lib = handle
    return _lib


def require_cuda() -> None:
    if not torch.cuda.is_available():
        raise RuntimeError("numbagg_gb300 runs on a CUDA GPU and none is available")


def check(status: int, what: str) -> None:
    if status != 0:
        raise NbgError(f"{what}: {STATUS.get(status, 'unknown status')} (status {status})")


def stream_handle(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


class _Workspaces:
    """Per-(device, stream) buffers.  A scan workspace is zeroed when allocated or
    grown and must not be shared across streams (its header counts launches)."""

    def __init__(self) -> None:
        self._scan: dict[tuple[int, int], torch.Tensor] = {}
        self._scratch: dict[tuple[int, int], torch.Tensor] = {}
        self._lock = threading.Lock()

    def scan(self, nbytes: int, device: torch.device) -> torch.Tensor:
        key = (device.index or 0, stream_handle(device))
        with self._lock:
            buf = self._scan.get(key)
            if buf is None or buf.numel() < nbytes:
                size = max(nbytes, 1 << 20)
                if buf is not None:
                    size = max(size, 2 * buf.numel())
                # the old buffer was used on this stream only, so the caching allocator
                # orders its reuse; no synchronisation (which stream capture forbids)
                buf = torch.zeros(size, dtype=torch.uint8, device=device)
                self._scan[key] = buf
            return buf

    def scratch(self, nbytes: int, device: torch.device) -> torch.Tensor:
        key = (device.index or 0, stream_handle(device))
        with self._lock:
            buf = self._scratch.get(key)
            if buf is None or buf.numel() < nbytes:
                size = max(nbytes, 1 << 20)
                if buf is not None:
                    size = max(size, 2 * buf.numel())
                buf = torch.empty(size, dtype=torch.uint8, device=device)
                self._scratch[key] = buf
            return buf

    def all_scan(self):
        return list(self._scan.values())


workspaces = _Workspaces()


def launch_count() -> int:
    """Kernels launched by the library so far in this process."""
    return int(lib().nbg_launch_count())


def workspace_error(ws: torch.Tensor) -> tuple[int, int]:
    """(code, tile) recorded on the device in a scan workspace; clears it."""
    code = c_i(0)
    tile = ctypes.c_uint(0)
    check(
        lib().nbg_workspace_error(ws.data_ptr(), ctypes.byref(code), ctypes.byref(tile), stream_handle(ws.device)),
        "nbg_workspace_error",
    )
    return code.value, tile.value
