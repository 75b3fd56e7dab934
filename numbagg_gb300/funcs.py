"""ffill / bfill (numbagg/funcs.py:294-326) and the static pairwise-complete
matrices nancorrmatrix / nancovmatrix (numbagg/funcs.py:338-532), on CUDA.

Same keywords and checks as numbagg's ``ndfill`` decorator
(numbagg/decorators.py:465-487): ``limit=None`` means the length of the axis, a
negative limit raises ValueError, a non-numeric dtype raises TypeError.  The output
has the input's dtype.  float64/float32/int32/int64 run natively; float16 is filled
in float32 and other integer widths as int64 (selection only, so exact).
"""

from __future__ import annotations

import numpy as np
import torch

import math

from . import _host, _lib

_NUMERIC = (
    torch.float64,
    torch.float32,
    torch.float16,
    torch.bfloat16,
    torch.int64,
    torch.int32,
    torch.int16,
    torch.int8,
    torch.uint8,
)


def _fill(name: str, arr, limit, axis):
    if _host.is_tensor(arr):
        if arr.dtype not in _NUMERIC:
            raise TypeError(f"Unsupported dtype for fill operation: {arr.dtype}")
    else:
        arr = np.asarray(arr)
        if not np.issubdtype(arr.dtype, np.number):
            raise TypeError(f"Unsupported dtype for fill operation: {arr.dtype}")
    shape0 = _host.shape_of(arr)
    if len(shape0) == 0:
        raise ValueError(f"{name} requires an array with at least one dimension")
    axis = _host.normalize_axis(axis, len(shape0))
    if limit is None:
        limit = shape0[axis]
    if limit < 0:
        raise ValueError(f"`limit` must be positive: {limit}")
    limit = _host.check_int("limit", limit)
    a, restore = _host.to_device(arr)
    orig = a.dtype
    if orig in (torch.float16, torch.bfloat16):
        work = torch.float32
    elif orig in (torch.int16, torch.int8, torch.uint8):
        work = torch.int64
    else:
        work = orig
    aw = a.to(work)
    cols = _host.column_layout(aw, axis)
    if cols is not None:  # a non-last axis of a contiguous array: filled in place, no copy
        outer, n, inner = cols
        out = torch.empty_like(aw)
        if out.numel():
            fn = getattr(_lib.lib(), f"nbg_{name}_cols_{_host.ALL_SFX[work]}")
            _lib.check(fn(aw.data_ptr(), out.data_ptr(), outer, n, inner, limit, _host.stream(a.device)), name)
        return restore(out.to(orig) if work != orig else out)
    flat, shape = _host.rows_last(aw, axis)
    rows, n = flat.shape
    out = torch.empty((rows, n), dtype=work, device=a.device)
    if out.numel():
        L = _lib.lib()
        sfx = _host.ALL_SFX[work]
        if work.is_floating_point:
            ws = _lib.workspaces.scan(L.nbg_fill_workspace_bytes(rows, n), a.device)
            wp, wn = ws.data_ptr(), ws.numel()
        else:
            wp, wn = None, 0
        fn = getattr(L, f"nbg_{name}_{sfx}")
        _lib.check(fn(flat.data_ptr(), out.data_ptr(), rows, n, limit, wp, wn, _host.stream(a.device)), name)
    res = _host.restore_axis(out, shape, axis)
    if work != orig:
        res = res.to(orig)
    return restore(res)


def ffill(arr, *, limit=None, axis=-1):
    """Forward fill missing values, at most `limit` positions (numbagg/funcs.py:313-326)."""
    return _fill("ffill", arr, limit, axis)


def bfill(arr, *, limit=None, axis=-1):
    """Backward fill missing values, at most `limit` positions (numbagg/funcs.py:294-311)."""
    return _fill("bfill", arr, limit, axis)


def _static_matrix(name: str, a):
    """ndmatrix.__call__ (numbagg/decorators.py:700-717): (..., vars, obs) ->
    (..., vars, vars); float32 input keeps the float32 loop, everything else that
    casts safely runs the float64 one."""
    shape = _host.shape_of(a)
    if len(shape) < 2:
        raise ValueError(
            f"{name} requires at least a 2D array with shape (..., vars, obs). "
            "For 1D arrays, use nanvar for variance calculations."
        )
    from .moving_exp import loop_dtype

    t, restore = _host.to_device(a)
    dtype = loop_dtype([t], np.float32(0), 0.0)
    n_vars, n_obs = t.shape[-2:]
    lead = tuple(t.shape[:-2])
    batch = math.prod(lead)
    flat = t.to(dtype).contiguous().reshape(batch, n_vars, n_obs)
    out = torch.empty((batch, n_vars, n_vars), dtype=dtype, device=t.device)
    if out.numel():
        L = _lib.lib()
        corr = 1 if name == "nancorrmatrix" else 0
        f64 = 1 if dtype == torch.float64 else 0
        fn = getattr(L, f"nbg_{name}_{_host.FLOAT_SFX[dtype]}")
        for b0 in range(0, batch, 65535):
            b1 = min(batch, b0 + 65535)
            ws = _lib.workspaces.scratch(L.nbg_pair_matrix_workspace_bytes(corr, f64, b1 - b0, n_vars, n_obs), t.device)
            _lib.check(
                fn(flat[b0:b1].data_ptr(), out[b0:b1].data_ptr(), b1 - b0, n_vars, n_obs, ws.data_ptr(), ws.numel(),
                   _host.stream(t.device)),
                name,
            )
    return restore(out.reshape(lead + (n_vars, n_vars)))


def nancorrmatrix(a, **kwargs):
    """Pairwise-complete correlation matrix of the variables (axis -2) over the
    observations (axis -1), NaN as missing (numbagg/funcs.py:338-451)."""
    if kwargs:
        raise TypeError(f"unexpected keyword arguments: {sorted(kwargs)}")
    return _static_matrix("nancorrmatrix", a)


def nancovmatrix(a, **kwargs):
    """Pairwise-complete covariance matrix of the variables (axis -2) over the
    observations (axis -1), NaN as missing (numbagg/funcs.py:454-532)."""
    if kwargs:
        raise TypeError(f"unexpected keyword arguments: {sorted(kwargs)}")
    return _static_matrix("nancovmatrix", a)


__all__ = ["bfill", "ffill", "nancorrmatrix", "nancovmatrix"]
