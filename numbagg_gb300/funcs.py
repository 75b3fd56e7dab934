"""ffill / bfill (numbagg/funcs.py:294-326), on CUDA.

Same keywords and checks as numbagg's ``ndfill`` decorator
(numbagg/decorators.py:465-487): ``limit=None`` means the length of the axis, a
negative limit raises ValueError, a non-numeric dtype raises TypeError.  The output
has the input's dtype.  float64/float32/int32/int64 run natively; float16 is filled
in float32 and other integer widths as int64 (selection only, so exact).
"""

from __future__ import annotations

import numpy as np
import torch

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
    flat, shape = _host.rows_last(a.to(work), axis)
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


__all__ = ["bfill", "ffill"]
