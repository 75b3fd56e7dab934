"""Static aggregations over one or more axes (numbagg/funcs.py:23-242, :329), on CUDA.

The ndaggregate functions -- ``allnan``, ``anynan``, ``nancount`` (alias ``count``),
``nansum``, ``nanmean``, ``nanvar``, ``nanstd`` -- take ``axis=None`` (every axis), an
int or a tuple of ints, and ``ddof=1`` for nanvar / nanstd
(numbagg/decorators.py:231-255).  The ndreduce functions -- ``nanmax``, ``nanmin``,
``nanargmax``, ``nanargmin`` -- take the same ``axis`` (numbagg/decorators.py:1002-1028).
The reduced axes are moved last, in the order given, and flattened
(numbagg/utils.py:20-32), so ``nanargmax`` over several axes indexes that flattening.
A reduction over every axis returns a scalar: a numpy scalar for array input, a 0-d
tensor for tensor input.

Input dtypes select the reference's gufunc loop the way numpy does, the first loop the
input casts to safely: (int32, int64, float32, float64) for most functions, (float32,
float64) for nanmean / nanvar / nanstd.  Errors match the reference:
``nanmax``/``nanmin`` of an empty reduction raise "zero-size array to reduction
operation fmax/fmin which has no identity", ``nanargmax``/``nanargmin`` raise "All-NaN
slice encountered" for an empty or all-NaN slice.
"""

from __future__ import annotations

import math

import numpy as np
import torch

from . import _host, _lib

_INT_FLOAT_LOOPS = (np.int32, np.int64, np.float32, np.float64)
_FLOAT_LOOPS = (np.float32, np.float64)
_TORCH_TO_NP = {
    torch.float64: np.float64,
    torch.float32: np.float32,
    torch.float16: np.float16,
    torch.bfloat16: np.float32,  # no numpy bfloat16; it casts safely to float32 as well
    torch.int64: np.int64,
    torch.int32: np.int32,
    torch.int16: np.int16,
    torch.int8: np.int8,
    torch.uint8: np.uint8,
    torch.bool: np.bool_,
}
# the in-place path for middle axes wants whole warps of consecutive outputs
_MIN_INNER = 32
_NP_TO_TORCH = {np.float64: torch.float64, np.float32: torch.float32, np.int64: torch.int64, np.int32: torch.int32}


def _np_dtype(arr) -> np.dtype:
    if _host.is_tensor(arr):
        if arr.dtype not in _TORCH_TO_NP:
            raise TypeError(f"unsupported dtype {arr.dtype}")
        return np.dtype(_TORCH_TO_NP[arr.dtype])
    return np.asarray(arr).dtype


def _loop(name: str, dt: np.dtype, loops) -> type:
    """The first of the reference's loops that `dt` casts to safely (numpy's rule)."""
    for lp in loops:
        if np.can_cast(dt, lp, casting="safe"):
            return lp
    raise TypeError(f"ufunc '{name}' not supported for the input types {dt}")


def _axes(axis, ndim: int) -> tuple[int, ...]:
    if axis is None:
        return tuple(range(ndim))
    if not isinstance(axis, tuple):
        axis = (axis,)
    out = tuple(_host.normalize_axis(_host.check_int("axis", a), ndim) for a in axis)
    if len(set(out)) != len(out):
        raise ValueError("repeated axis in `source` argument")
    return out


def middle_inner(shape, axes) -> int | None:
    """The product of the trailing unreduced axes when the reduced axes are consecutive,
    in increasing order and not last, with at least _MIN_INNER outputs per reduced
    position: such axes are reduced in place through their stride (numbagg's gufuncs
    read them so), with no copy.  None otherwise."""
    if not axes:
        return None
    k0 = axes[0]
    if axes != tuple(range(k0, k0 + len(axes))) or axes[-1] >= len(shape) - 1:
        return None
    inner = math.prod(shape[axes[-1] + 1 :])
    return inner if inner >= _MIN_INNER else None


def _aggregate(name: str, arr, axis, *, ddof=None):
    dt = _np_dtype(arr)
    loops = _FLOAT_LOOPS if name in ("nanmean", "nanvar", "nanstd") else _INT_FLOAT_LOOPS
    loop = _loop(name, dt, loops)
    shape = _host.shape_of(arr)
    scalar_in = len(shape) == 0
    if scalar_in:
        shape = (1,)
    axes = _axes(axis, len(shape))
    keep = [d for d in range(len(shape)) if d not in axes]
    out_shape = tuple(shape[d] for d in keep)
    rows = math.prod(out_shape)
    m = math.prod(shape[d] for d in axes)
    if ddof is not None:
        ddof = _host.check_int("ddof", ddof)
    if rows > 0 and m == 0:
        if name in ("nanmax", "nanmin"):
            op = "fmax" if name == "nanmax" else "fmin"
            raise ValueError(f"zero-size array to reduction operation {op} which has no identity")
        if name in ("nanargmax", "nanargmin"):
            raise ValueError("All-NaN slice encountered")
    a, restore = _host.to_device(arr)
    if scalar_in:
        a = a.reshape(1)
    work = _NP_TO_TORCH[loop]
    if a.dtype != work:
        a = a.to(work)
    inner = middle_inner(shape, axes) if a.is_contiguous() else None
    middle = inner is not None
    flat = None
    if not middle:
        flat = torch.movedim(a, axes, tuple(range(len(shape) - len(axes), len(shape)))).contiguous().reshape(rows, m)
    if name in ("allnan", "anynan"):
        out_dt = torch.bool
    elif name in ("nancount", "nanargmax", "nanargmin"):
        out_dt = torch.int64
    else:
        out_dt = work
    out = torch.empty(rows, dtype=out_dt, device=a.device)
    if rows > 0:
        L = _lib.lib()
        if middle:
            outer = rows // inner
            ws = _lib.workspaces.scratch(L.nbg_aggregate_cols_workspace_bytes(outer, m, inner), a.device)
            fn = getattr(L, f"nbg_{name}_cols_{_host.ALL_SFX[work]}")
            args = [a.data_ptr() if m > 0 else None, out.data_ptr(), outer, m, inner]
        else:
            ws = _lib.workspaces.scratch(L.nbg_aggregate_workspace_bytes(rows, m), a.device)
            fn = getattr(L, f"nbg_{name}_{_host.ALL_SFX[work]}")
            args = [flat.data_ptr() if m > 0 else None, out.data_ptr(), rows, m]
        if ddof is not None:
            args.append(ddof)
        _lib.check(fn(*args, ws.data_ptr(), ws.numel(), _host.stream(a.device)), name)
        if name in ("nanargmax", "nanargmin") and bool((out < 0).any()):
            raise ValueError("All-NaN slice encountered")
    res = restore(out.reshape(out_shape))
    if len(out_shape) == 0 and isinstance(res, np.ndarray):
        return res[()]
    return res


def allnan(a, *, axis=None):
    """True where every element of the reduced axes is NaN (numbagg/funcs.py:23-36)."""
    return _aggregate("allnan", a, axis)


def anynan(a, *, axis=None):
    """True where any element of the reduced axes is NaN (numbagg/funcs.py:39-52)."""
    return _aggregate("anynan", a, axis)


def nancount(a, *, axis=None):
    """Number of non-NaN elements, int64 (numbagg/funcs.py:55-68)."""
    return _aggregate("nancount", a, axis)


count = nancount  # numbagg/funcs.py:329


def nansum(a, *, axis=None):
    """Sum ignoring NaN, in the input's loop dtype (numbagg/funcs.py:71-84)."""
    return _aggregate("nansum", a, axis)


def nanmean(a, *, axis=None):
    """Mean ignoring NaN; NaN where nothing is valid (numbagg/funcs.py:87-103)."""
    return _aggregate("nanmean", a, axis)


def nanvar(a, *, ddof=1, axis=None):
    """Variance ignoring NaN, two-pass (numbagg/funcs.py:106-133)."""
    return _aggregate("nanvar", a, axis, ddof=ddof)


def nanstd(a, *, ddof=1, axis=None):
    """Standard deviation ignoring NaN, two-pass (numbagg/funcs.py:136-159)."""
    return _aggregate("nanstd", a, axis, ddof=ddof)


def nanmax(a, *, axis=None):
    """Maximum ignoring NaN; NaN where every element is NaN (numbagg/funcs.py:202-221)."""
    return _aggregate("nanmax", a, axis)


def nanmin(a, *, axis=None):
    """Minimum ignoring NaN; NaN where every element is NaN (numbagg/funcs.py:224-242)."""
    return _aggregate("nanmin", a, axis)


def nanargmax(a, *, axis=None):
    """Index of the first maximum ignoring NaN (numbagg/funcs.py:162-180)."""
    return _aggregate("nanargmax", a, axis)


def nanargmin(a, *, axis=None):
    """Index of the first minimum ignoring NaN (numbagg/funcs.py:183-199)."""
    return _aggregate("nanargmin", a, axis)


__all__ = [
    "allnan",
    "anynan",
    "count",
    "nanargmax",
    "nanargmin",
    "nancount",
    "nanmax",
    "nanmean",
    "nanmin",
    "nanstd",
    "nansum",
    "nanvar",
]
