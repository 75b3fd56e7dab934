"""Moving-window functions (numbagg/moving.py), on CUDA.

Same names, keywords and checks as numbagg's ``ndmove`` decorator
(numbagg/decorators.py:305-341):

* ``min_count=None`` means ``window``; a negative ``min_count`` raises ValueError;
* ``axis`` may be an int or a 1-tuple; ``axis=()`` returns the input unchanged (a
  ValueError with two arrays); more than one axis raises ValueError;
* ``0 < window <= shape[axis]`` else ValueError; a non-integer window raises
  TypeError (numba's int64 signature refuses it).

float32 and float64 arrays run natively; float16 computes in float32 and integer
arrays in float64, which is the gufunc loop numpy selects for them.
"""

from __future__ import annotations

import torch

from . import _host, _lib


PRECISIONS = ("f64", "fp32c")


def _move(name: str, arrs, window, min_count, axis, precision="f64"):
    if precision not in PRECISIONS:
        raise ValueError(f"precision must be one of {PRECISIONS}: {precision!r}")
    if min_count is None:
        min_count = window
    elif min_count < 0:
        raise ValueError(f"min_count must be positive: {min_count}")
    if isinstance(axis, tuple):
        if axis == ():
            if len(arrs) > 1:
                raise ValueError(
                    "`axis` cannot be an empty tuple when passing more than one array; since we default to returning the input."
                )
            return arrs[0]
        if len(axis) > 1:
            raise ValueError(f"only one axis can be passed to {name}; got {axis}")
        (axis,) = axis
    shape0 = _host.shape_of(arrs[0])
    if len(shape0) == 0:
        raise ValueError(f"{name} requires an array with at least one dimension")
    axis = _host.normalize_axis(axis, len(shape0))
    if not 0 < window <= shape0[axis]:
        raise ValueError(f"window not in valid range: {window}")
    window = _host.check_int("window", window)
    min_count = _host.check_int("min_count", min_count)
    tensors = []
    restore = None
    for x in arrs:
        t, r = _host.to_device(x)
        tensors.append(t)
        restore = restore or r
    a = tensors[0]
    dtype = _host.float_compute_dtype(a.dtype)
    if len(tensors) > 1:
        tensors = list(torch.broadcast_tensors(*tensors))
        dtype = _host.float_compute_dtype(torch.promote_types(tensors[0].dtype, tensors[1].dtype))
    tensors = [t.to(dtype) for t in tensors]
    if precision == "f64":
        cols_out = _move_columns(name, tensors, window, min_count, axis)
        if cols_out is not None:
            return restore(cols_out)
    flats = []
    shape = None
    for t in tensors:
        f, shape = _host.rows_last(t, axis)
        flats.append(f)
    rows, n = flats[0].shape
    out = torch.empty((rows, n), dtype=dtype, device=a.device)
    if out.numel():
        L = _lib.lib()
        ws = _lib.workspaces.scratch(L.nbg_move_workspace_bytes(rows, n), a.device)
        sfx = _host.FLOAT_SFX[dtype]
        if precision == "fp32c" and dtype == torch.float64:
            sfx += "_fp32c"
        fn = getattr(L, f"nbg_{name}_{sfx}")
        args = [f.data_ptr() for f in flats] + [
            out.data_ptr(),
            rows,
            n,
            window,
            min_count,
            ws.data_ptr(),
            ws.numel(),
            _host.stream(a.device),
        ]
        _lib.check(fn(*args), name)
    return restore(_host.restore_axis(out, shape, axis))


def _move_columns(name, tensors, window, min_count, axis):
    """A non-last axis of contiguous arrays: one thread per column runs numbagg's loop
    down it in place (no copy), bit for bit the reference's float64 arithmetic.  None
    when the layout does not apply."""
    cols = _host.column_layout(tensors[0], axis)
    if cols is None or any(t.shape != tensors[0].shape or not t.is_contiguous() for t in tensors):
        return None
    outer, n, inner = cols
    out = torch.empty_like(tensors[0])
    if out.numel():
        fn = getattr(_lib.lib(), f"nbg_{name}_cols_{_host.FLOAT_SFX[out.dtype]}")
        args = [t.data_ptr() for t in tensors] + [
            out.data_ptr(),
            outer,
            n,
            inner,
            window,
            min_count,
            _host.stream(out.device),
        ]
        _lib.check(fn(*args), name)
    return out


def move_sum(arr, /, *, window, min_count=None, axis=-1, precision="f64"):
    """Moving sum over the last `window` values, skipping NaN (numbagg/moving.py:58-99)."""
    return _move("move_sum", (arr,), window, min_count, axis, precision)


def move_mean(arr, /, *, window, min_count=None, axis=-1, precision="f64"):
    """Moving mean over the last `window` values, skipping NaN (numbagg/moving.py:12-55)."""
    return _move("move_mean", (arr,), window, min_count, axis, precision)


def move_std(arr, /, *, window, min_count=None, axis=-1, precision="f64"):
    """Moving sample standard deviation (ddof=1) (numbagg/moving.py:123-151)."""
    return _move("move_std", (arr,), window, min_count, axis, precision)


def move_var(arr, /, *, window, min_count=None, axis=-1, precision="f64"):
    """Moving sample variance (ddof=1) (numbagg/moving.py:154-181)."""
    return _move("move_var", (arr,), window, min_count, axis, precision)


def move_cov(a, b, /, *, window, min_count=None, axis=-1, precision="f64"):
    """Moving sample covariance of pairwise-complete values (numbagg/moving.py:184-220)."""
    return _move("move_cov", (a, b), window, min_count, axis, precision)


def move_corr(a, b, /, *, window, min_count=None, axis=-1, precision="f64"):
    """Moving correlation of pairwise-complete values (numbagg/moving.py:223-275)."""
    return _move("move_corr", (a, b), window, min_count, axis, precision)


__all__ = ["move_corr", "move_cov", "move_mean", "move_std", "move_sum", "move_var"]
