"""Exponentially weighted moving functions (numbagg/moving_exp.py), on CUDA.

Same names, keywords and checks as numbagg's ``ndmoveexp`` decorator
(numbagg/decorators.py:374-414): ``alpha`` is a scalar, a 1-D array along the
scanned axis, or an array shaped like the input; ``axis`` may be an int or a
1-tuple, ``axis=()`` returns the input.

The loop dtype follows numpy's resolution of the gufunc's two loops (float32,
float64) over the array operands: numbagg turns a scalar alpha into
``np.broadcast_to(alpha, n)``, a float64 array for a Python float, so float32 input
with a scalar alpha runs (and returns) float64; the float32 loop runs only when the
arrays and an alpha array all cast safely to float32.  alpha and min_weight are then
rounded to the loop dtype.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _host, _lib


PRECISIONS = ("f64", "fp32c")


def _operand_dtype(x) -> np.dtype:
    if isinstance(x, torch.Tensor):
        return np.dtype(str(x.dtype).replace("torch.", "")) if x.dtype != torch.bfloat16 else np.dtype(np.float32)
    return np.asarray(x).dtype


def loop_dtype(arrays, alpha, min_weight) -> torch.dtype:
    """float32 when every array operand (the inputs, alpha broadcast as numbagg does it,
    and min_weight when it is a numpy scalar) casts safely to float32, else float64:
    the first of the gufunc's loops (float32, float64) that numpy's type resolution
    accepts."""
    dts = [_operand_dtype(x) for x in arrays]
    dts.append(_operand_dtype(alpha))
    if isinstance(min_weight, np.generic):
        dts.append(min_weight.dtype)
    if all(np.can_cast(d, np.float32, casting="safe") for d in dts):
        return torch.float32
    return torch.float64


def _move_exp(name: str, arrs, alpha, min_weight, axis, precision="f64"):
    if precision not in PRECISIONS:
        raise ValueError(f"precision must be one of {PRECISIONS}: {precision!r}")
    if isinstance(axis, tuple):
        if axis == ():
            if len(arrs) > 1:
                raise ValueError(
                    "`axis` cannot be an empty tuple when passing more than one array; since we default to returning the input."
                )
            return arrs[0]
        if len(axis) > 1:
            raise ValueError(f"Only one axis can be passed to {name}; got {axis}")
        (axis,) = axis
    shape0 = _host.shape_of(arrs[0])
    if len(shape0) == 0:
        raise ValueError(f"{name} requires an array with at least one dimension")
    axis = _host.normalize_axis(axis, len(shape0))
    if isinstance(alpha, (np.ndarray, torch.Tensor)) and np.ndim(alpha) == 1 and len(alpha) != shape0[axis]:
        raise ValueError(f"alpha has length {len(alpha)}, expected {shape0[axis]} (the length of axis {axis})")
    tensors = []
    restore = None
    for x in arrs:
        t, r = _host.to_device(x)
        tensors.append(t)
        restore = restore or r
    a = tensors[0]
    dtype = loop_dtype(tensors, alpha, min_weight)
    if len(tensors) > 1:
        tensors = list(torch.broadcast_tensors(*tensors))
    np_dtype = np.float64 if dtype == torch.float64 else np.float32
    cols_out = _move_exp_columns(name, [t.to(dtype) for t in tensors], alpha, min_weight, axis, dtype, np_dtype,
                                 precision)
    if cols_out is not None:
        return restore(cols_out)
    flats = []
    shape = None
    for t in tensors:
        f, shape = _host.rows_last(t.to(dtype), axis)
        flats.append(f)
    rows, n = flats[0].shape

    alpha_t = None
    alpha_scalar = 0.0
    if isinstance(alpha, (np.ndarray, torch.Tensor)) and np.ndim(alpha) > 0:
        at, _ = _host.to_device(alpha)
        at = at.to(device=a.device, dtype=dtype)
        if at.ndim == 1:
            if at.shape[0] != n:
                raise ValueError(f"alpha has length {at.shape[0]}, expected {n} (the length of axis {axis})")
            alpha_t = at.contiguous()
            mode = 1
        else:
            at = torch.broadcast_to(at, tensors[0].shape)
            alpha_t, _ = _host.rows_last(at, axis)
            mode = 2
    else:
        alpha_scalar = float(np_dtype(np.asarray(alpha).item() if hasattr(alpha, "shape") else alpha))
        mode = 0
    mw = float(np_dtype(min_weight))

    out = torch.empty((rows, n), dtype=dtype, device=a.device)
    if out.numel():
        L = _lib.lib()
        ws = _lib.workspaces.scratch(L.nbg_move_exp_workspace_bytes(rows, n), a.device)
        sfx = _host.FLOAT_SFX[dtype]
        if precision == "fp32c" and dtype == torch.float64:
            sfx += "_fp32c"
        fn = getattr(L, f"nbg_{name}_{sfx}")
        args = [f.data_ptr() for f in flats] + [
            None if alpha_t is None else alpha_t.data_ptr(),
            alpha_scalar,
            mode,
            mw,
            out.data_ptr(),
            rows,
            n,
            ws.data_ptr(),
            ws.numel(),
            _host.stream(a.device),
        ]
        _lib.check(fn(*args), name)
    return restore(_host.restore_axis(out, shape, axis))


def _move_exp_columns(name, tensors, alpha, min_weight, axis, dtype, np_dtype, precision):
    """A non-last axis of contiguous arrays: one thread per column runs numbagg's loop
    down it in place (no copy).  None when the layout does not apply."""
    cols = _host.column_layout(tensors[0], axis)
    if cols is None or any(t.shape != tensors[0].shape or not t.is_contiguous() for t in tensors):
        return None
    outer, n, inner = cols
    alpha_t, alpha_scalar = None, 0.0
    if isinstance(alpha, (np.ndarray, torch.Tensor)) and np.ndim(alpha) > 0:
        at, _ = _host.to_device(alpha)
        at = at.to(device=tensors[0].device, dtype=dtype)
        if at.ndim == 1:
            if at.shape[0] != n:
                raise ValueError(f"alpha has length {at.shape[0]}, expected {n} (the length of axis {axis})")
            alpha_t, mode = at.contiguous(), 1
        elif tuple(at.shape) == tuple(tensors[0].shape):
            alpha_t, mode = at.contiguous(), 2
        else:
            return None  # a broadcast alpha: the rows path handles it
    else:
        alpha_scalar = float(np_dtype(np.asarray(alpha).item() if hasattr(alpha, "shape") else alpha))
        mode = 0
    out = torch.empty_like(tensors[0])
    if out.numel():
        sfx = _host.FLOAT_SFX[dtype]
        if precision == "fp32c" and dtype == torch.float64:
            sfx += "_fp32c"
        fn = getattr(_lib.lib(), f"nbg_{name}_cols_{sfx}")
        args = [t.data_ptr() for t in tensors] + [
            None if alpha_t is None else alpha_t.data_ptr(),
            alpha_scalar,
            mode,
            float(np_dtype(min_weight)),
            out.data_ptr(),
            outer,
            n,
            inner,
            _host.stream(tensors[0].device),
        ]
        _lib.check(fn(*args), name)
    return out


def move_exp_nancount(arr, /, *, alpha, min_weight=0, axis=-1, precision="f64"):
    """Exponentially decayed count of non-NaN values (numbagg/moving_exp.py:12-38)."""
    return _move_exp("move_exp_nancount", (arr,), alpha, min_weight, axis, precision)


def move_exp_nanmean(arr, /, *, alpha, min_weight=0, axis=-1, precision="f64"):
    """Exponentially weighted moving mean (numbagg/moving_exp.py:41-71)."""
    return _move_exp("move_exp_nanmean", (arr,), alpha, min_weight, axis, precision)


def move_exp_nansum(arr, /, *, alpha, min_weight=0, axis=-1, precision="f64"):
    """Exponentially weighted moving sum (numbagg/moving_exp.py:74-102)."""
    return _move_exp("move_exp_nansum", (arr,), alpha, min_weight, axis, precision)


def move_exp_nanvar(arr, /, *, alpha, min_weight=0, axis=-1, precision="f64"):
    """Exponentially weighted moving variance, bias-corrected (numbagg/moving_exp.py:105-156)."""
    return _move_exp("move_exp_nanvar", (arr,), alpha, min_weight, axis, precision)


def move_exp_nanstd(arr, /, *, alpha, min_weight=0, axis=-1, precision="f64"):
    """Exponentially weighted moving standard deviation (numbagg/moving_exp.py:158-223)."""
    return _move_exp("move_exp_nanstd", (arr,), alpha, min_weight, axis, precision)


def move_exp_nancov(a1, a2, /, *, alpha, min_weight=0, axis=-1, precision="f64"):
    """Exponentially weighted moving covariance (numbagg/moving_exp.py:226-272)."""
    return _move_exp("move_exp_nancov", (a1, a2), alpha, min_weight, axis, precision)


def move_exp_nancorr(a1, a2, /, *, alpha, min_weight=0, axis=-1, precision="f64"):
    """Exponentially weighted moving correlation (numbagg/moving_exp.py:275-335)."""
    return _move_exp("move_exp_nancorr", (a1, a2), alpha, min_weight, axis, precision)


__all__ = [
    "move_exp_nancorr",
    "move_exp_nancount",
    "move_exp_nancov",
    "move_exp_nanmean",
    "move_exp_nanstd",
    "move_exp_nansum",
    "move_exp_nanvar",
]
