"""CPU oracle for numbagg's scan / reduction hot path -- TEST INFRASTRUCTURE ONLY.

A ctypes front end to ``nbg_oracle.c``, the loop-for-loop C restatement of the
reference kernels (numbagg/moving.py, numbagg/moving_exp.py, numbagg/funcs.py:294-326,
numbagg/grouped.py, numbagg/moving_matrix.py:16-201).  It is imported only by the
tests, by the smoke check and by the CPU-baseline leg of the benchmark -- as the
checker, never as the thing measured or shipped.  The product package
``numbagg_gb300`` never imports it.

The argument handling mirrors numbagg's decorators (numbagg/decorators.py:305-341,
:374-414, :465-487, :558-674, :778-807) so that a test reads like the reference's
own tests: the scanned axis is moved last and made contiguous, and the grouped
functions apply the same dtype promotions (bool -> int32, ints -> float64 where
``supports_ints=False``).
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

from .build import LIB, build

_lib = None

_F = {np.dtype(np.float64): "f64", np.dtype(np.float32): "f32"}
_ALL = {
    np.dtype(np.float64): "f64",
    np.dtype(np.float32): "f32",
    np.dtype(np.int32): "i32",
    np.dtype(np.int64): "i64",
}

MOVE_FUNCS = ("move_sum", "move_mean", "move_var", "move_std", "move_cov", "move_corr")
MOVE2 = ("move_cov", "move_corr")
MOVE_EXP_FUNCS = (
    "move_exp_nancount",
    "move_exp_nanmean",
    "move_exp_nansum",
    "move_exp_nanvar",
    "move_exp_nanstd",
    "move_exp_nancov",
    "move_exp_nancorr",
)
MOVE_EXP2 = ("move_exp_nancov", "move_exp_nancorr")
GROUP_FUNCS = (
    "group_nanall",
    "group_nanany",
    "group_nanargmax",
    "group_nanargmin",
    "group_nancount",
    "group_nanfirst",
    "group_nanlast",
    "group_nanmax",
    "group_nanmean",
    "group_nanmin",
    "group_nanprod",
    "group_nanstd",
    "group_nansum",
    "group_nansum_of_squares",
    "group_nanvar",
)
# groupndreduce flags, numbagg/grouped.py:7, :148, :179
GROUP_NO_INTS = ("group_nanmean", "group_nanvar", "group_nanstd")
GROUP_NO_BOOL = ("group_nanvar", "group_nanstd")


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        path = LIB if os.path.exists(LIB) else build()
        _lib = ctypes.CDLL(path)
    return _lib


def _p(a: np.ndarray) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data)


def _i(v) -> ctypes.c_int64:
    return ctypes.c_int64(int(v))


def _rows_last(a: np.ndarray, axis: int) -> tuple[np.ndarray, tuple[int, ...]]:
    moved = np.moveaxis(np.asarray(a), axis, -1)
    shape = moved.shape
    n = shape[-1] if moved.ndim else 1
    flat = np.ascontiguousarray(moved.reshape(-1, n) if moved.ndim else moved.reshape(1, 1))
    return flat, shape


def _restore(flat: np.ndarray, shape: tuple[int, ...], axis: int) -> np.ndarray:
    return np.moveaxis(flat.reshape(shape), -1, axis)


def move(name, a, b=None, *, window, min_count=None, axis=-1, nthreads=0, ext=False):
    """numbagg.move_* restated (ndmove.__call__, numbagg/decorators.py:305-341).

    ext=True runs the same loop with long double accumulators (IEEE binary128 on
    aarch64, 80-bit on x86-64): an estimate of the exact result."""
    a = np.asarray(a)
    if min_count is None:
        min_count = window
    elif min_count < 0:
        raise ValueError(f"min_count must be positive: {min_count}")
    if not 0 < window <= a.shape[axis]:
        raise ValueError(f"window not in valid range: {window}")
    dt = _F[np.dtype(a.dtype).newbyteorder("=")]
    fa, shape = _rows_last(a.astype(a.dtype.newbyteorder("="), copy=False), axis)
    out = np.empty_like(fa)
    rows, n = fa.shape
    fn = getattr(lib(), f"orc_{name}_ext_{dt}" if ext else f"orc_{name}_{dt}")
    if name in MOVE2:
        fb, _ = _rows_last(np.asarray(b).astype(fa.dtype), axis)
        fn(_p(fa), _p(fb), _p(out), _i(rows), _i(n), _i(window), _i(min_count), ctypes.c_int(nthreads))
    else:
        fn(_p(fa), _p(out), _i(rows), _i(n), _i(window), _i(min_count), ctypes.c_int(nthreads))
    return _restore(out, shape, axis)


def move_exp(name, a, b=None, *, alpha, min_weight=0.0, axis=-1, nthreads=0, ext=False):
    """numbagg.move_exp_* restated (ndmoveexp.__call__, numbagg/decorators.py:374-414).

    The loop dtype is numpy's choice between the gufunc's float32 and float64 loops
    (numbagg/moving_exp.py:12-17): a scalar alpha becomes np.broadcast_to(alpha, n),
    a float64 array for a Python float, so the float32 loop runs only when the arrays
    and an alpha array all cast safely to float32.
    ext=True: long double accumulators, as for move()."""
    a = np.asarray(a)
    operands = [a] + ([np.asarray(b)] if b is not None else [])
    alpha_dt = alpha.dtype if isinstance(alpha, np.ndarray) else np.asarray(alpha).dtype
    dts = [x.dtype for x in operands] + [alpha_dt]
    if isinstance(min_weight, np.generic):
        dts.append(min_weight.dtype)
    f32 = all(np.can_cast(d, np.float32, casting="safe") for d in dts)
    dtype = np.dtype(np.float32 if f32 else np.float64)
    dt = _F[dtype]
    fa, shape = _rows_last(a.astype(dtype, copy=False), axis)
    rows, n = fa.shape
    if not isinstance(alpha, np.ndarray):
        al = np.full((1, n), alpha, dtype=dtype)
        stride = 0
    elif alpha.ndim == 1:
        al = np.ascontiguousarray(alpha.astype(dtype)).reshape(1, n)
        stride = 0
    else:
        al, _ = _rows_last(np.broadcast_to(alpha, a.shape).astype(dtype), axis)
        stride = n
    out = np.empty_like(fa)
    mw = ctypes.c_double(min_weight) if dt == "f64" else ctypes.c_float(min_weight)
    fn = getattr(lib(), f"orc_{name}_ext_{dt}" if ext else f"orc_{name}_{dt}")
    if name in MOVE_EXP2:
        fb, _ = _rows_last(np.asarray(b).astype(dtype), axis)
        fn(_p(fa), _p(fb), _p(al), _i(stride), mw, _p(out), _i(rows), _i(n), ctypes.c_int(nthreads))
    else:
        fn(_p(fa), _p(al), _i(stride), mw, _p(out), _i(rows), _i(n), ctypes.c_int(nthreads))
    return _restore(out, shape, axis)


def fill(name, a, *, limit=None, axis=-1, nthreads=0):
    """numbagg.ffill / bfill restated (ndfill.__call__, numbagg/decorators.py:465-487)."""
    a = np.asarray(a)
    if limit is None:
        limit = a.shape[axis]
    if limit < 0:
        raise ValueError(f"`limit` must be positive: {limit}")
    dtype = np.dtype(a.dtype).newbyteorder("=")
    dt = _ALL[dtype]
    fa, shape = _rows_last(a.astype(dtype, copy=False), axis)
    out = np.empty_like(fa)
    rows, n = fa.shape
    getattr(lib(), f"orc_{name}_{dt}")(
        _p(fa), _p(out), _i(rows), _i(n), _i(limit), ctypes.c_int(nthreads)
    )
    return _restore(out, shape, axis)


def group(name, values, labels, *, num_labels=None, axis=None, ddof=1, nthreads=0):
    """numbagg.group_* restated (groupndreduce.__call__, numbagg/decorators.py:558-674)."""
    values = np.asarray(values)
    labels = np.asarray(labels)
    if labels.dtype.kind != "i":
        raise TypeError("labels must be an integer array")
    if values.dtype == np.bool_:
        if name in GROUP_NO_BOOL:
            raise TypeError(f"{name} does not support boolean input.")
        values = values.astype(np.int32)
    if num_labels is None:
        num_labels = int(np.max(labels)) + 1
    if name in GROUP_NO_INTS and np.issubdtype(values.dtype, np.integer):
        values = values.astype(np.float64)
    if values.dtype.kind == "i" and values.dtype not in (np.dtype(np.int32), np.dtype(np.int64)):
        values = values.astype(np.int64)
    if axis is None:
        if values.shape != labels.shape:
            raise ValueError("axis required if values and labels have different shapes")
        core = values.ndim
    elif isinstance(axis, int):
        if labels.shape != (values.shape[axis],):
            raise ValueError("values must have same shape along axis as labels")
        values = np.moveaxis(values, axis, -1)
        core = 1
    else:
        vshape = tuple(values.shape[ax] for ax in axis)
        if labels.shape != vshape:
            raise ValueError("values must have same shape along axis as labels")
        values = np.moveaxis(values, axis, range(-len(axis), 0, 1))
        core = len(axis)
    bshape = values.shape[: values.ndim - core]
    m = int(np.prod(values.shape[values.ndim - core :], dtype=np.int64))
    dtype = np.dtype(values.dtype).newbyteorder("=")
    fv = np.ascontiguousarray(values.astype(dtype, copy=False)).reshape(-1, m)
    fl = np.ascontiguousarray(labels.astype(np.int64)).reshape(m)
    rows = fv.shape[0]
    out = np.zeros((rows, num_labels), dtype=dtype)
    getattr(lib(), f"orc_{name}_{_ALL[dtype]}")(
        _p(fv), _p(fl), _p(out), _i(rows), _i(m), _i(num_labels), _i(ddof), ctypes.c_int(nthreads)
    )
    return out.reshape(bshape + (num_labels,))


def move_matrix(name, a, *, window, min_count=None, nthreads=0, ext=False):
    """numbagg.move_covmatrix / move_corrmatrix restated (ndmovematrix.__call__,
    numbagg/decorators.py:778-807).  ext=True computes in long double (arrays and
    accumulators) and returns float64."""
    a = np.asarray(a)
    if a.ndim < 2:
        raise ValueError(f"{name} requires at least a 2D array with shape (..., obs, vars).")
    if min_count is None:
        min_count = window
    elif min_count < 0:
        raise ValueError(f"min_count must be positive: {min_count}")
    if not 0 < window <= a.shape[-2]:
        raise ValueError(f"window not in valid range: {window}")
    dtype = np.dtype(a.dtype).newbyteorder("=")
    dt = _F[dtype]
    if ext:
        dtype, dt = np.dtype(np.longdouble), "ld"
    t_obs, n_vars = a.shape[-2:]
    fa = np.ascontiguousarray(a.astype(dtype, copy=False)).reshape(-1, t_obs, n_vars)
    out = np.empty((fa.shape[0], t_obs, n_vars, n_vars), dtype=dtype)
    getattr(lib(), f"orc_{name}_{dt}")(
        _p(fa), _p(out), _i(fa.shape[0]), _i(t_obs), _i(n_vars), _i(window), _i(min_count),
        ctypes.c_int(nthreads),
    )
    if ext:
        out = out.astype(np.float64)
    return out.reshape(a.shape[:-2] + (t_obs, n_vars, n_vars))


def move_exp_matrix(name, a, *, alpha, min_weight=0.0, nthreads=0, ext=False):
    """numbagg.move_exp_nancovmatrix / move_exp_nancorrmatrix restated
    (ndmoveexpmatrix.__call__, numbagg/decorators.py:1061-1087): a (..., obs, vars),
    alpha a scalar (broadcast along obs as np.broadcast_to does, hence float64 for a
    Python float) or an array (..., obs).  The loop dtype is numpy's choice between the
    float32 and float64 loops (numbagg/moving_matrix.py:204-212).  ext=True computes
    in long double and returns float64."""
    a = np.asarray(a)
    if a.ndim < 2:
        raise ValueError(f"{name} requires at least a 2D array with shape (..., obs, vars).")
    if not isinstance(alpha, np.ndarray):
        alpha = np.broadcast_to(alpha, a.shape[-2])
    dts = [a.dtype, alpha.dtype] + ([min_weight.dtype] if isinstance(min_weight, np.generic) else [])
    f32 = all(np.can_cast(d, np.float32, casting="safe") for d in dts)
    dtype = np.dtype(np.float32 if f32 else np.float64)
    dt = _F[dtype]
    if ext:
        dtype, dt = np.dtype(np.longdouble), "ld"
    lead = np.broadcast_shapes(a.shape[:-2], alpha.shape[:-1])
    t_obs, n_vars = a.shape[-2:]
    fa = np.ascontiguousarray(np.broadcast_to(a, lead + (t_obs, n_vars)).astype(dtype)).reshape(-1, t_obs, n_vars)
    if alpha.ndim == 1:
        al = np.ascontiguousarray(alpha.astype(dtype)).reshape(1, t_obs)
        stride = 0
    else:
        al = np.ascontiguousarray(np.broadcast_to(alpha, lead + (t_obs,)).astype(dtype)).reshape(-1, t_obs)
        stride = t_obs
    out = np.empty((fa.shape[0], t_obs, n_vars, n_vars), dtype=dtype)
    mw = {"f64": ctypes.c_double, "f32": ctypes.c_float, "ld": ctypes.c_longdouble}[dt](min_weight)
    getattr(lib(), f"orc_{name}_{dt}")(
        _p(fa), _p(al), _i(stride), mw, _p(out), _i(fa.shape[0]), _i(t_obs), _i(n_vars), ctypes.c_int(nthreads)
    )
    if ext:
        out = out.astype(np.float64)
    return out.reshape(lead + (t_obs, n_vars, n_vars))


def static_matrix(name, a, *, nthreads=0, ext=False):
    """numbagg.nancovmatrix / nancorrmatrix restated (ndmatrix.__call__,
    numbagg/decorators.py:700-717): a (..., vars, obs) -> (..., vars, vars), float32
    or float64 (other dtypes take the first loop they cast to safely).  ext=True
    computes in long double and returns float64."""
    a = np.asarray(a)
    if a.ndim < 2:
        raise ValueError(
            f"{name} requires at least a 2D array with shape (..., vars, obs). "
            "For 1D arrays, use nanvar for variance calculations."
        )
    dtype = np.dtype(np.float32 if np.can_cast(a.dtype, np.float32, casting="safe") else np.float64)
    dt = _F[dtype]
    if ext:
        dtype, dt = np.dtype(np.longdouble), "ld"
    n_vars, n_obs = a.shape[-2:]
    fa = np.ascontiguousarray(a.astype(dtype)).reshape(-1, n_vars, n_obs)
    out = np.empty((fa.shape[0], n_vars, n_vars), dtype=dtype)
    getattr(lib(), f"orc_{name}_{dt}")(_p(fa), _p(out), _i(fa.shape[0]), _i(n_vars), _i(n_obs), ctypes.c_int(nthreads))
    if ext:
        out = out.astype(np.float64)
    return out.reshape(a.shape[:-2] + (n_vars, n_vars))


__all__ = [
    "GROUP_FUNCS",
    "MOVE_EXP_FUNCS",
    "MOVE_FUNCS",
    "fill",
    "group",
    "lib",
    "move",
    "move_exp",
    "move_exp_matrix",
    "move_matrix",
    "static_matrix",
]


# ---- static aggregations (numbagg/funcs.py:23-242), restated in numpy --------------------
AGG_INT_FLOAT_LOOPS = (np.int32, np.int64, np.float32, np.float64)
AGG_FLOAT_LOOPS = (np.float32, np.float64)


def _seq_sum(x: np.ndarray, dtype) -> np.ndarray:
    """Sequential left-to-right sum along the last axis in `dtype` (a numba loop's
    order): the last element of the running sum."""
    if x.shape[-1] == 0:
        return np.zeros(x.shape[:-1], dtype=dtype)
    return np.add.accumulate(x.astype(dtype), axis=-1, dtype=dtype)[..., -1]


def aggregate(name, a, *, axis=None, ddof=1, ext=False):
    """numbagg.<name> for the static aggregations, restated from numbagg/funcs.py:23-242
    with the axis handling of ndaggregate / ndreduce (numbagg/decorators.py:231-255,
    :1002-1028; numbagg/utils.py:20-32).  The loop dtype is the first of the reference's
    signatures the input casts to safely.  ext=True sums in long double (the
    accuracy yardstick); otherwise sums run left to right in the reference's
    accumulator dtype."""
    a = np.asarray(a)
    loops = AGG_FLOAT_LOOPS if name in ("nanmean", "nanvar", "nanstd") else AGG_INT_FLOAT_LOOPS
    loop = next((lp for lp in loops if np.can_cast(a.dtype, lp, casting="safe")), None)
    if loop is None:
        raise TypeError(f"ufunc '{name}' not supported for the input types {a.dtype}")
    a = a.astype(loop)
    if a.ndim == 0:
        a = a.reshape(1)
    if axis is None:
        axes = tuple(range(a.ndim))
    elif isinstance(axis, tuple):
        axes = tuple(ax % a.ndim for ax in axis)
    else:
        axes = (axis % a.ndim,)
    moved = np.moveaxis(a, axes, range(a.ndim - len(axes), a.ndim))
    out_shape = moved.shape[: a.ndim - len(axes)]
    m = int(np.prod(moved.shape[a.ndim - len(axes) :], dtype=np.int64))
    x = np.ascontiguousarray(moved).reshape(out_shape + (m,))
    is_float = np.issubdtype(loop, np.floating)
    nan = np.isnan(x) if is_float else np.zeros(x.shape, dtype=bool)
    cnt = (~nan).sum(axis=-1).astype(np.int64)
    acc = np.longdouble if ext else np.float64
    zeroed = np.where(nan, 0, x)
    if name == "allnan":
        return nan.all(axis=-1)
    if name == "anynan":
        return nan.any(axis=-1)
    if name == "nancount":
        return cnt
    if name == "nansum":
        if not is_float:
            return zeroed.sum(axis=-1, dtype=loop)  # wraps like the integer loop
        return _seq_sum(zeroed, acc if ext else loop).astype(loop)  # numbagg/funcs.py:79-84
    if name == "nanmean":
        with np.errstate(invalid="ignore", divide="ignore"):
            return (_seq_sum(zeroed, acc) / cnt).astype(loop)  # :93-103
    if name in ("nanvar", "nanstd"):  # two passes, :113-133 / :143-159
        with np.errstate(invalid="ignore", divide="ignore"):
            mean = _seq_sum(zeroed, acc) / cnt
            dev = np.where(nan, 0, x.astype(acc) - mean[..., None])
            ss = _seq_sum(dev * dev, acc)
            v = ss / (cnt - ddof)
            v = np.where((cnt > ddof) & (cnt > 0), v, np.nan)
            if name == "nanstd":
                v = np.sqrt(v)
        return v.astype(loop)
    if name in ("nanmax", "nanmin"):  # :207-242
        if m == 0 and x.size == 0 and int(np.prod(out_shape)) > 0:
            op = "fmax" if name == "nanmax" else "fmin"
            raise ValueError(f"zero-size array to reduction operation {op} which has no identity")
        if not is_float:
            return x.max(axis=-1) if name == "nanmax" else x.min(axis=-1)
        fill = -np.inf if name == "nanmax" else np.inf
        r = np.where(nan, fill, x)
        r = r.max(axis=-1) if name == "nanmax" else r.min(axis=-1)
        return np.where(cnt > 0, r, np.nan).astype(loop)
    if name in ("nanargmax", "nanargmin"):  # :167-199: the first extreme, raising on all-NaN
        if int(np.prod(out_shape)) > 0 and (m == 0 or (cnt == 0).any()):
            raise ValueError("All-NaN slice encountered")
        fill = -np.inf if name == "nanargmax" else np.inf
        r = np.where(nan, fill, x) if is_float else x
        return (r.argmax(axis=-1) if name == "nanargmax" else r.argmin(axis=-1)).astype(np.int64)
    raise ValueError(f"unknown aggregation {name}")
