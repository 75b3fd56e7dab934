"""Moving and exponentially weighted covariance / correlation matrices
(numbagg/moving_matrix.py), on CUDA.

move_covmatrix / move_corrmatrix take the arguments and checks of numbagg's
``ndmovematrix`` decorator (numbagg/decorators.py:778-807): input (..., obs, vars),
output (..., obs, vars, vars); at least 2-D (ValueError); ``min_count=None`` means
``window``; negative ``min_count`` and a window outside ``(0, obs]`` raise ValueError.

move_exp_nancovmatrix / move_exp_nancorrmatrix take those of ``ndmoveexpmatrix``
(numbagg/decorators.py:1061-1087): input (..., obs, vars), alpha a scalar or an array
(..., obs) broadcast against the leading dimensions, min_weight; the loop dtype is
numpy's choice between the gufunc's float32 and float64 loops (a Python float alpha
is broadcast to a float64 array, so float32 input then runs and returns float64).
"""

from __future__ import annotations

import math

import numpy as np
import torch

from . import _host, _lib
from .moving_exp import loop_dtype


def _move_matrix(name: str, a, window, min_count):
    shape = _host.shape_of(a)
    if len(shape) < 2:
        raise ValueError(f"{name} requires at least a 2D array with shape (..., obs, vars).")
    if min_count is None:
        min_count = window
    elif min_count < 0:
        raise ValueError(f"min_count must be positive: {min_count}")
    if not 0 < window <= shape[-2]:
        raise ValueError(f"window not in valid range: {window}")
    window = _host.check_int("window", window)
    min_count = _host.check_int("min_count", min_count)
    t, restore = _host.to_device(a)
    dtype = _host.float_compute_dtype(t.dtype)
    n_obs, n_vars = t.shape[-2:]
    lead = tuple(t.shape[:-2])
    batch = math.prod(lead)
    flat = t.to(dtype).contiguous().reshape(batch, n_obs, n_vars)
    out = torch.empty((batch, n_obs, n_vars, n_vars), dtype=dtype, device=t.device)
    if out.numel():
        L = _lib.lib()
        fn = getattr(L, f"nbg_{name}_{_host.FLOAT_SFX[dtype]}")
        for b0 in range(0, batch, 65535):
            b1 = min(batch, b0 + 65535)
            _lib.check(
                fn(flat[b0:b1].data_ptr(), out[b0:b1].data_ptr(), b1 - b0, n_obs, n_vars, window, min_count,
                   _host.stream(t.device)),
                name,
            )
    return restore(out.reshape(lead + (n_obs, n_vars, n_vars)))


def move_covmatrix(a, window, min_count=None, **kwargs):
    """Rolling pairwise-complete covariance matrix (numbagg/moving_matrix.py:117-201)."""
    if kwargs:
        raise TypeError(f"unexpected keyword arguments: {sorted(kwargs)}")
    return _move_matrix("move_covmatrix", a, window, min_count)


def move_corrmatrix(a, window, min_count=None, **kwargs):
    """Rolling pairwise-complete correlation matrix (numbagg/moving_matrix.py:16-114)."""
    if kwargs:
        raise TypeError(f"unexpected keyword arguments: {sorted(kwargs)}")
    return _move_matrix("move_corrmatrix", a, window, min_count)


def _move_exp_matrix(name: str, a, alpha, min_weight):
    shape = _host.shape_of(a)
    if len(shape) < 2:
        raise ValueError(f"{name} requires at least a 2D array with shape (..., obs, vars).")
    t, restore = _host.to_device(a)
    n_obs, n_vars = t.shape[-2:]
    if not isinstance(alpha, (np.ndarray, torch.Tensor)):
        alpha = np.broadcast_to(np.asarray(alpha), (n_obs,))
    dtype = loop_dtype([t], alpha, min_weight)
    at, _ = _host.to_device(alpha)
    at = at.to(device=t.device, dtype=dtype)
    if at.ndim == 0 or at.shape[-1] != n_obs:
        raise ValueError(f"alpha must have {n_obs} values along its last axis (the observations)")
    lead = torch.broadcast_shapes(tuple(t.shape[:-2]), tuple(at.shape[:-1]))
    batch = math.prod(lead)
    flat = torch.broadcast_to(t.to(dtype), lead + (n_obs, n_vars)).contiguous().reshape(batch, n_obs, n_vars)
    if at.ndim == 1:
        al, stride = at.contiguous(), 0
    else:
        al, stride = torch.broadcast_to(at, lead + (n_obs,)).contiguous().reshape(batch, n_obs), n_obs
    mw = float(np.float32(min_weight)) if dtype == torch.float32 else float(min_weight)
    out = torch.empty((batch, n_obs, n_vars, n_vars), dtype=dtype, device=t.device)
    if out.numel():
        L = _lib.lib()
        corr = 1 if name.endswith("corrmatrix") else 0
        f64 = 1 if dtype == torch.float64 else 0
        fn = getattr(L, f"nbg_{name}_{_host.FLOAT_SFX[dtype]}")
        for b0 in range(0, batch, 65535):
            b1 = min(batch, b0 + 65535)
            ws = _lib.workspaces.scratch(L.nbg_move_exp_matrix_workspace_bytes(corr, f64, b1 - b0, n_obs, n_vars), t.device)
            al_b = al if stride == 0 else al[b0:b1]
            _lib.check(
                fn(flat[b0:b1].data_ptr(), al_b.data_ptr(), stride, mw, out[b0:b1].data_ptr(), b1 - b0, n_obs, n_vars,
                   ws.data_ptr(), ws.numel(), _host.stream(t.device)),
                name,
            )
    return restore(out.reshape(tuple(lead) + (n_obs, n_vars, n_vars)))


def move_exp_nancovmatrix(a, alpha, min_weight=0, **kwargs):
    """Exponentially weighted pairwise-complete covariance matrix at every step
    (numbagg/moving_matrix.py:323-432)."""
    if kwargs:
        raise TypeError(f"unexpected keyword arguments: {sorted(kwargs)}")
    return _move_exp_matrix("move_exp_nancovmatrix", a, alpha, min_weight)


def move_exp_nancorrmatrix(a, alpha, min_weight=0, **kwargs):
    """Exponentially weighted pairwise-complete correlation matrix at every step
    (numbagg/moving_matrix.py:204-320)."""
    if kwargs:
        raise TypeError(f"unexpected keyword arguments: {sorted(kwargs)}")
    return _move_exp_matrix("move_exp_nancorrmatrix", a, alpha, min_weight)


__all__ = ["move_corrmatrix", "move_covmatrix", "move_exp_nancorrmatrix", "move_exp_nancovmatrix"]
