"""move_covmatrix / move_corrmatrix (numbagg/moving_matrix.py:16-201), on CUDA.

Same arguments and checks as numbagg's ``ndmovematrix`` decorator
(numbagg/decorators.py:778-807): input (..., obs, vars), output (..., obs, vars,
vars); at least 2-D (ValueError); ``min_count=None`` means ``window``; negative
``min_count`` and a window outside ``(0, obs]`` raise ValueError.
"""

from __future__ import annotations

import math

import torch

from . import _host, _lib


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


__all__ = ["move_corrmatrix", "move_covmatrix"]
