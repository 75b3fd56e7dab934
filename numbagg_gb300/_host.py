"""Host-side helpers shared by the public functions: device placement, dtype
promotion and the "move the scanned axis last, make it contiguous" step that numba's
gufunc machinery performs for numbagg (numbagg/decorators.py:340-341, :409-414)."""

from __future__ import annotations

import numbers
from collections.abc import Callable

import numpy as np
import torch

from . import _lib

_NP_TO_TORCH = {
    np.dtype(np.float64): torch.float64,
    np.dtype(np.float32): torch.float32,
    np.dtype(np.float16): torch.float16,
    np.dtype(np.int64): torch.int64,
    np.dtype(np.int32): torch.int32,
    np.dtype(np.int16): torch.int16,
    np.dtype(np.int8): torch.int8,
    np.dtype(np.uint8): torch.uint8,
    np.dtype(np.bool_): torch.bool,
}

FLOAT_SFX = {torch.float64: "f64", torch.float32: "f32"}
ALL_SFX = {torch.float64: "f64", torch.float32: "f32", torch.int32: "i32", torch.int64: "i64"}


def is_tensor(x) -> bool:
    return isinstance(x, torch.Tensor)


def to_device(x) -> tuple[torch.Tensor, Callable[[torch.Tensor], object]]:
    """A CUDA tensor for `x` and a function that returns a result in `x`'s kind.

    torch CUDA tensors are used as they are.  numpy arrays (and anything
    array-like) and CPU tensors are copied to the current CUDA device and the
    result is copied back, so numbagg's numpy callers can switch unchanged.
    """
    _lib.require_cuda()
    if is_tensor(x):
        if x.is_cuda:
            return x, lambda r: r
        dev = torch.device("cuda", torch.cuda.current_device())
        return x.to(dev), lambda r: r.cpu()
    arr = np.asarray(x)
    if not arr.dtype.isnative:
        arr = arr.astype(arr.dtype.newbyteorder("="))
    if arr.dtype not in _NP_TO_TORCH:
        if arr.dtype.kind == "u":
            arr = arr.astype(np.int64)
        elif arr.dtype.kind == "f":
            arr = arr.astype(np.float64)
        else:
            raise TypeError(f"unsupported dtype {arr.dtype}")
    dev = torch.device("cuda", torch.cuda.current_device())
    t = torch.from_numpy(np.ascontiguousarray(arr)).to(dev)
    return t, lambda r: r.cpu().numpy()


def shape_of(x) -> tuple[int, ...]:
    """Shape of a tensor or array-like without moving it."""
    if is_tensor(x):
        return tuple(x.shape)
    return tuple(np.shape(x))


def float_compute_dtype(dt: torch.dtype) -> torch.dtype:
    """The gufunc loop numpy would pick: float32 for float32/float16, else float64."""
    if dt in (torch.float32, torch.float16, torch.bfloat16):
        return torch.float32
    return torch.float64


def rows_last(t: torch.Tensor, axis: int) -> tuple[torch.Tensor, tuple[int, ...]]:
    """View `t` with `axis` last as a C-contiguous (rows, n) tensor."""
    moved = torch.movedim(t, axis, -1)
    shape = tuple(moved.shape)
    n = shape[-1]
    flat = moved.contiguous().reshape(-1, n)
    return flat, shape


# The one-thread-per-column kernels walk each column serially (0.2 us a position for a
# fill, about 0.5 for a grouped reduction, 0.8-1.1 for a moving window or an EWM, which
# run numbagg's float64 loop), so they need many columns to beat moving the axis last
# with a copy and running the row kernels.  Measured on a GB300, float64 along axis 0:
# 16,384 x 8,192 took 1.06 / 3.36 / 4.46 / 1.28 ms (fill / move_mean / EWM mean / grouped
# sum) through the copy against 3.2 / 13.0 / 17.6 / 7.3 ms in place; 2,048 x 65,536 took
# 1.26 / 3.57 / 4.47 / 4.26 ms through the copy against 0.54 / 3.11 / 4.38 / 0.93 ms in
# place.  The crossover is near 256 KB of columns per position.
MIN_COLUMNS = 2048
COLUMN_MIN_ROW_BYTES = 256 * 1024


def column_min(itemsize: int) -> int:
    """Fewest columns for the in-place column kernels at this element size."""
    return max(MIN_COLUMNS, COLUMN_MIN_ROW_BYTES // max(int(itemsize), 1))


def column_layout(t: torch.Tensor, axis: int, min_columns: int | None = None) -> tuple[int, int, int] | None:
    """(outer, n, inner) when `t` is C-contiguous and `axis` is not its last axis: the
    array is then `outer` blocks of n x `inner` values, and a kernel with one thread per
    column scans it along `axis` in place, with no copy (numbagg's gufuncs take such
    strided core axes directly, numbagg/decorators.py:340-341).  None when that does
    not apply or the columns are too few to fill the GPU."""
    if t.ndim < 2 or axis == t.ndim - 1 or not t.is_contiguous():
        return None
    outer = 1
    for d in t.shape[:axis]:
        outer *= int(d)
    inner = 1
    for d in t.shape[axis + 1 :]:
        inner *= int(d)
    if outer * inner < (column_min(t.element_size()) if min_columns is None else min_columns):
        return None
    return outer, int(t.shape[axis]), inner


def restore_axis(flat: torch.Tensor, shape: tuple[int, ...], axis: int) -> torch.Tensor:
    return torch.movedim(flat.reshape(shape), -1, axis)


def normalize_axis(axis: int, ndim: int) -> int:
    if not -ndim <= axis < ndim:
        raise np.exceptions.AxisError(axis, ndim)
    return axis % ndim


def check_int(name: str, value) -> int:
    if isinstance(value, bool) or not isinstance(value, numbers.Integral):
        raise TypeError(f"`{name}` must be an integer, got {type(value).__name__}")
    return int(value)


def stream(device: torch.device) -> int:
    return _lib.stream_handle(device)
