"""Labelled reductions group_nan* (numbagg/grouped.py), on CUDA.

Same keywords, axis modes, dtype rules and errors as numbagg's ``groupndreduce``
decorator (numbagg/decorators.py:558-674):

* labels must be an integer array (TypeError otherwise); negative labels are
  skipped; ``num_labels=None`` means ``max(labels) + 1``;
* ``axis=None``: labels have the values' shape; ``axis=int``: labels are 1-D along
  that axis; ``axis=tuple``: labels have the shape of those axes;
* bool values become int32 (TypeError for nanvar/nanstd); nanmean/nanvar/nanstd
  compute integer values in float64 and return float64;
* the result has shape ``broadcast_dims + (num_labels,)`` and the values' dtype.

Label values >= num_labels are skipped (numba leaves them undefined).  For integer
outputs, a group with no values reads as the dtype's minimum where numbagg stores NaN
(nanargmax/argmin/min/max/last; numba converts that NaN with fptosi, whose x86-64
result is the minimum) and as 0 for nanfirst (numbagg leaves np.empty memory there).
"""

from __future__ import annotations

import math

import numpy as np
import torch

from . import _host, _lib

# name -> (supports_bool, supports_ints, supports_ddof), numbagg/grouped.py decorators
_FLAGS = {
    "nanmean": (True, False, False),
    "nansum": (True, True, False),
    "nancount": (True, True, False),
    "nanargmax": (True, True, False),
    "nanargmin": (True, True, False),
    "nanfirst": (True, True, False),
    "nanlast": (True, True, False),
    "nanprod": (True, True, False),
    "nansum_of_squares": (True, True, False),
    "nanvar": (False, False, True),
    "nanstd": (False, False, True),
    "nanmin": (True, True, False),
    "nanmax": (True, True, False),
    "nanany": (True, True, False),
    "nanall": (True, True, False),
}

_MAX_ROWS = 65535
_LABELS_MSG = (
    "labels must be an integer array; it's expected to have already been factorized with a function such as `pd.factorize`"
)


def _group(name, values, labels, *, ddof=1, num_labels=None, axis=None):
    supports_bool, supports_ints, _ = _FLAGS[name]
    # ---- checks on metadata only (no device work) ----
    if not _host.is_tensor(values):
        values = np.asarray(values)
    if not _host.is_tensor(labels):
        labels = np.asarray(labels)
        if labels.dtype.kind != "i":
            raise TypeError(_LABELS_MSG)
    elif labels.dtype not in (torch.int8, torch.int16, torch.int32, torch.int64):
        raise TypeError(_LABELS_MSG)
    is_bool = values.dtype == (torch.bool if _host.is_tensor(values) else np.bool_)
    if is_bool and not supports_bool:
        raise TypeError(f"group_{name} does not support boolean input. Convert to a numeric type first.")
    vshape = _host.shape_of(values)
    lshape = _host.shape_of(labels)
    ndim = len(vshape)
    if axis is None:
        if vshape != lshape:
            raise ValueError(f"axis required if values and labels have different shapes: {vshape} vs {lshape}")
        moved_axes = None
    elif isinstance(axis, int):
        ax = _host.normalize_axis(axis, ndim)
        if lshape != (vshape[ax],):
            raise ValueError(f"values must have same shape along axis as labels: {(vshape[ax],)} vs {lshape}")
        moved_axes = (ax,)
    else:
        axes = tuple(_host.normalize_axis(a, ndim) for a in axis)
        want = tuple(vshape[a] for a in axes)
        if lshape != want:
            raise ValueError(f"values must have same shape along axis as labels: {want} vs {lshape}")
        moved_axes = axes
    if num_labels is None:
        if int(np.prod(lshape)) == 0:
            raise ValueError("zero-size array to reduction operation maximum which has no identity")
        num_labels = int(labels.max().item() if _host.is_tensor(labels) else np.max(labels)) + 1
    num_labels = _host.check_int("num_labels", num_labels)
    if num_labels < 0:
        raise ValueError(f"num_labels must be non-negative: {num_labels}")

    # ---- device work ----
    v, restore = _host.to_device(values)
    lab = labels.to(v.device) if _host.is_tensor(labels) else _host.to_device(labels)[0]
    if v.dtype == torch.bool:
        v = v.to(torch.int32)
    if not supports_ints and not v.dtype.is_floating_point:
        v = v.to(torch.float64)
    result_dtype = v.dtype
    if v.dtype in (torch.float16, torch.bfloat16):
        work = torch.float32
    elif v.dtype in (torch.int8, torch.int16, torch.uint8):
        work = torch.int64
    else:
        work = v.dtype
    cols = _group_columns(name, v, lab, moved_axes, num_labels, ddof)
    if cols is not None:
        return restore(cols)
    if moved_axes is None:
        core = v.ndim
    else:
        v = torch.movedim(v, moved_axes, tuple(range(-len(moved_axes), 0)))
        core = len(moved_axes)
    bshape = tuple(v.shape[: v.ndim - core])
    m = math.prod(v.shape[v.ndim - core :])
    rows = math.prod(bshape)
    flat = v.to(work).contiguous().reshape(rows, m)
    lab_dt = torch.int64 if lab.dtype == torch.int64 else torch.int32
    flat_lab = lab.to(lab_dt).contiguous().reshape(m)
    out = torch.empty((rows, num_labels), dtype=work, device=flat.device)
    if rows and num_labels:
        L = _lib.lib()
        # torch.use_deterministic_algorithms(True) selects the reproducible kernels
        deterministic = torch.are_deterministic_algorithms_enabled()
        L.nbg_set_deterministic(1 if deterministic else 0)
        fid = _lib.GROUP_FUNC_IDS[name]
        fn = getattr(L, f"nbg_group_{name}_{_host.ALL_SFX[work]}_{'i64' if lab_dt == torch.int64 else 'i32'}")
        for r0 in range(0, rows, _MAX_ROWS):
            r1 = min(rows, r0 + _MAX_ROWS)
            nb = L.nbg_group_workspace_bytes(fid, r1 - r0, m, num_labels)
            ws = _lib.workspaces.scratch(nb, flat.device)
            status = fn(
                flat[r0:r1].data_ptr() if m else None,
                flat_lab.data_ptr() if m else None,
                out[r0:r1].data_ptr(),
                r1 - r0,
                m,
                num_labels,
                int(ddof),
                ws.data_ptr(),
                ws.numel(),
                _host.stream(flat.device),
            )
            if status == _lib.UNSUPPORTED and deterministic:
                raise RuntimeError(
                    f"group_{name} with num_labels={num_labels} on floating-point values has no deterministic "
                    "implementation (its bins do not fit in shared memory), but torch.use_deterministic_algorithms "
                    "is on"
                )
            _lib.check(status, f"group_{name}")
    res = out.reshape(bshape + (num_labels,))
    if work != result_dtype:
        res = res.to(result_dtype)
    return restore(res)


_COLS_DTYPES = {torch.float64: "f64", torch.float32: "f32", torch.int32: "i32", torch.int64: "i64"}


def group_columns_layout(shape, moved_axes, itemsize=8):
    """(outer, m, inner) when the reduced axes are consecutive, increasing and not last
    (a C-contiguous array is then `outer` blocks of m x `inner` values, the labels
    running over m) and there are enough columns for the column kernel to beat the copy
    (`_host.column_min`); else None."""
    if not moved_axes:
        return None
    axes = tuple(moved_axes)
    k0 = axes[0]
    if axes != tuple(range(k0, k0 + len(axes))) or axes[-1] >= len(shape) - 1:
        return None
    outer = math.prod(shape[:k0])
    m = math.prod(shape[k0 : axes[-1] + 1])
    inner = math.prod(shape[axes[-1] + 1 :])
    if outer * inner < _host.column_min(itemsize):
        return None
    return outer, m, inner


def _group_columns(name, v, lab, moved_axes, num_labels, ddof):
    """Values reduced over consecutive, increasing, non-last axes of a C-contiguous
    array: one thread per column runs numbagg's loop in place (no copy, the reference's
    results bit for bit).  None when that does not apply."""
    if v.dtype not in _COLS_DTYPES or not v.is_contiguous():
        return None
    layout = group_columns_layout(tuple(v.shape), moved_axes, v.element_size())
    if layout is None:
        return None
    L = _lib.lib()
    if num_labels > L.nbg_group_cols_max_labels(_lib.GROUP_FUNC_IDS[name]):
        return None
    outer, m, inner = layout
    k0, k1 = moved_axes[0], moved_axes[-1]
    lab_dt = torch.int64 if lab.dtype == torch.int64 else torch.int32
    flat_lab = lab.to(lab_dt).contiguous().reshape(m)
    out = torch.empty(tuple(v.shape[:k0]) + tuple(v.shape[k1 + 1 :]) + (num_labels,), dtype=v.dtype, device=v.device)
    if out.numel():
        fn = getattr(L, f"nbg_group_{name}_cols_{_COLS_DTYPES[v.dtype]}_{'i64' if lab_dt == torch.int64 else 'i32'}")
        _lib.check(fn(v.data_ptr() if m else None, flat_lab.data_ptr() if m else None, out.data_ptr(), outer, m, inner,
                      num_labels, int(ddof), _host.stream(v.device)), f"group_{name}")
    return out


def _make(name: str, doc_lines: str):
    supports_ddof = _FLAGS[name][2]
    if supports_ddof:

        def f(values, labels, *, ddof=1, num_labels=None, axis=None):
            return _group(name, values, labels, ddof=ddof, num_labels=num_labels, axis=axis)

    else:
        # numbagg accepts ddof for every grouped function and ignores it where the
        # function has none (groupndreduce.__call__, numbagg/decorators.py:558-674)

        def f(values, labels, *, ddof=1, num_labels=None, axis=None):
            return _group(name, values, labels, num_labels=num_labels, axis=axis)

    f.__name__ = f.__qualname__ = f"group_{name}"
    f.__doc__ = doc_lines
    f.supports_bool, f.supports_ints, f.supports_ddof = _FLAGS[name]
    return f


group_nanmean = _make("nanmean", "Mean of non-NaN values per label (numbagg/grouped.py:7-27).")
group_nansum = _make("nansum", "Sum of non-NaN values per label (numbagg/grouped.py:30-40).")
group_nancount = _make("nancount", "Count of non-NaN values per label (numbagg/grouped.py:43-51).")
group_nanargmax = _make("nanargmax", "Flat index of the first maximum per label (numbagg/grouped.py:54-75).")
group_nanargmin = _make("nanargmin", "Flat index of the first minimum per label (numbagg/grouped.py:78-92).")
group_nanfirst = _make("nanfirst", "First non-NaN value per label (numbagg/grouped.py:95-110).")
group_nanlast = _make("nanlast", "Last non-NaN value per label (numbagg/grouped.py:113-121).")
group_nanprod = _make("nanprod", "Product of non-NaN values per label (numbagg/grouped.py:124-132).")
group_nansum_of_squares = _make(
    "nansum_of_squares", "Sum of squares of non-NaN values per label (numbagg/grouped.py:135-145)."
)
group_nanvar = _make("nanvar", "Variance (ddof, default 1) per label (numbagg/grouped.py:148-176).")
group_nanstd = _make("nanstd", "Standard deviation (ddof, default 1) per label (numbagg/grouped.py:179-208).")
group_nanmin = _make("nanmin", "Minimum of non-NaN values per label (numbagg/grouped.py:211-226).")
group_nanmax = _make("nanmax", "Maximum of non-NaN values per label (numbagg/grouped.py:229-244).")
group_nanany = _make("nanany", "Any non-NaN truthy value per label (numbagg/grouped.py:247-257).")
group_nanall = _make("nanall", "All non-NaN values truthy per label (numbagg/grouped.py:260-270).")

__all__ = [
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
]
