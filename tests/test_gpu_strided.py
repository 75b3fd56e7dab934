"""A scanned axis that is not the last one (numbagg's gufuncs take such strided core
axes directly, numbagg/decorators.py:340-341, :409-414, :480-487).

For C-contiguous arrays with enough columns (256 KB of them per position, where the
in-place kernel beats moving the axis last with a copy) the fills, the moving windows,
the exponentially weighted family and the grouped reductions run one thread per column,
in place.  That kernel repeats numbagg's loop operation for operation, so float64 (and
float32 with a float32 alpha) results must equal the oracle bit for bit; the
FP32-compensated form keeps its stated 2e-6.  Narrower arrays take the copy and the row
kernels.  The last tests make the calls that xarray's rolling_exp and flox's grouped
reductions make.
"""

import numpy as np
import pytest
import torch

import numbagg_gb300 as nb
import oracle
from numbagg_gb300 import _host
from tests.parity import assert_bit_equal, exp_degenerate, exp_scale, scaled_error

pytestmark = pytest.mark.gpu

MOVE_EXP = ["move_exp_nancount", "move_exp_nanmean", "move_exp_nansum", "move_exp_nanvar", "move_exp_nanstd",
            "move_exp_nancov", "move_exp_nancorr"]


def _data(shape, seed, p_nan=0.1, dtype=np.float64):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(shape)
    x[rng.random(shape) < p_nan] = np.nan
    return x.astype(dtype)


# The first three are wide enough for the in-place column kernel (for 4-byte values
# too); the last two take the copy and the row kernel (the fills are exact either way)
@pytest.mark.parametrize("shape,axis", [
    ((200, 65536), 0), ((5, 300, 13200), 1), ((120, 3, 22000), 0), ((3000, 4096), 0), ((5, 2000, 600), 1),
])
@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32])
@pytest.mark.parametrize("fname", ["ffill", "bfill"])
def test_fill_non_last_axis(fname, dtype, shape, axis):
    x = _data(shape, 31) if dtype != np.int32 else np.random.default_rng(31).integers(-9, 9, size=shape).astype(dtype)
    if dtype != np.int32:
        x = x.astype(dtype)
        x[(np.random.default_rng(32).random(shape) < 0.3)] = np.nan  # runs of missing values
    xt = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    cols = int(np.prod(shape)) // shape[axis]
    assert (_host.column_layout(xt, axis) is not None) == (cols >= _host.column_min(x.itemsize))
    for limit in (None, 3):
        got = getattr(nb, fname)(xt, limit=limit, axis=axis).cpu().numpy()
        want = oracle.fill(fname, x, limit=limit, axis=axis)
        assert_bit_equal(got, want, f"{fname} axis={axis} limit={limit}")


MOVE = ["move_sum", "move_mean", "move_var", "move_std", "move_cov", "move_corr"]


@pytest.mark.parametrize("fname", MOVE)
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("shape,axis", [((320, 65536), 0), ((2, 400, 32768), 1)])
def test_move_non_last_axis_bit_exact(fname, dtype, shape, axis):
    x = _data(shape, 41, dtype=dtype)
    y = _data(shape, 42, dtype=dtype) if fname in ("move_cov", "move_corr") else None
    x[tuple(s // 3 for s in shape)] = np.inf  # the reference's running sums never recover
    func = getattr(nb, fname)
    xt = torch.from_numpy(x).cuda()
    assert _host.column_layout(xt, axis) is not None  # the in-place column path
    args = (xt,) if y is None else (xt, torch.from_numpy(y).cuda())
    for window, min_count in ((1, None), (7, 3), (300, 150)):
        got = func(*args, window=window, min_count=min_count, axis=axis).cpu().numpy()
        want = oracle.move(fname, x, y, window=window, min_count=min_count, axis=axis)
        assert_bit_equal(got, want, f"{fname} {np.dtype(dtype).name} w={window}")


def test_move_non_last_axis_fp32c_keeps_its_bound():
    # the compensated form runs the rows kernels (moved axis); same 2e-6 bar
    x = 1e6 + _data((2000, 2100), 43)
    got = nb.move_std(x, window=50, min_count=25, axis=0, precision="fp32c")
    ext = oracle.move("move_std", x, window=50, min_count=25, axis=0, ext=True)
    m = ~np.isnan(ext)
    assert np.array_equal(np.isnan(got), np.isnan(ext))
    assert np.max(np.abs(got[m] - ext[m]) / np.abs(ext[m])) <= 2e-6


@pytest.mark.parametrize("fname", MOVE_EXP)
@pytest.mark.parametrize("alpha_kind", ["scalar", "1d", "nd"])
def test_move_exp_non_last_axis_bit_exact(fname, alpha_kind):
    shape, axis = (300, 32768), 0
    x = _data(shape, 33)
    y = _data(shape, 34) if fname in ("move_exp_nancov", "move_exp_nancorr") else None
    rng = np.random.default_rng(35)
    alpha = {"scalar": 0.07, "1d": rng.uniform(0.01, 0.5, size=shape[axis]),
             "nd": rng.uniform(0.01, 0.5, size=shape)}[alpha_kind]
    func = getattr(nb, fname)
    xt = torch.from_numpy(x).cuda()
    assert _host.column_layout(xt, axis) is not None
    args = (xt,) if y is None else (xt, torch.from_numpy(y).cuda())
    at = alpha if alpha_kind == "scalar" else (torch.from_numpy(alpha).cuda() if alpha_kind == "nd" else alpha)
    got = func(*args, alpha=at, min_weight=0.2, axis=axis).cpu().numpy()
    # the oracle takes a 1-D alpha along the axis the same way; an N-D one laid out like x
    want = oracle.move_exp(fname, x, y, alpha=alpha, min_weight=0.2, axis=axis)
    assert_bit_equal(got, want, f"{fname} alpha={alpha_kind}")


@pytest.mark.parametrize("fname", ["move_exp_nanmean", "move_exp_nanvar", "move_exp_nancorr"])
def test_move_exp_non_last_axis_float32_and_fp32c(fname):
    shape, axis = (200, 65536), 0  # float32 needs 65,536 columns for the in-place kernel
    x = _data(shape, 36)
    y = _data(shape, 37) if fname == "move_exp_nancorr" else None
    func = getattr(nb, fname)
    # float32 arrays with a float32 alpha array: numbagg's float32 loop, float64 locals
    x32 = x.astype(np.float32)
    y32 = None if y is None else y.astype(np.float32)
    al32 = np.full(shape[axis], 0.05, dtype=np.float32)
    got = func(x32, y32, alpha=al32, axis=axis) if y is not None else func(x32, alpha=al32, axis=axis)
    want = oracle.move_exp(fname, x32, y32, alpha=al32, axis=axis)
    assert_bit_equal(got, want, f"{fname} float32")
    # the compensated form: within its stated 2e-6 of the extended-precision result
    got = func(x, y, alpha=0.05, axis=axis, precision="fp32c") if y is not None else func(x, alpha=0.05, axis=axis, precision="fp32c")
    ext = oracle.move_exp(fname, x, y, alpha=0.05, axis=axis, ext=True)
    r = scaled_error(got, ext, exp_scale(fname, x, y, 0.05, axis=axis), exp_degenerate(fname, x, y, 0.05, 0.0, axis=axis))
    assert r["nan_mismatch"] == 0 and r["max_err"] <= 2e-6, r


def test_narrow_arrays_keep_the_copy_path():
    # too few columns to occupy the GPU: the axis is moved last and copied, same results
    x = _data((5000, 7), 38)
    xt = torch.from_numpy(x).cuda()
    assert _host.column_layout(xt, 0) is None
    assert_bit_equal(nb.ffill(xt, axis=0).cpu().numpy(), oracle.fill("ffill", x, axis=0), "narrow ffill")
    got = nb.move_exp_nanmean(xt, alpha=0.1, axis=0).cpu().numpy()
    want = oracle.move_exp("move_exp_nanmean", x, alpha=0.1, axis=0)
    assert np.array_equal(np.isnan(got), np.isnan(want))
    m = ~np.isnan(want)
    assert np.max(np.abs(got[m] - want[m]) / np.maximum(np.abs(want[m]), 1.0)) < 1e-12


def test_xarray_style_calls():
    # xarray's rolling_exp calls numbagg.move_exp_nanmean / nansum(array, axis=..., alpha=...,
    # min_weight=...) with the time axis anywhere; its ffill / bfill pass limit and axis
    rng = np.random.default_rng(39)
    da = rng.standard_normal((365, 128, 256))  # time, lat, lon: 32,768 columns, in place
    da[rng.random(da.shape) < 0.05] = np.nan
    for f in ("move_exp_nanmean", "move_exp_nansum", "move_exp_nanstd"):
        got = getattr(nb, f)(da, axis=0, alpha=0.2, min_weight=0.5)
        want = oracle.move_exp(f, da, alpha=0.2, min_weight=0.5, axis=0)
        assert got.shape == da.shape and isinstance(got, np.ndarray)
        assert_bit_equal(got, want, f)
    assert_bit_equal(nb.ffill(da, limit=2, axis=0), oracle.fill("ffill", da, limit=2, axis=0), "xarray ffill")
    assert_bit_equal(nb.bfill(da, axis=-3), oracle.fill("bfill", da, axis=0), "xarray bfill")


def test_flox_style_grouped_calls():
    # flox hands numbagg's grouped reductions an array whose trailing axes are the ones
    # reduced, integer codes laid out like them, num_labels and a tuple axis
    rng = np.random.default_rng(40)
    values = rng.standard_normal((6, 30, 50))
    values[rng.random(values.shape) < 0.1] = np.nan
    codes = rng.integers(-1, 12, size=(30, 50))
    for f in ("group_nansum", "group_nanmean", "group_nancount", "group_nanmax", "group_nanargmax", "group_nanvar"):
        got = getattr(nb, f)(values, codes, axis=(-2, -1), num_labels=12)
        want = oracle.group(f, values, codes, axis=(-2, -1), num_labels=12)
        assert got.shape == (6, 12)
        if f in ("group_nancount", "group_nanmax", "group_nanargmax"):
            assert_bit_equal(got, want, f)
        else:
            np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12, err_msg=f)


_GROUP_FUNCS = [
    "group_nansum", "group_nanmean", "group_nancount", "group_nanvar", "group_nanstd", "group_nansum_of_squares",
    "group_nanprod", "group_nanargmax", "group_nanargmin", "group_nanmax", "group_nanmin", "group_nanfirst",
    "group_nanlast", "group_nanany", "group_nanall",
]


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32, np.int64])
@pytest.mark.parametrize("fname", _GROUP_FUNCS)
def test_group_non_last_axes_bit_exact(fname, dtype):
    # values grouped over consecutive leading / middle axes: one thread per column runs
    # numbagg's loop in place, so every function's results are the reference's bit for
    # bit (float sums rounded per addition, integer sums and products wrapping)
    rng = np.random.default_rng(44)
    c = _host.column_min(np.dtype(dtype).itemsize)  # columns for the in-place kernel
    cases = [((64, c), 0, 12), ((2, 8, 4, c // 2), (1, 2), 7), ((2, 50, c // 2), 1, 30)]
    for shape, axis, K in cases:
        if np.issubdtype(dtype, np.floating):
            x = (rng.standard_normal(shape) * 3 + 1).astype(dtype)
            if fname == "group_nanprod":
                x = (1 + 0.01 * rng.standard_normal(shape)).astype(dtype)
            x[rng.random(shape) < 0.1] = np.nan
            x[rng.random(shape) < 0.05] = 0
        else:
            x = rng.integers(-40, 40, size=shape).astype(dtype)
        ax = (axis,) if isinstance(axis, int) else axis
        lshape = tuple(shape[a] for a in ax)
        labels = rng.integers(-1, K + 2, size=lshape)  # negative and >= num_labels skipped
        xt = torch.from_numpy(x).cuda()
        lt = torch.from_numpy(labels).cuda()
        assert nb.grouped.group_columns_layout(shape, ax, x.itemsize) is not None
        kw = {"ddof": 0} if fname in ("group_nanvar", "group_nanstd") else {}
        got = getattr(nb, fname)(xt, lt, axis=axis, num_labels=K, **kw).cpu().numpy()
        want = oracle.group(fname, x, labels, axis=axis, num_labels=K, **kw)
        assert got.shape == want.shape and got.dtype == want.dtype, (shape, axis, got.dtype, want.dtype)
        assert_bit_equal(got, want, f"{fname} {np.dtype(dtype)} {shape} axis={axis}")
    if dtype is not np.float64:
        return
    # more labels than the shared-memory bins hold: the moved-axis path, same values
    x = rng.standard_normal((200, 2048))
    labels = rng.integers(0, 3000, size=200)
    got = getattr(nb, fname)(x, labels, axis=0, num_labels=3000)
    want = oracle.group(fname, x, labels, axis=0, num_labels=3000)
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12, equal_nan=True)
