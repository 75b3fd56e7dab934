"""Static aggregations on the GPU against the oracle (numbagg/funcs.py:23-242).

Exact for counts, NaN flags, extremes and their indices and integer sums; float sums,
means and the two-pass variance within 1e-12 (float64) / 2e-6 (float32) of the
long-double oracle, relative to the sum of magnitudes (sums, means) or to the result
(variance), which bounds the reference's own float64 rounding as well.
"""

import warnings

import numpy as np
import pytest
import torch

import numbagg_gb300 as nb
import oracle

pytestmark = pytest.mark.gpu

EXACT = ["allnan", "anynan", "nancount", "nanmax", "nanmin", "nanargmax", "nanargmin"]
AXES = [None, -1, 0, 1, (0, 2), (2, 0), (-1, -2)]


def _data(dtype, seed=11, shape=(6, 5, 3001), p=0.15):
    rng = np.random.default_rng(seed)
    if np.issubdtype(dtype, np.integer):
        return rng.integers(-1000, 1000, size=shape).astype(dtype)
    a = rng.standard_normal(shape) * 10.0 + 3.0
    a[rng.random(shape) < p] = np.nan
    a[0, 0, :] = np.nan  # an all-NaN slice along the last axis
    a[1, 2, 7] = np.inf
    a[2, 3, 11] = -np.inf
    a[3, 1, 5] = -0.0
    return a.astype(dtype)


def _ok_axis(name, a, axis):
    """argmax/argmin raise on an all-NaN slice; both sides are checked to agree."""
    try:
        return oracle.aggregate(name, a, axis=axis), None
    except ValueError as err:
        return None, str(err)


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32, np.int64])
@pytest.mark.parametrize("name", EXACT)
def test_exact_functions(name, dtype):
    warnings.simplefilter("ignore")
    a = _data(dtype)
    for axis in AXES:
        want, err = _ok_axis(name, a, axis)
        if err is not None:
            with pytest.raises(ValueError, match="All-NaN slice encountered"):
                getattr(nb, name)(a, axis=axis)
            continue
        got = getattr(nb, name)(a, axis=axis)
        assert np.asarray(got).dtype == np.asarray(want).dtype, (name, axis)
        np.testing.assert_array_equal(got, want, err_msg=f"{name} axis={axis}")


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("name", ["nansum", "nanmean"])
def test_sums_and_means(name, dtype):
    warnings.simplefilter("ignore")
    a = _data(dtype)
    a[np.isinf(a)] = 1.0  # finite data: the bound is relative to the sum of magnitudes
    tol = 1e-12 if dtype == np.float64 else 2e-6
    for axis in AXES:
        got = np.asarray(getattr(nb, name)(a, axis=axis), dtype=np.float64)
        ext = np.asarray(oracle.aggregate(name, a, axis=axis, ext=True), dtype=np.float64)
        mag = np.asarray(oracle.aggregate(name, np.abs(a), axis=axis, ext=True), dtype=np.float64)
        assert np.array_equal(np.isnan(got), np.isnan(ext)), (name, axis)
        err = np.abs(got - ext)[~np.isnan(ext)] / np.maximum(mag[~np.isnan(ext)], 1e-300)
        assert err.max(initial=0.0) <= tol, (name, axis, err.max())


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("name", ["nanvar", "nanstd"])
@pytest.mark.parametrize("ddof", [0, 1, 5])
def test_two_pass_variance(name, dtype, ddof):
    warnings.simplefilter("ignore")
    a = _data(dtype)
    a[np.isinf(a)] = 2.0
    a = a + np.asarray(1e6, dtype)  # a large offset: the two-pass form keeps the digits
    tol = 1e-10 if dtype == np.float64 else 2e-5
    for axis in AXES:
        got = np.asarray(getattr(nb, name)(a, ddof=ddof, axis=axis), dtype=np.float64)
        ext = np.asarray(oracle.aggregate(name, a, axis=axis, ddof=ddof, ext=True), dtype=np.float64)
        assert np.array_equal(np.isnan(got), np.isnan(ext)), (name, axis)
        ok = ~np.isnan(ext)
        err = np.abs(got - ext)[ok] / np.maximum(np.abs(ext[ok]), 1e-300)
        assert err.max(initial=0.0) <= tol, (name, axis, ddof, err.max())


def test_infinities_in_sums_and_variance():
    a = np.array([[1.0, np.inf, 2.0], [1.0, np.inf, -np.inf], [np.nan, -np.inf, 3.0]])
    np.testing.assert_array_equal(nb.nansum(a, axis=1), [np.inf, np.nan, -np.inf])
    np.testing.assert_array_equal(np.isnan(nb.nanvar(a, axis=1)), [True, True, True])
    np.testing.assert_array_equal(nb.nanmax(a, axis=1), [np.inf, np.inf, 3.0])
    np.testing.assert_array_equal(nb.nanargmin(a, axis=1), [0, 2, 1])


def test_integer_sum_wraps_like_the_int32_loop():
    a = np.full((3, 4), 2**30, dtype=np.int32)
    np.testing.assert_array_equal(nb.nansum(a, axis=1), oracle.aggregate("nansum", a, axis=1))
    assert nb.nansum(a, axis=1).dtype == np.int32


def test_dtype_casting_matches_the_reference_loops():
    assert nb.nansum(np.ones(5, np.int16)).dtype == np.int32
    assert nb.nansum(np.ones(5, np.float16)).dtype == np.float32
    assert nb.nanmean(np.arange(5, dtype=np.int64)).dtype == np.float64
    assert nb.nancount(np.ones((2, 3)), axis=1).dtype == np.int64
    assert nb.allnan(np.ones((2, 3)), axis=1).dtype == np.bool_
    b = np.array([[True, False], [True, True]])
    np.testing.assert_array_equal(nb.nansum(b, axis=1), [1, 2])


def test_scalar_and_tensor_results():
    a = np.array([1.0, np.nan, 3.0])
    r = nb.nanmean(a)
    assert isinstance(r, np.generic) and r == 2.0
    assert nb.nanargmax(a) == 2
    t = torch.tensor([[1.0, np.nan], [5.0, 2.0]], dtype=torch.float64, device="cuda")
    rt = nb.nanmax(t, axis=1)
    assert rt.is_cuda and torch.equal(rt.cpu(), torch.tensor([1.0, 5.0], dtype=torch.float64))


def test_all_nan_slices():
    a = np.full((2, 4), np.nan)
    a[1, 2] = 5.0
    np.testing.assert_array_equal(nb.allnan(a, axis=1), [True, False])
    np.testing.assert_array_equal(nb.anynan(a, axis=1), [True, True])
    np.testing.assert_array_equal(nb.nancount(a, axis=1), [0, 1])
    np.testing.assert_array_equal(nb.nansum(a, axis=1), [0.0, 5.0])
    assert np.isnan(nb.nanmean(a, axis=1)[0]) and np.isnan(nb.nanmax(a, axis=1)[0])
    with pytest.raises(ValueError, match="All-NaN slice encountered"):
        nb.nanargmax(a, axis=1)


def test_empty_rows_and_zero_length_axes():
    a = np.empty((0, 5))
    assert nb.nansum(a, axis=1).shape == (0,)
    b = np.empty((3, 0))
    np.testing.assert_array_equal(nb.nansum(b, axis=1), [0.0, 0.0, 0.0])
    np.testing.assert_array_equal(nb.allnan(b, axis=1), [True, True, True])
    np.testing.assert_array_equal(nb.anynan(b, axis=1), [False, False, False])
    assert np.isnan(nb.nanmean(b, axis=1)).all()


def test_large_row_sum_and_determinism():
    rng = np.random.default_rng(3)
    a = rng.standard_normal((4, 3_000_017))
    a[rng.random(a.shape) < 0.05] = np.nan
    got = nb.nansum(a, axis=1)
    again = nb.nansum(a, axis=1)
    np.testing.assert_array_equal(got, again)
    ext = oracle.aggregate("nansum", a, axis=1, ext=True)
    mag = oracle.aggregate("nansum", np.abs(a), axis=1, ext=True)
    assert (np.abs(got - ext) / mag).max() <= 1e-12
    np.testing.assert_array_equal(nb.nanargmax(a, axis=1), oracle.aggregate("nanargmax", a, axis=1))


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int64])
def test_middle_axes_in_place(dtype):
    # consecutive reduced axes that are not last run in place through their stride
    # (one warp of consecutive outputs per CTA, chunks of the reduced extent)
    warnings.simplefilter("ignore")
    a = _data(dtype, seed=12, shape=(4, 40, 50, 64))
    for name in EXACT + ["nansum"]:
        for axis in ((1, 2), 0, (0, 1, 2)):
            want, err = _ok_axis(name, a, axis)
            if err is not None:
                continue
            got = getattr(nb, name)(a, axis=axis)
            if name == "nansum" and dtype != np.int64:
                mag = oracle.aggregate(name, np.abs(np.nan_to_num(a, posinf=0, neginf=0)), axis=axis)
                mag = np.asarray(mag, dtype=np.float64)
                g64, w64 = np.asarray(got, dtype=np.float64), np.asarray(want, dtype=np.float64)
                ok = np.isfinite(w64)
                assert np.array_equal(g64[~ok], w64[~ok], equal_nan=True)
                err = np.abs(g64 - w64)[ok] / np.maximum(mag[ok], 1e-300)
                assert err.max(initial=0.0) <= (1e-12 if dtype == np.float64 else 2e-6), (axis, err.max(initial=0.0))
            else:
                np.testing.assert_array_equal(got, want, err_msg=f"{name} axis={axis}")
    # a long reduced axis over few outputs: many chunks per warp of outputs
    rng = np.random.default_rng(13)
    b = rng.standard_normal((400_000, 64))
    b[rng.random(b.shape) < 0.05] = np.nan
    for name in ("nanmean", "nanvar"):
        got = getattr(nb, name)(b, axis=0)
        ext = oracle.aggregate(name, b, axis=0, ext=True)
        assert (np.abs(got - ext) / np.abs(ext)).max() <= 1e-12, name
    np.testing.assert_array_equal(nb.nanargmin(b, axis=0), oracle.aggregate("nanargmin", b, axis=0))
