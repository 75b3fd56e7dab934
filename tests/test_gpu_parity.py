"""GPU results against the C oracle on seeded inputs at sizes where rows span many
tiles (so the look-back carries are exercised), across axes, dtypes and edge cases,
plus size-independent properties (causality / determinism) at larger sizes."""

import numpy as np
import pytest
import torch

import numbagg_gb300 as nb
import oracle
from tests.parity import (
    F32_TOL,
    F64_TOL,
    assert_bit_equal,
    assert_parity,
    assert_scaled_close,
    exp_degenerate,
    exp_scale,
    move_degenerate,
    move_scale,
)

pytestmark = pytest.mark.gpu

MOVE = ["move_sum", "move_mean", "move_var", "move_std", "move_cov", "move_corr"]
MOVE_EXP = [
    "move_exp_nancount",
    "move_exp_nanmean",
    "move_exp_nansum",
    "move_exp_nanvar",
    "move_exp_nanstd",
    "move_exp_nancov",
    "move_exp_nancorr",
]


def _data(shape, seed, p_nan=0.1, dtype=np.float64, normal=True):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(shape) if normal else rng.random(shape)
    x[rng.random(shape) < p_nan] = np.nan
    return x.astype(dtype)


@pytest.mark.parametrize("fname", MOVE)
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("window,min_count", [(1, None), (7, 3), (20, 20), (252, 100), (5000, 1)])
def test_move_vs_oracle(fname, dtype, window, min_count):
    x = _data((6, 40_000), 1, dtype=dtype)
    y = _data((6, 40_000), 2, dtype=dtype) if fname in ("move_cov", "move_corr") else None
    func = getattr(nb, fname)
    got = func(x, y, window=window, min_count=min_count) if y is not None else func(x, window=window, min_count=min_count)
    want = oracle.move(fname, x, y, window=window, min_count=min_count)
    ext = oracle.move(fname, x, y, window=window, min_count=min_count, ext=True)
    tol = F64_TOL if dtype == np.float64 else F32_TOL
    r = assert_parity(got, want, ext, move_scale(fname, x, y, window), tol, move_degenerate(fname, x, y, window), fname)
    # the exact sums make the GPU at least as close to the extended result as the reference
    if dtype == np.float64:
        assert r["gpu_vs_ext"] <= max(r["ref_vs_ext"], 1e-14), r


@pytest.mark.parametrize("fname", ["move_mean", "move_std", "move_corr"])
def test_move_axis_and_torch(fname):
    x = _data((300, 5, 7), 3)
    y = _data((300, 5, 7), 4)
    func = getattr(nb, fname)
    two = fname == "move_corr"
    for axis in (0, 1, -1):
        got = func(x, y, window=3, axis=axis) if two else func(x, window=3, axis=axis)
        want = oracle.move(fname, x, y if two else None, window=3, axis=axis)
        ext = oracle.move(fname, x, y if two else None, window=3, axis=axis, ext=True)
        assert_parity(got, want, ext, move_scale(fname, x, y, 3, axis), F64_TOL, move_degenerate(fname, x, y, 3, axis), f"{fname} axis={axis}")
    # torch CUDA tensors in, torch CUDA tensors out
    xt = torch.from_numpy(x).cuda()
    yt = torch.from_numpy(y).cuda()
    res = func(xt, yt, window=3, axis=0) if two else func(xt, window=3, axis=0)
    assert isinstance(res, torch.Tensor) and res.is_cuda
    want = oracle.move(fname, x, y if two else None, window=3, axis=0)
    ext = oracle.move(fname, x, y if two else None, window=3, axis=0, ext=True)
    assert_parity(res.cpu().numpy(), want, ext, move_scale(fname, x, y, 3, 0), F64_TOL, move_degenerate(fname, x, y, 3, 0), fname)


def test_move_edge_cases():
    # one element, window == n, all-NaN rows, int input promoted to float64
    one = np.array([3.0])
    assert nb.move_mean(one, window=1)[0] == 3.0
    x = _data((3, 17), 5)
    x[1] = np.nan
    for fname in ("move_sum", "move_mean", "move_var", "move_std"):
        got = getattr(nb, fname)(x, window=17, min_count=0)
        want = oracle.move(fname, x, window=17, min_count=0)
        ext = oracle.move(fname, x, window=17, min_count=0, ext=True)
        assert_parity(got, want, ext, move_scale(fname, x, None, 17), F64_TOL, None, fname)
    ints = np.arange(50, dtype=np.int64).reshape(5, 10)
    got = nb.move_sum(ints, window=3)
    assert got.dtype == np.float64
    np.testing.assert_array_equal(got, oracle.move("move_sum", ints.astype(np.float64), window=3))
    empty = np.zeros((0, 10))
    assert nb.move_mean(empty, window=3).shape == (0, 10)


def test_move_float32_exact_tiles():
    # numbagg/test/test_moving.py:186-192
    rs = np.random.RandomState(0)
    arr = np.tile((rs.rand(10) * 1e13).astype(np.float32), 100)
    res = nb.move_sum(arr, window=10)
    assert res[-1] == np.sum(arr[:10])
    # numbagg/test/test_moving.py:180-183
    arr = (rs.random(1000) * 1e13).astype(np.float32)
    np.testing.assert_allclose(nb.move_mean(arr, window=1), arr)


@pytest.mark.parametrize("fname", MOVE_EXP)
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("alpha,min_weight", [(0.5, 0.0), (0.01, 0.0), (1e-4, 0.5), (0.9, 0.3)])
def test_move_exp_vs_oracle(fname, dtype, alpha, min_weight):
    x = _data((5, 30_000), 6, normal=False, dtype=dtype)
    y = _data((5, 30_000), 7, normal=False, dtype=dtype) if fname in ("move_exp_nancov", "move_exp_nancorr") else None
    func = getattr(nb, fname)
    if dtype == np.float32:
        # a float32 alpha array selects numbagg's float32 loop; a Python float alpha
        # is broadcast to a float64 array and selects the float64 loop
        wide = func(x, y, alpha=alpha, min_weight=min_weight) if y is not None else func(x, alpha=alpha, min_weight=min_weight)
        assert wide.dtype == np.float64
        x64 = x.astype(np.float64)
        y64 = None if y is None else y.astype(np.float64)
        ref64 = func(x64, y64, alpha=alpha, min_weight=min_weight) if y is not None else func(x64, alpha=alpha, min_weight=min_weight)
        assert_bit_equal(wide, ref64, f"{fname} float32 input, float64 loop")
        alpha = np.full(x.shape[-1], alpha, dtype=np.float32)
    got = func(x, y, alpha=alpha, min_weight=min_weight) if y is not None else func(x, alpha=alpha, min_weight=min_weight)
    want = oracle.move_exp(fname, x, y, alpha=alpha, min_weight=min_weight)
    ext = oracle.move_exp(fname, x, y, alpha=alpha, min_weight=min_weight, ext=True)
    tol = F64_TOL if dtype == np.float64 else F32_TOL
    allow = exp_degenerate(fname, x, y, alpha, min_weight)
    r = assert_parity(got, want, ext, exp_scale(fname, x, y, alpha), tol, allow, fname)
    assert r["allowed"] <= 0.001 * r["n"] + 20


@pytest.mark.parametrize("fname", MOVE_EXP)
@pytest.mark.parametrize("alpha,min_weight", [(0.5, 0.0), (0.9, 0.3), (0.01, 0.0)])
def test_move_exp_one_pass_vs_oracle(fname, alpha, min_weight):
    # 40 rows: a scalar alpha over this many rows takes the one-pass scan (tiles chained
    # row by row), fewer rows the three-phase one
    x = _data((40, 20_000), 16, normal=False)
    y = _data((40, 20_000), 17, normal=False) if fname in ("move_exp_nancov", "move_exp_nancorr") else None
    func = getattr(nb, fname)
    got = func(x, y, alpha=alpha, min_weight=min_weight) if y is not None else func(x, alpha=alpha, min_weight=min_weight)
    want = oracle.move_exp(fname, x, y, alpha=alpha, min_weight=min_weight)
    ext = oracle.move_exp(fname, x, y, alpha=alpha, min_weight=min_weight, ext=True)
    allow = exp_degenerate(fname, x, y, alpha, min_weight)
    r = assert_parity(got, want, ext, exp_scale(fname, x, y, alpha), F64_TOL, allow, fname)
    assert r["allowed"] <= 0.001 * r["n"] + 50


@pytest.mark.parametrize("fname", ["move_exp_nanmean", "move_exp_nanvar", "move_exp_nancorr"])
def test_move_exp_alpha_forms(fname):
    # numbagg/test/test_moving_exp.py:348-368: scalar, 1-D and N-D alpha agree
    x = _data((4, 3000), 8, normal=False)
    y = _data((4, 3000), 9, normal=False)
    two = fname == "move_exp_nancorr"
    func = getattr(nb, fname)
    alphas = np.linspace(0.01, 0.6, 3000)
    got1 = func(x, y, alpha=alphas) if two else func(x, alpha=alphas)
    want1 = oracle.move_exp(fname, x, y if two else None, alpha=alphas)
    ext1 = oracle.move_exp(fname, x, y if two else None, alpha=alphas, ext=True)
    assert_parity(got1, want1, ext1, exp_scale(fname, x, y, alphas), F64_TOL, exp_degenerate(fname, x, y, alphas, 0.0), fname)
    full = np.broadcast_to(alphas, x.shape).copy()
    got2 = func(x, y, alpha=full) if two else func(x, alpha=full)
    assert_bit_equal(got2, got1, "N-D alpha vs 1-D alpha")
    gotT = func(x.T, y.T, alpha=alphas, axis=0) if two else func(x.T, alpha=alphas, axis=0)
    assert_bit_equal(np.ascontiguousarray(gotT.T), got1, "axis=0 vs axis=-1")


def test_move_exp_known_answers():
    # numbagg/test/test_moving_exp.py:111-157, :239-295, :335-345
    a = np.array([1, 0, np.nan, np.nan, 1, 0])
    np.testing.assert_allclose(nb.move_exp_nancount(a, alpha=0.5), [1.0, 1.5, 0.75, 0.375, 1.1875, 1.59375])
    a = np.array([10, 0, np.nan, 10])
    np.testing.assert_allclose(nb.move_exp_nanmean(a, alpha=0.5), [10.0, 3.3333333, 3.3333333, 8.1818182], rtol=1e-7)
    np.testing.assert_allclose(nb.move_exp_nansum(a, alpha=0.25), [10.0, 7.5, 5.625, 14.21875])
    r = nb.move_exp_nancorr(np.array([10, 0, 5, 10.0]), np.array([10, 0, 10, 5.0]), alpha=0.5)
    np.testing.assert_allclose(r, [np.nan, 1.0, 0.8485281, 0.2274294], rtol=1e-6)
    allnan = np.array([np.nan] * 4)
    np.testing.assert_array_equal(nb.move_exp_nancount(allnan, alpha=0.5), [0.0] * 4)
    assert np.all(np.isnan(nb.move_exp_nansum(allnan, alpha=0.5)))
    np.testing.assert_array_equal(nb.move_exp_nanmean(np.array([np.inf]), alpha=0.25), [np.inf])
    np.testing.assert_array_equal(nb.move_exp_nanmean(np.array([[0, np.nan]]), alpha=1.0), [[0, np.nan]])
    big = np.array([[0.0, 1.19846209e308], [1.19846209e308, 1.19846209e308]])
    np.testing.assert_array_equal(nb.move_exp_nanmean(big, alpha=1.0), big)


@pytest.mark.parametrize("func_n", [("move_exp_nanvar", 1), ("move_exp_nanstd", 1), ("move_exp_nancov", 2), ("move_exp_nancorr", 2)])
@pytest.mark.parametrize("alpha", [0.1, 0.5, 0.9])
def test_move_exp_nans_var(func_n, alpha):
    # numbagg/test/test_moving_exp.py:160-236: NaN placement of the variance family
    fname, n = func_n
    func = getattr(nb, fname)
    cases = [
        ([np.nan, np.nan], [True, True]),
        ([5.0, np.nan], [True, True]),
        ([1.0, np.nan, 2.0], [True, True, False]),
        ([1.0, np.nan], [True, True]),
        ([0.9, np.nan], [True, True]),
        ([0.95, np.nan, 1.0], [True, True, False]),
        ([0.59288027, np.nan, 0.4758262, 0.70877039], [True, True, False, False]),
    ]
    for arr, expected in cases:
        a = np.array(arr)
        res = np.isnan(func(*[a] * n, alpha=alpha))
        np.testing.assert_array_equal(res, expected, err_msg=f"{fname} {arr}")
    a = np.array([1.0, np.nan, 1.0])
    expected = [True, True, True] if fname == "move_exp_nancorr" else [True, True, False]
    np.testing.assert_array_equal(np.isnan(func(*[a] * n, alpha=alpha)), expected)


@pytest.mark.parametrize("fname", ["move_exp_nancount", "move_exp_nanmean", "move_exp_nanstd", "move_exp_nansum", "move_exp_nanvar"])
def test_move_exp_min_weight(fname):
    # numbagg/test/test_moving_exp.py:34-79
    func = getattr(nb, fname)
    array = np.ones(25)
    array[:5] = np.nan
    for mw, alpha, expected in [
        (0.0, 0.2, 19), (0.0, 0.8, 19), (0.5, 0.2, 17), (0.5, 0.8, 19),
        (0.9, 0.2, 10), (0.9, 0.8, 19), (1.0, 0.2, 0), (1.0, 0.8, 0),
    ]:
        assert np.sum(~np.isnan(func(array, min_weight=mw, alpha=alpha))[6:]) == expected, (mw, alpha)


# n = 100,003: odd rows, so every other row starts off a 16-byte boundary; n = 100,000:
# aligned rows with a partial last tile; n = 57,344: whole 4,096-position tiles only
@pytest.mark.parametrize("n", [100_003, 100_000, 57_344])
@pytest.mark.parametrize("fname", ["ffill", "bfill"])
@pytest.mark.parametrize("limit", [None, 0, 1, 5, 10_000])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_fill_vs_oracle(fname, limit, dtype, n):
    rng = np.random.default_rng(10)
    x = rng.standard_normal((5, n)).astype(dtype)
    x[rng.random(x.shape) < 0.3] = np.nan
    x[2, 1000:60_000] = np.nan  # runs across many tiles
    x[3] = np.nan
    x[4, :50_000] = np.nan
    got = getattr(nb, fname)(x, limit=limit)
    assert_bit_equal(got, oracle.fill(fname, x, limit=limit), f"{fname} limit={limit}")


def test_fill_int_and_axes():
    ints = np.random.default_rng(11).integers(-1000, 1000, size=(7, 33)).astype(np.int32)
    assert_bit_equal(nb.ffill(ints), ints, "int32 ffill")
    i64 = ints.astype(np.int64) * (1 << 40)
    assert_bit_equal(nb.bfill(i64), oracle.fill("bfill", i64), "int64 bfill")
    x = _data((40, 3, 9), 12, p_nan=0.4)
    for axis in (0, 1, 2):
        assert_bit_equal(nb.ffill(x, limit=2, axis=axis), oracle.fill("ffill", x, limit=2, axis=axis), f"axis {axis}")


GROUP_EXACT = ["group_nancount", "group_nanargmax", "group_nanargmin", "group_nanmax", "group_nanmin",
               "group_nanfirst", "group_nanlast", "group_nanany", "group_nanall"]
GROUP_FLOAT = ["group_nansum", "group_nanmean", "group_nanvar", "group_nanstd", "group_nansum_of_squares"]


@pytest.mark.parametrize("K", [16, 300, 4096, 70_000])
@pytest.mark.parametrize("fname", GROUP_EXACT + GROUP_FLOAT)
def test_group_vs_oracle(fname, K):
    rng = np.random.default_rng(13)
    m = 200_000
    values = rng.standard_normal((3, m))
    values[rng.random(values.shape) < 0.05] = np.nan
    values[:, :10] = np.round(values[:, :10])  # ties for the selection functions
    labels = rng.integers(-1, K, size=m).astype(np.int32)
    got = getattr(nb, fname)(values, labels, num_labels=K, axis=-1)
    want = oracle.group(fname, values, labels, num_labels=K, axis=-1)
    if fname in GROUP_EXACT:
        assert_bit_equal(got, want, fname)
    else:
        absv = np.where(np.isnan(values), 0.0, np.abs(values))
        lab = np.where(labels >= 0, labels, K)
        s1 = np.stack([np.bincount(lab, weights=absv[r], minlength=K + 1)[:K] for r in range(3)])
        s2 = np.stack([np.bincount(lab, weights=absv[r] ** 2, minlength=K + 1)[:K] for r in range(3)])
        cnt = np.stack([np.bincount(lab, weights=(~np.isnan(values[r])).astype(float), minlength=K + 1)[:K] for r in range(3)])
        scale = {
            "group_nansum": s1,
            "group_nanmean": s1 / np.maximum(cnt, 1),
            "group_nanvar": s2 / np.maximum(cnt, 1),
            "group_nanstd": np.sqrt(s2 / np.maximum(cnt, 1)),
            "group_nansum_of_squares": s2,
        }[fname]
        assert_scaled_close(got, want, scale, F64_TOL, None, fname)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("fname", ["group_nansum", "group_nanmean", "group_nanvar", "group_nansum_of_squares"])
def test_group_few_labels_infinities(fname, dtype):
    # K <= 16 (lane-private bins): a lane's elements alternate between its fixed-point
    # and (for sums and means) float64 bins, so infinities land at every position of a
    # tile; label 0 holds +inf, label 1 -inf, label 2 both (NaN), the rest finite
    rng = np.random.default_rng(16)
    m, K = 300_000, 8
    values = rng.standard_normal((4, m)).astype(dtype)
    values[rng.random(values.shape) < 0.05] = np.nan
    labels = rng.integers(0, K, size=m).astype(np.int32)
    cols0 = np.flatnonzero(labels == 0)[:40]
    cols1 = np.flatnonzero(labels == 1)[:40]
    cols2 = np.flatnonzero(labels == 2)[:40]
    values[:, cols0[::3]] = np.inf
    values[:, cols1[1::3]] = -np.inf
    values[:, cols2[::5]] = np.inf
    values[:, cols2[2::5]] = -np.inf
    got = getattr(nb, fname)(values, labels, num_labels=K, axis=-1)
    want = oracle.group(fname, values, labels, num_labels=K, axis=-1)
    assert np.array_equal(np.isnan(got), np.isnan(want)), fname
    assert np.array_equal(np.isposinf(got), np.isposinf(want)) and np.array_equal(np.isneginf(got), np.isneginf(want))
    fin = np.isfinite(want)
    v64 = np.where(np.isfinite(values), values, 0.0).astype(np.float64)
    s1 = np.stack([np.bincount(labels, weights=np.abs(v64[r]), minlength=K) for r in range(4)])
    s2 = np.stack([np.bincount(labels, weights=v64[r] ** 2, minlength=K) for r in range(4)])
    cnt = np.stack([np.bincount(labels, weights=(~np.isnan(values[r])).astype(float), minlength=K) for r in range(4)])
    scale = {"group_nansum": s1, "group_nanmean": s1 / np.maximum(cnt, 1), "group_nanvar": s2 / np.maximum(cnt, 1),
             "group_nansum_of_squares": s2}[fname]
    # float32: the reference accumulates in float32 over ~37,000 terms per group
    tol = 1e-4 if dtype == np.float32 else F64_TOL
    assert_scaled_close(got[fin], want[fin], scale[fin], tol, None, f"{fname} {np.dtype(dtype)}")


@pytest.mark.parametrize("dtype", [np.int32, np.int64, np.float32, np.bool_])
@pytest.mark.parametrize("fname", [f.__name__ for f in nb.GROUPED_FUNCS])
def test_group_dtypes(fname, dtype):
    rng = np.random.default_rng(14)
    func = getattr(nb, fname)
    if dtype == np.bool_:
        values = rng.random((2, 5000)) < 0.5
        if not func.supports_bool:
            return
    elif np.issubdtype(dtype, np.integer):
        values = rng.integers(-100, 100, size=(2, 5000)).astype(dtype)
    else:
        values = rng.standard_normal((2, 5000)).astype(dtype)
        values[rng.random(values.shape) < 0.1] = np.nan
    labels = rng.integers(-1, 12, size=5000)
    got = func(values, labels, axis=-1)
    want = oracle.group(fname, values, labels, axis=-1)
    assert got.dtype == want.dtype, (got.dtype, want.dtype)
    if want.dtype.kind in "iu" or fname in GROUP_EXACT:
        if fname == "group_nanfirst" and want.dtype.kind == "i":
            want = want.copy()
        assert_bit_equal(got, want, f"{fname} {dtype}")
    else:
        tol = 1e-5 if want.dtype == np.float32 else F64_TOL
        scale = np.nanmax(np.abs(want), axis=-1, keepdims=True) * np.ones_like(want)
        if fname == "group_nanprod":
            scale = np.abs(want)
        assert_scaled_close(got, want, scale, tol, None, f"{fname} {dtype}")


def test_group_axis_modes():
    # numbagg/test/test_grouped.py:476-590
    values = np.arange(24.0).reshape(2, 3, 4)
    labels = np.array([[0, 0, 1, 1], [0, 1, 1, 2], [2, 2, 2, 2]])
    np.testing.assert_allclose(nb.group_nanargmax(values, labels, axis=(1, 2))[0], [4.0, 6.0, 11.0])
    np.testing.assert_allclose(nb.group_nanargmin(values, labels, axis=(1, 2))[0], [0.0, 2.0, 7.0])
    v2 = np.array([[1.0, 5.0, 3.0], [2.0, 4.0, 6.0]])
    l2 = np.array([[0, 0, 1], [1, 2, 2]])
    np.testing.assert_allclose(nb.group_nanargmax(v2, l2), [1.0, 2.0, 5.0])
    np.testing.assert_allclose(nb.group_nanargmin(v2, l2), [0.0, 3.0, 4.0])
    values2d = np.arange(25.0).reshape(5, 5)
    lab = np.arange(5)
    np.testing.assert_allclose(nb.group_nansum(values2d, lab, axis=1), values2d)
    np.testing.assert_allclose(nb.group_nansum(values2d, lab, axis=0), values2d.T)
    np.testing.assert_allclose(
        nb.group_nansum(values2d, [0, 0, -1, 1, 1], axis=1),
        np.stack([values2d[:, :2].sum(1), values2d[:, 3:].sum(1)], -1),
    )
    assert nb.group_nansum(np.arange(24).reshape(6, 4).reshape(1, 6, 2, 2), np.arange(4).reshape(2, 2), axis=(-1, -2)).shape == (1, 6, 4)
    np.testing.assert_allclose(nb.group_nanmean(np.array([True, True, False]), np.array([0, 0, 0])), [2 / 3])
    # empty groups
    np.testing.assert_equal(nb.group_nansum(np.array([np.nan] * 3), np.array([0, 1, 2])), [0.0] * 3)
    np.testing.assert_equal(nb.group_nanprod(np.array([np.nan] * 3), np.array([0, 1, 2])), [1.0] * 3)
    assert np.all(np.isnan(nb.group_nanargmin(np.array([np.nan] * 3), np.array([0, 1, 2]))))


def test_group_signed_zero_first_wins():
    # nanmax keeps the first of equal values (numbagg/grouped.py:239-242)
    v = np.array([-0.0, 0.0, -0.0])
    lab = np.array([0, 0, 1])
    got = nb.group_nanmax(v, lab)
    want = oracle.group("group_nanmax", v, lab)
    assert_bit_equal(got, want, "signed zero")
    assert np.signbit(got[0])


@pytest.mark.parametrize("fname", ["move_covmatrix", "move_corrmatrix"])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_move_matrix_vs_oracle(fname, dtype):
    rng = np.random.default_rng(15)
    a = rng.standard_normal((2, 700, 37)).astype(dtype)
    a[rng.random(a.shape) < 0.05] = np.nan
    for window, mc in [(50, 40), (7, None), (700, 1)]:
        got = getattr(nb, fname)(a, window=window, min_count=mc)
        # the reference accumulates in the input dtype (numbagg/moving_matrix.py:149-152):
        # float32 input is compared with the float32 restatement
        want = oracle.move_matrix(fname, a, window=window, min_count=mc)
        ext = oracle.move_matrix(fname, a.astype(np.float64), window=window, min_count=mc, ext=True)
        # float32: accumulators are float32 in the reference and here, with different
        # rounding paths (segments are re-seeded here); the reference's own error on this
        # data reaches 7e-5 of the scale, so the bar is 1e-4 of the scale
        tol = F64_TOL if dtype == np.float64 else 1e-4
        if fname == "move_covmatrix":
            scale = np.sqrt(np.abs(np.einsum("...ii->...i", np.nan_to_num(want)))[..., :, None] * np.abs(np.einsum("...ii->...i", np.nan_to_num(want)))[..., None, :]) + 1e-300
        else:
            scale = np.ones_like(want)
        assert_parity(got, want, ext, scale, tol, None, f"{fname} w={window}")


def test_move_matrix_known_answers():
    # numbagg/test/test_matrix_functions.py:202-286
    data = np.array([[1, 2], [2, 4], [3, 6], [4, 8], [5, 10], [6, 12]], dtype=np.float64)
    r = nb.move_corrmatrix(data, window=3, min_count=2)
    for i in range(1, 6):
        np.testing.assert_allclose(r[i], [[1.0, 1.0], [1.0, 1.0]], rtol=1e-10)
    data = np.array([[1, 2], [1, 2], [1, 2], [2, 3], [3, 4], [4, 5]], dtype=np.float64)
    cov = nb.move_covmatrix(data, window=3, min_count=2)
    assert cov[2, 0, 0] == 0.0 and cov[2, 1, 1] == 0.0 and cov[2, 0, 1] == 0.0
    assert np.isnan(nb.move_corrmatrix(data, window=3, min_count=2)[2, 0, 1])


# ---- size-independent properties at larger sizes ------------------------------------------


@pytest.mark.parametrize("fname", ["move_mean", "move_std", "move_exp_nanvar", "ffill"])
@pytest.mark.parametrize("rows", [4, 64])
def test_prefix_causality_bit_exact(fname, rows):
    """A prefix of a longer input gives bit-identical results
    (numbagg/test/test_property.py:86-150); 64 rows take the one-pass EWM scan."""
    x = torch.randn(rows, 3_000_001 if rows == 4 else 400_001, dtype=torch.float64, device="cuda")
    x[torch.rand_like(x) < 0.05] = float("nan")
    func = getattr(nb, fname)
    kw = {"window": 20} if fname.startswith("move_") and "exp" not in fname else {}
    if "exp" in fname:
        kw = {"alpha": 0.01}
    cut = 2_000_000 if rows == 4 else 250_000
    full = func(x, **kw)
    part = func(x[:, :cut].contiguous(), **kw)
    again = func(x, **kw)
    assert torch.equal(torch.isnan(full[:, :cut]), torch.isnan(part))
    m = ~torch.isnan(part)
    assert torch.equal(full[:, :cut][m], part[m])
    assert torch.equal(torch.nan_to_num(full, nan=7.0), torch.nan_to_num(again, nan=7.0))  # run to run


@pytest.fixture
def deterministic_algorithms():
    torch.use_deterministic_algorithms(True)
    try:
        yield
    finally:
        torch.use_deterministic_algorithms(False)


@pytest.mark.parametrize("fname", ["group_nansum", "group_nanmean", "group_nanvar", "group_nansum_of_squares"])
def test_group_deterministic_mode(fname, deterministic_algorithms):
    # torch.use_deterministic_algorithms(True) routes float moments with a few thousand
    # labels to the exact fixed-point shared-memory kernels: same bits on every run
    rng = np.random.default_rng(21)
    values = rng.standard_normal((6, 300_001))
    values[rng.random(values.shape) < 0.05] = np.nan
    values[2, 17] = np.inf
    labels = rng.integers(-1, 3000, size=300_001)
    x = torch.from_numpy(values).cuda()
    lab = torch.from_numpy(labels).cuda()
    func = getattr(nb, fname)
    a = func(x, lab, num_labels=3000, axis=-1)
    b = func(x, lab, num_labels=3000, axis=-1)
    assert torch.equal(torch.nan_to_num(a, nan=7.0), torch.nan_to_num(b, nan=7.0))
    want = oracle.group(fname, values, labels, num_labels=3000, axis=-1)
    scale = np.nanmax(np.abs(np.where(np.isinf(want), np.nan, want)), axis=-1, keepdims=True) * np.ones_like(want)
    assert_scaled_close(a.cpu().numpy(), want, scale, F64_TOL, None, fname)


def test_group_deterministic_mode_refuses_atomic_sums(deterministic_algorithms):
    x = torch.randn(2, 50_000, dtype=torch.float64, device="cuda")
    lab = torch.randint(0, 40_000, (50_000,), device="cuda")
    with pytest.raises(RuntimeError, match="deterministic"):
        nb.group_nanmean(x, lab, num_labels=40_000, axis=-1)
    # counts and selections are exact on every path
    got = nb.group_nancount(x, lab, num_labels=40_000, axis=-1).cpu().numpy()
    want = oracle.group("group_nancount", x.cpu().numpy(), lab.cpu().numpy(), num_labels=40_000, axis=-1)
    assert_bit_equal(got, want, "count")


def test_determinism_large():
    x = torch.randn(8, 2_000_000, dtype=torch.float64, device="cuda")
    x[torch.rand_like(x) < 0.05] = float("nan")
    lab = torch.randint(0, 16, (2_000_000,), device="cuda", dtype=torch.int32)
    for fn in (
        lambda: nb.move_var(x, window=100),
        lambda: nb.bfill(x, limit=5),
        lambda: nb.move_exp_nanmean(x, alpha=0.05),
        lambda: nb.group_nansum(x, lab, num_labels=16, axis=-1),
        lambda: nb.group_nanargmax(x, lab, num_labels=16, axis=-1),
    ):
        a, b = fn(), fn()
        assert torch.equal(torch.nan_to_num(a, nan=123.0), torch.nan_to_num(b, nan=123.0))
