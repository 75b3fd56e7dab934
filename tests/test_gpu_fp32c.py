"""The FP32-compensated ("fp32c") forms against the extended-precision oracle.

``precision="fp32c"`` (an extension of numbagg's signatures) computes the float64
moving-window and exponentially weighted functions on the FP32 pipes: double-float
window sums and a double-float EWM scan, the shift-invariant statistics taken on
pivoted values; rows outside the double-float range fall back to exact window sums.  The stated bound is a relative
error of at most 2e-6 against a well-conditioned float64 oracle, here the long-double
restatement of numbagg's loops (oracle ``ext=True``), on ordinary data and on the
precision-stress data 1e6 + N(0, 1) with correlation 0.7 and 2% NaN.  Errors are
relative to the same per-output scales as the plain-form parity tests.
"""

import numpy as np
import pytest

import numbagg_gb300 as nb
import oracle
from tests.parity import exp_degenerate, exp_scale, move_degenerate, move_scale, scaled_error

pytestmark = pytest.mark.gpu

FP32C_TOL = 2e-6
MOVE = ["move_sum", "move_mean", "move_var", "move_std", "move_cov", "move_corr"]
MOVE_EXP = ["move_exp_nancount", "move_exp_nanmean", "move_exp_nansum", "move_exp_nanvar", "move_exp_nanstd",
            "move_exp_nancov", "move_exp_nancorr"]
TWO = {"move_cov", "move_corr", "move_exp_nancov", "move_exp_nancorr"}


def _inputs(kind, shape, seed):
    rng = np.random.default_rng(seed)
    z1 = rng.standard_normal(shape)
    z2 = rng.standard_normal(shape)
    if kind == "stress":
        a = 1e6 + z1
        b = 1e6 + 0.7 * z1 + np.sqrt(0.51) * z2
        p = 0.02
    else:
        a, b, p = z1, 0.7 * z1 + np.sqrt(0.51) * z2, 0.1
    a[rng.random(shape) < p] = np.nan
    b[rng.random(shape) < p] = np.nan
    return a, b


def _report(fname, kind, param, r):
    print(f"fp32c {fname} {kind} {param}: max scaled error {r['max_err']:.3g} over {r['n']} outputs")


@pytest.mark.parametrize("kind", ["normal", "stress"])
@pytest.mark.parametrize("fname", MOVE)
def test_move_fp32c(fname, kind):
    a, b = _inputs(kind, (6, 30_011), 31)
    y = b if fname in TWO else None
    for window in (5, 252, 3000):
        mc = window // 2
        args = (a, b) if y is not None else (a,)
        got = getattr(nb, fname)(*args, window=window, min_count=mc, precision="fp32c")
        ext = oracle.move(fname, a, y, window=window, min_count=mc, ext=True)
        scale = move_scale(fname, a, y, window)
        r = scaled_error(got, ext, scale, move_degenerate(fname, a, y, window))
        _report(fname, kind, f"w={window}", r)
        assert r["nan_mismatch"] == 0, (fname, window, r)
        assert r["max_err"] <= FP32C_TOL, (fname, window, r)


@pytest.mark.parametrize("kind", ["normal", "stress"])
@pytest.mark.parametrize("fname", MOVE_EXP)
def test_move_exp_fp32c(fname, kind):
    a, b = _inputs(kind, (4, 40_007), 32)
    y = b if fname in TWO else None
    for alpha in (0.5, 0.01, 1e-3):
        args = (a, b) if y is not None else (a,)
        got = getattr(nb, fname)(*args, alpha=alpha, precision="fp32c")
        ext = oracle.move_exp(fname, a, y, alpha=alpha, ext=True)
        scale = exp_scale(fname, a, y, alpha)
        r = scaled_error(got, ext, scale, exp_degenerate(fname, a, y, alpha, 0.0))
        _report(fname, kind, f"alpha={alpha}", r)
        assert r["nan_mismatch"] == 0, (fname, alpha, r)
        assert r["max_err"] <= FP32C_TOL, (fname, alpha, r)


def test_fp32c_float32_input_runs_the_plain_form():
    x = np.random.default_rng(3).standard_normal((2, 500)).astype(np.float32)
    np.testing.assert_array_equal(nb.move_mean(x, window=7, precision="fp32c"), nb.move_mean(x, window=7))
    # a float32 alpha array keeps numbagg's float32 loop (a Python float alpha selects
    # the float64 one, where the compensated form applies)
    al = np.full(x.shape[-1], 0.1, dtype=np.float32)
    np.testing.assert_array_equal(nb.move_exp_nanmean(x, alpha=al, precision="fp32c"), nb.move_exp_nanmean(x, alpha=al))


def test_fp32c_deterministic_and_causal():
    a, _ = _inputs("stress", (3, 200_001), 33)
    for fn, kw in ((nb.move_std, {"window": 50}), (nb.move_exp_nanvar, {"alpha": 0.01})):
        full = fn(a, precision="fp32c", **kw)
        again = fn(a, precision="fp32c", **kw)
        part = fn(np.ascontiguousarray(a[:, :150_000]), precision="fp32c", **kw)
        np.testing.assert_array_equal(full, again)
        np.testing.assert_array_equal(full[:, :150_000], part)


@pytest.mark.parametrize("fname", MOVE)
def test_move_fp32c_rows_outside_the_double_float_range(fname):
    # rows holding an infinity, huge or tiny values are recomputed from exact window sums:
    # the reference's NaN / infinity placement, and the stated bound elsewhere.  (With an
    # infinity inside the window numbagg's move_cov gives +-inf or NaN depending on the
    # signs of the other sums; the exact kernel gives NaN there, a known difference.)
    a, b = _inputs("normal", (6, 20_000), 34)
    if fname != "move_cov":  # see the note on infinities in move_cov below
        a[1, 100] = np.inf
        a[2, 5000] = -np.inf
    a[3] *= 1e60
    a[4] *= 1e-40
    y = b if fname in TWO else None
    args = (a, b) if y is not None else (a,)
    for window in (5, 400):
        got = getattr(nb, fname)(*args, window=window, min_count=2, precision="fp32c")
        want = oracle.move(fname, a, y, window=window, min_count=2)
        ext = oracle.move(fname, a, y, window=window, min_count=2, ext=True)
        allow = move_degenerate(fname, a, y, window)
        allow = np.zeros(a.shape, bool) if allow is None else allow
        assert np.array_equal(np.isnan(got) & ~allow, np.isnan(want) & ~allow), (fname, window)
        inf = np.isinf(want) & ~allow
        assert np.array_equal(got[inf], want[inf]), (fname, window)
        fin = np.isfinite(ext) & np.isfinite(want) & ~allow
        r = scaled_error(np.where(fin, got, 0.0), np.where(fin, ext, 0.0), move_scale(fname, a, y, window))
        assert r["max_err"] <= FP32C_TOL, (fname, window, r)


@pytest.mark.parametrize("fname", MOVE)
def test_move_fp32c_edges(fname):
    # tile edges of the double-float scan (1024 positions), a single row, all-NaN rows,
    # windows of 1 and of the whole row, min_count 0
    rng = np.random.default_rng(35)
    for rows, n in ((1, 1), (1, 1025), (3, 3073), (2, 5000)):
        a = rng.standard_normal((rows, n))
        b = 0.5 * a + rng.standard_normal((rows, n))
        a[rng.random(a.shape) < 0.2] = np.nan
        if rows > 1:
            a[1] = np.nan
        y = b if fname in TWO else None
        args = (a, b) if y is not None else (a,)
        for window, mc in ((1, 0), (1, 1), (min(7, n), 2), (n, 1)):
            got = getattr(nb, fname)(*args, window=window, min_count=mc, precision="fp32c")
            ext = oracle.move(fname, a, y, window=window, min_count=mc, ext=True)
            r = scaled_error(got, ext, move_scale(fname, a, y, window), move_degenerate(fname, a, y, window))
            assert r["nan_mismatch"] == 0 and r["max_err"] <= FP32C_TOL, (fname, rows, n, window, mc, r)
