"""GPU parity of the exponentially weighted matrices (numbagg/moving_matrix.py:204-432)
and the static pairwise-complete matrices (numbagg/funcs.py:338-532) against the
oracle's restatements, plus the reference's own known answers
(numbagg/test/test_matrix_functions.py)."""

import numpy as np
import pytest
import torch

import numbagg_gb300 as nb
import oracle
from tests.parity import F64_TOL, assert_parity

pytestmark = pytest.mark.gpu


def _cov_scale(ext):
    d = np.abs(np.nan_to_num(np.einsum("...ii->...i", ext)))
    return np.sqrt(d[..., :, None] * d[..., None, :])


def _cond(msq, var):
    with np.errstate(invalid="ignore", divide="ignore"):
        c = np.where(var > 0, msq / np.where(var > 0, var, 1.0), np.inf)
    return np.where(np.isnan(c), np.inf, c)


def _exp_corr_scale(a, alpha):
    """max(1, cond_i, cond_j) with cond = EWM mean of x^2 / EWM variance of each variable:
    how much the variance cancellation amplifies rounding in a correlation."""
    x = np.moveaxis(np.asarray(a, dtype=np.float64), -1, -2)  # (..., V, T)
    al = np.moveaxis(np.broadcast_to(alpha, a.shape[:-1])[..., None, :], -2, -2) if isinstance(alpha, np.ndarray) else alpha
    if isinstance(al, np.ndarray):
        al = np.broadcast_to(al, x.shape)
    msq = oracle.move_exp("move_exp_nanmean", x * x, alpha=al)
    var = oracle.move_exp("move_exp_nanvar", x, alpha=al)
    c = np.moveaxis(_cond(msq, var), -1, -2)  # (..., T, V)
    return np.fmax(1.0, np.fmax(c[..., :, :, None], c[..., :, None, :]))


def _static_corr_scale(a):
    x = np.asarray(a, dtype=np.float64)  # (..., V, n_obs)
    with np.errstate(invalid="ignore"):
        c = _cond(np.nanmean(x * x, axis=-1), np.nanvar(x, axis=-1))
    return np.fmax(1.0, np.fmax(c[..., :, None], c[..., None, :]))


def _exp_allow(a, alpha, min_weight):
    """Pairs seen at most once (the bias is 0 mathematically, so the reference's NaN
    decision rests on rounding noise) and steps whose weight equals min_weight."""
    v = ~np.isnan(a)
    both = v[..., :, :, None] & v[..., :, None, :]
    seen = np.cumsum(both, axis=-3)
    allow = seen <= 1
    al = np.broadcast_to(alpha, a.shape[:-1]).astype(np.float64) if isinstance(alpha, np.ndarray) else np.full(a.shape[:-1], alpha)
    w = np.zeros(both.shape)
    acc = np.zeros(both.shape[:-3] + both.shape[-2:])
    for t in range(a.shape[-2]):
        acc = acc * (1.0 - al[..., t, None, None]) + np.where(both[..., t, :, :], al[..., t, None, None], 0.0)
        w[..., t, :, :] = acc
    return allow | (np.abs(w - min_weight) <= 1e-12)


@pytest.mark.parametrize("fname", ["move_exp_nancovmatrix", "move_exp_nancorrmatrix"])
@pytest.mark.parametrize("alpha,min_weight", [(0.5, 0.0), (0.05, 0.0), (0.01, 0.5), ("vec", 0.2), ("batch", 0.0)])
def test_exp_matrix_vs_oracle(fname, alpha, min_weight):
    rng = np.random.default_rng(21)
    a = rng.standard_normal((2, 700, 37))
    a[rng.random(a.shape) < 0.05] = np.nan
    a[:, 100:110, 3] = np.nan  # a run of missing values in one variable
    if alpha == "vec":
        alpha = rng.uniform(0.01, 0.6, size=700)
    elif alpha == "batch":
        alpha = rng.uniform(0.01, 0.6, size=(2, 700))
    func = getattr(nb, fname)
    got = func(a, alpha=alpha, min_weight=min_weight)
    want = oracle.move_exp_matrix(fname, a, alpha=alpha, min_weight=min_weight)
    ext = oracle.move_exp_matrix(fname, a, alpha=alpha, min_weight=min_weight, ext=True)
    assert got.shape == want.shape == (2, 700, 37, 37) and got.dtype == np.float64
    scale = _cov_scale(ext) if fname == "move_exp_nancovmatrix" else _exp_corr_scale(a, alpha)
    r = assert_parity(got, want, ext, scale, F64_TOL, _exp_allow(a, alpha, min_weight), f"{fname} alpha={alpha}")
    assert r["allowed"] <= 0.01 * r["n"], r


@pytest.mark.parametrize("fname", ["move_exp_nancovmatrix", "move_exp_nancorrmatrix"])
def test_exp_matrix_float32(fname):
    rng = np.random.default_rng(22)
    a = rng.standard_normal((900, 33)).astype(np.float32)
    a[rng.random(a.shape) < 0.05] = np.nan
    func = getattr(nb, fname)
    # a Python float alpha selects numbagg's float64 loop: the result is float64
    wide = func(a, alpha=0.1)
    assert wide.dtype == np.float64
    np.testing.assert_array_equal(wide, func(a.astype(np.float64), alpha=0.1))
    # a float32 alpha array keeps the float32 loop, float32 states as the reference's
    al = np.full(900, 0.1, dtype=np.float32)
    got = func(a, alpha=al)
    assert got.dtype == np.float32
    want = oracle.move_exp_matrix(fname, a, alpha=al)
    ext = oracle.move_exp_matrix(fname, a, alpha=al, ext=True)
    scale = _cov_scale(ext) if fname == "move_exp_nancovmatrix" else _exp_corr_scale(a, 0.1)
    assert_parity(got, want, ext, scale, 1e-4, _exp_allow(a, 0.1, 0.0), f"{fname} float32")


def test_exp_matrix_known_answers():
    # numbagg/test/test_matrix_functions.py:443-470, :620-654
    data = np.array([[1, 2], [2, 4], [3, 6], [4, 8]], dtype=np.float64)
    r = nb.move_exp_nancorrmatrix(data, alpha=0.5)
    np.testing.assert_allclose(r[-1], [[1.0, 1.0], [1.0, 1.0]], rtol=1e-10)
    np.random.seed(42)
    a1 = np.random.randn(50)
    a2 = np.random.randn(50) * 2 + 1
    m = np.column_stack([a1, a2])
    for alpha in (0.1, 0.5, 0.9):
        np.testing.assert_allclose(nb.move_exp_nancovmatrix(m, alpha=alpha)[:, 0, 1], nb.move_exp_nancov(a1, a2, alpha=alpha), rtol=1e-10)
        np.testing.assert_allclose(nb.move_exp_nancorrmatrix(m, alpha=alpha)[:, 0, 1], nb.move_exp_nancorr(a1, a2, alpha=alpha), rtol=1e-10)
    with pytest.raises(ValueError, match="requires at least a 2D array"):
        nb.move_exp_nancovmatrix(np.arange(5.0), alpha=0.5)
    # on device tensors the result stays on the device
    t = torch.from_numpy(m).cuda()
    assert nb.move_exp_nancovmatrix(t, alpha=0.3).is_cuda


@pytest.mark.parametrize("fname", ["nancovmatrix", "nancorrmatrix"])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("shape", [(3, 37, 1000), (1, 256, 5000), (2, 5, 200_000)])
def test_static_matrix_vs_oracle(fname, dtype, shape):
    rng = np.random.default_rng(23)
    a = (rng.standard_normal(shape) * rng.uniform(0.1, 10, size=shape[:-1] + (1,)) + 3).astype(dtype)
    a[rng.random(shape) < 0.05] = np.nan
    a[0, 1, :] = np.nan  # a variable never observed
    a[0, 2, 2:] = np.nan  # one observed twice
    func = getattr(nb, fname)
    got = func(a)
    want = oracle.static_matrix(fname, a)
    ext = oracle.static_matrix(fname, a.astype(np.float64), ext=True)
    assert got.shape == want.shape and got.dtype == want.dtype == dtype
    scale = _cov_scale(ext) if fname == "nancovmatrix" else _static_corr_scale(a)
    # float32: the reference sums observations one by one in float32; this sums slices
    # of them in float32 and folds the slices, so both carry float32 rounding
    tol = F64_TOL if dtype == np.float64 else 2e-4
    assert_parity(got, want, ext, scale, tol, None, f"{fname} {shape} {np.dtype(dtype).name}")
    g = np.asarray(got)
    np.testing.assert_array_equal(g, np.swapaxes(g, -1, -2))


def test_static_matrix_known_answers():
    # numbagg/test/test_matrix_functions.py:30-106, :108-141
    data = np.array([[1, 2, 3, 4], [2, 4, 6, 8]], dtype=np.float64)
    np.testing.assert_allclose(nb.nancorrmatrix(data), [[1.0, 1.0], [1.0, 1.0]])
    np.random.seed(42)
    data = np.random.randn(5, 100)
    np.testing.assert_allclose(nb.nancorrmatrix(data), np.corrcoef(data), rtol=1e-10)
    np.testing.assert_allclose(nb.nancovmatrix(data), np.cov(data), rtol=1e-10)
    data = np.array([[1, 1, 1, 1], [2, 2, 2, 2], [1, 2, 3, 4]], dtype=np.float64)
    corr = nb.nancorrmatrix(data)
    assert np.isnan(corr[0, 1]) and np.isnan(corr[0, 2]) and corr[2, 2] == 1.0
    cov = nb.nancovmatrix(data)
    assert cov[0, 0] == 0.0 and cov[1, 1] == 0.0 and cov[0, 1] == 0.0
    d4 = np.random.randn(2, 3, 4, 10)
    r = nb.nancovmatrix(d4)
    assert r.shape == (2, 3, 4, 4)
    np.testing.assert_allclose(r[1, 2], nb.nancovmatrix(d4[1, 2]), rtol=1e-10)
    assert nb.nancovmatrix(np.random.randn(3, 10).astype(np.float32)).dtype == np.float32
    with pytest.raises(ValueError, match="requires at least a 2D array"):
        nb.nancorrmatrix(np.arange(5.0))
