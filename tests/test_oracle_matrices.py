"""Pin the oracle's restatements of the exponentially weighted matrices
(numbagg/moving_matrix.py:204-432) and the static pairwise-complete matrices
(numbagg/funcs.py:338-532) to numbagg's own results (CPU only).

The golden vectors come from the reference's kernel bodies (tests/golden/make_golden.py).
float64 must agree bit for bit.  For float32 the Python run of the kernel bodies
keeps `1.0 - alpha_t` in float32 where numba computes it in float64, so the float32
vectors are compared within float32 tolerance.  The rest are the reference's own
known-answer and property tests (numbagg/test/test_matrix_functions.py), run on the
oracle.
"""

import numpy as np
import pytest

import oracle
from tests.conftest import same_values

EXP_MATRIX = ["move_exp_nancovmatrix", "move_exp_nancorrmatrix"]
STATIC_MATRIX = ["nancovmatrix", "nancorrmatrix"]


def _keys(golden, prefix):
    return sorted(k for k in golden if k.startswith(prefix + "|"))


@pytest.mark.parametrize("fname", EXP_MATRIX)
def test_exp_matrix_golden(golden, fname):
    keys = _keys(golden, fname)
    assert len(keys) == 12
    for key in keys:
        _, dt, atag, mw = key.split("|")
        a = golden[f"ematrix_in_{dt}"]
        alpha = golden[f"ematrix_alpha_vec_{dt}"] if atag == "vec" else np.full(a.shape[0], float(atag), dtype=a.dtype)
        got = oracle.move_exp_matrix(fname, a, alpha=alpha, min_weight=float(mw))
        want = golden[key]
        assert got.dtype == want.dtype, key
        if dt == "f64":
            assert same_values(got, want), key
        else:
            # while a pair has been seen at most once its bias is 0 mathematically and
            # the NaN decision is float32 rounding noise in either typing
            v = ~np.isnan(a)
            seen = np.cumsum(v[:, :, None] & v[:, None, :], axis=0)
            ok = seen > 1
            assert np.array_equal(np.isnan(got)[ok], np.isnan(want)[ok]), key
            # few-observation correlations amplify the float32 rounding of the variances
            np.testing.assert_allclose(got[ok], want[ok], rtol=2e-4, atol=2e-4, equal_nan=True, err_msg=key)


@pytest.mark.parametrize("fname", STATIC_MATRIX)
@pytest.mark.parametrize("dt", ["f64", "f32"])
def test_static_matrix_golden(golden, fname, dt):
    a = golden[f"smatrix_in_{dt}"]
    got = oracle.static_matrix(fname, a)
    assert same_values(got, golden[f"{fname}|{dt}"]), (fname, dt)


def test_exp_matrix_dtype_resolution():
    a32 = np.random.default_rng(0).standard_normal((12, 3)).astype(np.float32)
    # a Python float alpha is broadcast to a float64 array: numbagg's float64 loop
    assert oracle.move_exp_matrix("move_exp_nancovmatrix", a32, alpha=0.5).dtype == np.float64
    # a float32 alpha array keeps the float32 loop
    al = np.full(12, 0.5, dtype=np.float32)
    assert oracle.move_exp_matrix("move_exp_nancovmatrix", a32, alpha=al).dtype == np.float32
    assert oracle.static_matrix("nancovmatrix", a32.T).dtype == np.float32


# ---- numbagg/test/test_matrix_functions.py, run on the oracle ---------------------------


def test_static_known_answers():
    # :30-48 perfect linear relation
    data = np.array([[1, 2, 3, 4], [2, 4, 6, 8]], dtype=np.float64)
    np.testing.assert_allclose(oracle.static_matrix("nancorrmatrix", data), [[1.0, 1.0], [1.0, 1.0]])
    # :77-89 against numpy without NaNs
    np.random.seed(42)
    data = np.random.randn(5, 100)
    np.testing.assert_allclose(oracle.static_matrix("nancorrmatrix", data), np.corrcoef(data), rtol=1e-10)
    np.testing.assert_allclose(oracle.static_matrix("nancovmatrix", data), np.cov(data), rtol=1e-10)
    # :91-106 constant variables
    data = np.array([[1, 1, 1, 1], [2, 2, 2, 2], [1, 2, 3, 4]], dtype=np.float64)
    corr = oracle.static_matrix("nancorrmatrix", data)
    assert np.isnan(corr[0, 1]) and np.isnan(corr[0, 2]) and corr[2, 2] == 1.0
    cov = oracle.static_matrix("nancovmatrix", data)
    assert cov[0, 0] == 0.0 and cov[1, 1] == 0.0 and cov[0, 1] == 0.0
    # :53-66 NaNs: symmetric, unit diagonal
    data = np.array([[1, 2, np.nan, 4], [2, 4, 6, np.nan], [np.nan, 1, 2, 3]], dtype=np.float64)
    corr = oracle.static_matrix("nancorrmatrix", data)
    np.testing.assert_allclose(corr, corr.T, equal_nan=True)
    np.testing.assert_allclose(np.diag(corr), [1.0, 1.0, 1.0])
    # :143-154 correlation = covariance / (std_i std_j)
    np.random.seed(42)
    data = np.random.randn(4, 50)
    cov = oracle.static_matrix("nancovmatrix", data)
    s = np.sqrt(np.diag(cov))
    np.testing.assert_allclose(oracle.static_matrix("nancorrmatrix", data), cov / np.outer(s, s), rtol=1e-10)
    with pytest.raises(ValueError, match="requires at least a 2D array"):
        oracle.static_matrix("nancovmatrix", np.arange(5.0))


def test_exp_matrix_known_answers():
    # :443-470 perfect linear relation
    data = np.array([[1, 2], [2, 4], [3, 6], [4, 8]], dtype=np.float64)
    r = oracle.move_exp_matrix("move_exp_nancorrmatrix", data, alpha=0.5)
    np.testing.assert_allclose(r[-1], [[1.0, 1.0], [1.0, 1.0]], rtol=1e-10)
    # :490-503 min_weight
    hi = oracle.move_exp_matrix("move_exp_nancovmatrix", data, alpha=0.1, min_weight=0.8)
    lo = oracle.move_exp_matrix("move_exp_nancovmatrix", data, alpha=0.1, min_weight=0.1)
    assert np.isnan(hi[0]).sum() >= np.isnan(lo[0]).sum()
    # :539-552 array alpha differs from a constant one
    alpha = np.array([0.1, 0.5, 0.9, 0.3])
    assert not np.allclose(
        oracle.move_exp_matrix("move_exp_nancovmatrix", data, alpha=alpha),
        oracle.move_exp_matrix("move_exp_nancovmatrix", data, alpha=0.5),
    )


@pytest.mark.parametrize("alpha", [0.1, 0.5, 0.9])
def test_exp_matrix_matches_pairwise(alpha):
    # :620-654: the (0, 1) entry equals move_exp_nancov / nancorr of the two series
    np.random.seed(42)
    a1 = np.random.randn(50)
    a2 = np.random.randn(50) * 2 + 1
    a1[[3, 17]] = np.nan
    a2[[5, 17, 30]] = np.nan
    m = np.column_stack([a1, a2])
    cov = oracle.move_exp_matrix("move_exp_nancovmatrix", m, alpha=alpha)
    corr = oracle.move_exp_matrix("move_exp_nancorrmatrix", m, alpha=alpha)
    np.testing.assert_allclose(cov[:, 0, 1], oracle.move_exp("move_exp_nancov", a1, a2, alpha=alpha), rtol=1e-10)
    np.testing.assert_allclose(corr[:, 0, 1], oracle.move_exp("move_exp_nancorr", a1, a2, alpha=alpha), rtol=1e-10)
    np.testing.assert_allclose(cov[:, 0, 1], cov[:, 1, 0], rtol=1e-10)


def test_exp_matrix_broadcasting():
    # :555-572 leading dimensions and a per-batch alpha
    rng = np.random.default_rng(3)
    data = rng.standard_normal((2, 3, 15, 4))
    r = oracle.move_exp_matrix("move_exp_nancovmatrix", data, alpha=0.3)
    assert r.shape == (2, 3, 15, 4, 4)
    np.testing.assert_array_equal(r[1, 2], oracle.move_exp_matrix("move_exp_nancovmatrix", data[1, 2], alpha=0.3))
    al = rng.uniform(0.1, 0.9, size=(3, 15))
    r = oracle.move_exp_matrix("move_exp_nancorrmatrix", data, alpha=al)
    np.testing.assert_array_equal(r[0, 1], oracle.move_exp_matrix("move_exp_nancorrmatrix", data[0, 1], alpha=al[1]))
