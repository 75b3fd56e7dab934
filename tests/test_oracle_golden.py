"""Pin the C oracle to numbagg's own results (CPU only).

The golden vectors in ``golden/reference_vectors.npz`` were produced by running
numbagg's kernel bodies (``tests/golden/make_golden.py``).  The oracle must
reproduce every one of them bit for bit: same operations, same order, same types.
"""

import numpy as np
import pytest

import oracle
from tests.conftest import same_values

DT = {"f64": np.float64, "f32": np.float32, "i32": np.int32}


def _keys(golden, prefix):
    return sorted(k for k in golden if k.startswith(prefix + "|"))


@pytest.mark.parametrize("fname", oracle.MOVE_FUNCS)
def test_move_golden(golden, fname):
    keys = _keys(golden, fname)
    assert keys
    for key in keys:
        _, tag, dt, w, mc = key.split("|")
        x = golden[f"move_in_{tag}_{dt}"]
        b = golden.get(f"move_in_b_{dt}") if fname in ("move_cov", "move_corr") else None
        mc = None if mc == "None" else int(mc)
        got = oracle.move(fname, x, b, window=int(w), min_count=mc)
        assert same_values(got, golden[key]), key


@pytest.mark.parametrize("fname", oracle.MOVE_EXP_FUNCS)
def test_move_exp_golden(golden, fname):
    keys = _keys(golden, fname)
    assert keys
    for key in keys:
        _, dt, atag, mw = key.split("|")
        x = golden[f"exp_in_{dt}"]
        b = golden[f"exp_in_b_{dt}"] if fname in ("move_exp_nancov", "move_exp_nancorr") else None
        # the golden float32 runs used float32 alpha arrays, which select numbagg's
        # float32 loop (a Python-float alpha would select the float64 one)
        alpha = golden[f"exp_alpha_vec_{dt}"] if atag == "vec" else np.full(x.shape[-1], float(atag), dtype=x.dtype)
        got = oracle.move_exp(fname, x, b, alpha=alpha, min_weight=float(mw))
        assert same_values(got, golden[key]), key


@pytest.mark.parametrize("fname", ["ffill", "bfill"])
def test_fill_golden(golden, fname):
    keys = _keys(golden, fname)
    assert keys
    for key in keys:
        _, dt, lim = key.split("|")
        x = golden[f"fill_in_{dt}"]
        got = oracle.fill(fname, x, limit=None if lim == "None" else int(lim))
        assert same_values(got, golden[key]), key


@pytest.mark.parametrize("fname", oracle.GROUP_FUNCS)
def test_group_golden(golden, fname):
    keys = _keys(golden, fname)
    assert keys
    labels = golden["group_labels"]
    for key in keys:
        _, dt, K, ddof = key.split("|")
        v = golden[f"group_vals_{dt}"]
        kw = {} if ddof == "None" else {"ddof": int(ddof)}
        got = oracle.group(fname, v, labels, num_labels=int(K), axis=-1, **kw)
        want = golden[key]
        if fname == "group_nanfirst" and want.dtype.kind == "i":
            # unseen groups are np.empty garbage in the reference; compare seen ones
            seen = np.zeros(want.shape, bool)
            for r in range(v.shape[0]):
                vv = v[r].astype(np.int32) if v.dtype == np.bool_ else v[r]
                for lab in np.unique(labels[(labels >= 0) & (labels < int(K))]):
                    seen[r, lab] = True
                _ = vv
            assert np.array_equal(got[seen], want[seen]), key
            continue
        assert same_values(got, want), key


@pytest.mark.parametrize("fname", ["move_covmatrix", "move_corrmatrix"])
def test_move_matrix_golden(golden, fname):
    keys = _keys(golden, fname)
    assert keys
    for key in keys:
        _, dt, w, mc = key.split("|")
        a = golden[f"matrix_in_{dt}"]
        got = oracle.move_matrix(fname, a, window=int(w), min_count=None if mc == "None" else int(mc))
        assert same_values(got, golden[key]), key


# ---- the reference's own known-answer tests, run against the oracle ----------------


def test_move_exp_nancount_known_answer():
    # numbagg/test/test_moving_exp.py:111-120
    a = np.array([1, 0, np.nan, np.nan, 1, 0])
    np.testing.assert_allclose(
        oracle.move_exp("move_exp_nancount", a, alpha=0.5),
        [1.0, 1.5, 0.75, 0.375, 1.1875, 1.59375],
    )
    np.testing.assert_allclose(
        oracle.move_exp("move_exp_nancount", a, alpha=0.25),
        [1.0, 1.75, 1.3125, 0.984375, 1.7382812, 2.3037109],
        rtol=1e-7,
    )


def test_move_exp_nanmean_nansum_known_answer():
    # numbagg/test/test_moving_exp.py:239-248, :323-332
    a = np.array([10, 0, np.nan, 10])
    np.testing.assert_allclose(
        oracle.move_exp("move_exp_nanmean", a, alpha=0.5), [10.0, 3.3333333, 3.3333333, 8.1818182], rtol=1e-7
    )
    np.testing.assert_allclose(
        oracle.move_exp("move_exp_nanmean", a, alpha=0.25), [10.0, 4.2857143, 4.2857143, 7.1653543], rtol=1e-7
    )
    np.testing.assert_allclose(oracle.move_exp("move_exp_nansum", a, alpha=0.5), [10.0, 5.0, 2.5, 11.25])
    np.testing.assert_allclose(oracle.move_exp("move_exp_nansum", a, alpha=0.25), [10.0, 7.5, 5.625, 14.21875])


def test_move_exp_nancorr_known_answer():
    # numbagg/test/test_moving_exp.py:335-345
    a1 = np.array([10, 0, 5, 10.0])
    a2 = np.array([10, 0, 10, 5.0])
    np.testing.assert_allclose(
        oracle.move_exp("move_exp_nancorr", a1, a2, alpha=0.5), [np.nan, 1.0, 0.8485281, 0.2274294], rtol=1e-6
    )
    np.testing.assert_allclose(
        oracle.move_exp("move_exp_nancorr", a1, a2, alpha=0.25), [np.nan, 1.0, 0.85, 0.4789468], rtol=1e-6
    )


def test_move_sum_float32_exact_after_tiles():
    # numbagg/test/test_moving.py:186-192: exact equality after 100 tiles
    rs = np.random.RandomState(0)
    rs.random(1000)  # the fixture's generator was used once before in that module
    arr = np.tile((rs.rand(10) * 1e13).astype(np.float32), 100)
    res = oracle.move("move_sum", arr, window=10)
    assert res[-1] == np.sum(arr[:10])


def test_grouped_known_answers():
    # numbagg/test/test_grouped.py:359-394, :510-590
    v = np.array([1, 2, 3, 4, 5], dtype=np.int32)
    lab = np.array([0, 0, 0, 1, 1], dtype=np.int32)
    np.testing.assert_array_equal(oracle.group("group_nancount", v, lab), [3, 2])
    v = np.array([1, 2, 3, 4, 5, 6], dtype=np.int32)
    lab = np.array([0, 0, 0, 1, 1, 2], dtype=np.int32)
    np.testing.assert_allclose(oracle.group("group_nanmean", v, lab), [2.0, 4.5, 6.0])
    np.testing.assert_array_equal(oracle.group("group_nanmin", v, lab), [1, 4, 6])
    np.testing.assert_array_equal(oracle.group("group_nanprod", v, lab), [6, 20, 6])
    values = np.arange(24.0).reshape(2, 3, 4)
    labels = np.array([[0, 0, 1, 1], [0, 1, 1, 2], [2, 2, 2, 2]])
    np.testing.assert_allclose(oracle.group("group_nanargmax", values, labels, axis=(1, 2))[0], [4.0, 6.0, 11.0])
    np.testing.assert_allclose(oracle.group("group_nanargmin", values, labels, axis=(1, 2))[0], [0.0, 2.0, 7.0])
    values = np.array([[1.0, 5.0, 3.0], [2.0, 4.0, 6.0]])
    labels = np.array([[0, 0, 1], [1, 2, 2]])
    np.testing.assert_allclose(oracle.group("group_nanargmax", values, labels), [1.0, 2.0, 5.0])
    np.testing.assert_allclose(oracle.group("group_nanargmin", values, labels), [0.0, 3.0, 4.0])
    np.testing.assert_allclose(oracle.group("group_nanmean", np.array([True, True, False]), np.array([0, 0, 0])), [2 / 3])


def test_move_matrix_known_answers():
    # numbagg/test/test_matrix_functions.py:258-286 (zero variance windows)
    data = np.array([[1, 2], [1, 2], [1, 2], [2, 3], [3, 4], [4, 5]], dtype=np.float64)
    cov = oracle.move_matrix("move_covmatrix", data, window=3, min_count=2)
    assert cov[2, 0, 0] == 0.0 and cov[2, 1, 1] == 0.0 and cov[2, 0, 1] == 0.0
    corr = oracle.move_matrix("move_corrmatrix", data, window=3, min_count=2)
    assert np.isnan(corr[2, 0, 1])
    assert not np.all(np.isnan(corr[5]))
