"""GPU results against numbagg's own outputs (the golden vectors produced by running
the reference kernels, tests/golden/make_golden.py).

Selection results (fills, counts, argmax/argmin/min/max/first/last, any/all) must be
bit-identical; sums, means, variances and correlations must agree within the scaled
tolerance of tests/parity.py with identical NaN placement."""

import numpy as np
import pytest

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

TOL = {"f64": F64_TOL, "f32": F32_TOL}


def _keys(golden, prefix):
    return sorted(k for k in golden if k.startswith(prefix + "|"))


@pytest.mark.parametrize("fname", ["move_sum", "move_mean", "move_var", "move_std", "move_cov", "move_corr"])
def test_move_golden(golden, fname):
    func = getattr(nb, fname)
    for key in _keys(golden, fname):
        _, tag, dt, w, mc = key.split("|")
        x = golden[f"move_in_{tag}_{dt}"]
        b = golden.get(f"move_in_b_{dt}") if fname in ("move_cov", "move_corr") else None
        mc = None if mc == "None" else int(mc)
        w = int(w)
        got = func(x, b, window=w, min_count=mc) if b is not None else func(x, window=w, min_count=mc)
        want = golden[key]
        assert got.dtype == want.dtype
        scale = move_scale(fname, x, b, w)
        allow = move_degenerate(fname, x, b, w)
        ext = oracle.move(fname, x, b, window=w, min_count=mc, ext=True)
        assert_parity(got, want, ext, scale, TOL[dt], allow, key)


@pytest.mark.parametrize(
    "fname",
    [
        "move_exp_nancount",
        "move_exp_nanmean",
        "move_exp_nansum",
        "move_exp_nanvar",
        "move_exp_nanstd",
        "move_exp_nancov",
        "move_exp_nancorr",
    ],
)
def test_move_exp_golden(golden, fname):
    func = getattr(nb, fname)
    for key in _keys(golden, fname):
        _, dt, atag, mw = key.split("|")
        x = golden[f"exp_in_{dt}"]
        b = golden[f"exp_in_b_{dt}"] if fname in ("move_exp_nancov", "move_exp_nancorr") else None
        # the golden float32 runs used float32 alpha arrays, which select numbagg's
        # float32 loop (a Python-float alpha would select the float64 one)
        alpha = golden[f"exp_alpha_vec_{dt}"] if atag == "vec" else np.full(x.shape[-1], float(atag), dtype=x.dtype)
        mw = float(mw)
        got = func(x, b, alpha=alpha, min_weight=mw) if b is not None else func(x, alpha=alpha, min_weight=mw)
        want = golden[key]
        scale = exp_scale(fname, x, b, alpha)
        allow = exp_degenerate(fname, x, b, alpha, mw)
        ext = oracle.move_exp(fname, x, b, alpha=alpha, min_weight=mw, ext=True)
        assert_parity(got, want, ext, scale, TOL[dt], allow, key)


@pytest.mark.parametrize("fname", ["ffill", "bfill"])
def test_fill_golden(golden, fname):
    func = getattr(nb, fname)
    for key in _keys(golden, fname):
        _, dt, lim = key.split("|")
        got = func(golden[f"fill_in_{dt}"], limit=None if lim == "None" else int(lim))
        assert_bit_equal(got, golden[key], key)


EXACT_GROUP = {
    "group_nancount",
    "group_nanargmax",
    "group_nanargmin",
    "group_nanmax",
    "group_nanmin",
    "group_nanfirst",
    "group_nanlast",
    "group_nanany",
    "group_nanall",
}


@pytest.mark.parametrize("fname", [f.__name__ for f in nb.GROUPED_FUNCS])
def test_group_golden(golden, fname):
    func = getattr(nb, fname)
    labels = golden["group_labels"]
    for key in _keys(golden, fname):
        _, dt, K, ddof = key.split("|")
        v = golden[f"group_vals_{dt}"]
        kw = {} if ddof == "None" else {"ddof": int(ddof)}
        got = func(v, labels, num_labels=int(K), axis=-1, **kw)
        want = golden[key]
        if fname == "group_nanfirst" and want.dtype.kind == "i":
            present = np.zeros(int(K), bool)
            present[np.unique(labels[(labels >= 0) & (labels < int(K))])] = True
            assert np.array_equal(got[:, present], want[:, present]), key
            continue
        exact = fname in EXACT_GROUP or want.dtype.kind == "i"
        if exact:
            assert_bit_equal(got, want, key)
        else:
            vv = v.astype(np.float64)
            absv = np.abs(np.where(np.isnan(vv), 0, vv))
            if fname in ("group_nanvar", "group_nanstd", "group_nansum_of_squares"):
                scale = np.array([[np.sum(absv[r][labels == k] ** 2) / max(1, np.sum(labels == k)) for k in range(int(K))] for r in range(v.shape[0])])
                if fname == "group_nanstd":
                    scale = np.sqrt(scale)
                if fname == "group_nansum_of_squares":
                    scale = scale * np.array([max(1, np.sum(labels == k)) for k in range(int(K))])
            elif fname == "group_nanprod":
                scale = np.abs(want.astype(np.float64))
            else:
                scale = np.array([[np.sum(absv[r][labels == k]) for k in range(int(K))] for r in range(v.shape[0])])
                if fname == "group_nanmean":
                    scale = scale / np.maximum(1, [np.sum(~np.isnan(vv[r][labels == k])) for r in range(v.shape[0]) for k in range(int(K))]).reshape(scale.shape)
            tol = F32_TOL if want.dtype == np.float32 else F64_TOL
            assert_scaled_close(got, want, scale, tol, None, key)


@pytest.mark.parametrize("fname", ["move_covmatrix", "move_corrmatrix"])
def test_move_matrix_golden(golden, fname):
    func = getattr(nb, fname)
    for key in _keys(golden, fname):
        _, dt, w, mc = key.split("|")
        a = golden[f"matrix_in_{dt}"]
        got = func(a, window=int(w), min_count=None if mc == "None" else int(mc))
        want = golden[key]
        assert got.shape == want.shape and got.dtype == want.dtype
        mcv = None if mc == "None" else int(mc)
        ext = oracle.move_matrix(fname, a.astype(np.float64), window=int(w), min_count=mcv, ext=True)
        if dt == "f64":
            scale = np.ones_like(want) if fname == "move_corrmatrix" else np.nanmax(np.abs(want)) * np.ones_like(want)
            assert_parity(got, want, ext, scale, F64_TOL, None, key)
        else:
            # both the reference and this implementation accumulate float32 input in
            # float32, in different orders, so each carries float32 rounding error
            scale = np.ones_like(want) if fname == "move_corrmatrix" else np.nanmax(np.abs(want)) * np.ones_like(want)
            # a window holding <= 2 complete pairs has correlation +-1 exactly; the
            # float32-accumulated reference returns its rounding noise there
            v = (~np.isnan(a)).astype(np.int64)
            pairs = np.einsum("ti,tj->tij", v, v)
            csum = np.cumsum(pairs, axis=0)
            win = csum.copy()
            win[int(w):] -= csum[: -int(w)]
            allow = (win <= 2) if fname == "move_corrmatrix" else None
            assert_parity(got, want, ext, scale, 2e-4, allow, key)
