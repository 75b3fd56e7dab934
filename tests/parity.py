"""Comparison helpers for the GPU parity tests.

Floating-point results are compared with a scaled relative error
    err = |gpu - ref| / max(|ref|, S)
where S is the natural magnitude of the statistic at that position (the window sum
of |x| for a sum, the window mean of x^2 for a variance, 1 for a correlation...).
A plain relative error is meaningless where the statistic itself cancels to ~0: the
reference's own running sums carry rounding residue there.

NaN placement must agree exactly, except at positions where the reference's value is
itself rounding noise of a mathematically degenerate quantity; callers pass those as
`allow` (see the masks below).  The fraction of allowed positions is reported by the
tests and must stay small.
"""

from __future__ import annotations

import numpy as np

import oracle

F64_TOL = 1e-12
F32_TOL = 2e-6


def scaled_error(got, ref, scale, allow=None):
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    scale = np.broadcast_to(np.asarray(scale, dtype=np.float64), ref.shape)
    gn, rn = np.isnan(got), np.isnan(ref)
    allow = np.zeros(ref.shape, bool) if allow is None else np.asarray(allow, bool)
    nan_bad = (gn != rn) & ~allow
    both = ~gn & ~rn & ~allow
    inf = both & (np.isinf(ref) | np.isinf(got))
    inf_bad = inf & (got != ref)
    fin = both & ~inf
    denom = np.fmax(np.abs(ref[fin]), np.abs(scale[fin]))
    diff = np.abs(got[fin] - ref[fin])
    with np.errstate(invalid="ignore", divide="ignore"):
        err = np.where(denom > 0, diff / np.where(denom > 0, denom, 1), diff)
    return {
        "nan_mismatch": int(nan_bad.sum()),
        "inf_mismatch": int(inf_bad.sum()),
        "max_err": float(err.max()) if err.size else 0.0,
        "allowed": int(allow.sum()),
        "n": int(ref.size),
    }


def assert_scaled_close(got, ref, scale, tol, allow=None, what=""):
    r = scaled_error(got, ref, scale, allow)
    assert r["nan_mismatch"] == 0, f"{what}: NaN placement differs at {r['nan_mismatch']} positions ({r})"
    assert r["inf_mismatch"] == 0, f"{what}: inf differs ({r})"
    assert r["max_err"] <= tol, f"{what}: scaled error {r['max_err']:.3g} > {tol:g} ({r})"
    return r


def parity_error(got, ref, ext, scale, allow=None):
    """Deviation of `got` from the reference `ref` beyond the reference's own rounding
    error, measured against the extended-precision result `ext`:
        excess = max(0, |got - ref| - |ref - ext|) / max(|ref|, S)
    and the accuracy of `got` itself, |got - ext| / max(|ext|, S)."""
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    ext = np.asarray(ext, dtype=np.float64)
    scale = np.broadcast_to(np.asarray(scale, dtype=np.float64), ref.shape)
    gn, rn = np.isnan(got), np.isnan(ref)
    allow = np.zeros(ref.shape, bool) if allow is None else np.asarray(allow, bool)
    nan_bad = (gn != rn) & ~allow
    both = ~gn & ~rn & ~allow
    inf = both & (np.isinf(ref) | np.isinf(got))
    inf_bad = inf & (got != ref)
    fin = both & ~inf & ~np.isnan(ext) & ~np.isinf(ext)
    with np.errstate(invalid="ignore", divide="ignore"):
        denom = np.fmax(np.abs(ref[fin]), np.abs(scale[fin]))
        excess = np.maximum(0.0, np.abs(got[fin] - ref[fin]) - np.abs(ref[fin] - ext[fin]))
        err = np.where(denom > 0, excess / np.where(denom > 0, denom, 1), excess)
        dext = np.fmax(np.abs(ext[fin]), np.abs(scale[fin]))
        acc = np.abs(got[fin] - ext[fin])
        acc = np.where(dext > 0, acc / np.where(dext > 0, dext, 1), acc)
        refacc = np.abs(ref[fin] - ext[fin])
        refacc = np.where(dext > 0, refacc / np.where(dext > 0, dext, 1), refacc)
    return {
        "nan_mismatch": int(nan_bad.sum()),
        "inf_mismatch": int(inf_bad.sum()),
        "max_excess": float(err.max()) if err.size else 0.0,
        "gpu_vs_ext": float(acc.max()) if acc.size else 0.0,
        "ref_vs_ext": float(refacc.max()) if refacc.size else 0.0,
        "allowed": int(allow.sum()),
        "n": int(ref.size),
    }


def assert_parity(got, ref, ext, scale, tol, allow=None, what=""):
    r = parity_error(got, ref, ext, scale, allow)
    assert r["nan_mismatch"] == 0, f"{what}: NaN placement differs at {r['nan_mismatch']} positions ({r})"
    assert r["inf_mismatch"] == 0, f"{what}: inf differs ({r})"
    assert r["max_excess"] <= tol, f"{what}: deviation beyond the reference's own error {r['max_excess']:.3g} > {tol:g} ({r})"
    return r


def assert_bit_equal(got, ref, what=""):
    got = np.asarray(got)
    ref = np.asarray(ref)
    assert got.shape == ref.shape and got.dtype == ref.dtype, f"{what}: {got.shape}/{got.dtype} vs {ref.shape}/{ref.dtype}"
    if got.dtype.kind == "f":
        gn, rn = np.isnan(got), np.isnan(ref)
        assert np.array_equal(gn, rn), f"{what}: NaN placement differs"
        keep = ~gn
        assert np.array_equal(got[keep], ref[keep]), f"{what}: values differ"
        assert np.array_equal(np.signbit(got[keep]), np.signbit(ref[keep])), f"{what}: signed zeros differ"
    else:
        assert np.array_equal(got, ref), f"{what}: values differ"


# ---- scales -------------------------------------------------------------------------


def _cond(msq, var):
    """mean(x^2) / var(x): how much a rounding residue in the running sums is
    amplified in a variance-normalised result."""
    with np.errstate(invalid="ignore", divide="ignore"):
        return np.where(var > 0, msq / np.where(var > 0, var, 1.0), np.inf)


def move_scale(name, a, b, window, axis=-1):
    """Scales over a span of 2*window: the reference's running sums still carry the
    rounding residue of values that have just left the window."""
    absa = np.abs(np.asarray(a, dtype=np.float64))
    n = absa.shape[axis]
    w2 = min(2 * window, n)
    cnt = oracle.move("move_sum", (~np.isnan(absa)).astype(np.float64), window=window, min_count=0, axis=axis)
    if name == "move_sum":
        return oracle.move("move_sum", absa, window=w2, min_count=0, axis=axis)
    if name == "move_mean":
        return oracle.move("move_sum", absa, window=w2, min_count=0, axis=axis) / np.maximum(cnt, 1)
    sq = oracle.move("move_sum", absa * absa, window=w2, min_count=0, axis=axis) / np.maximum(cnt - 1, 1)
    if name == "move_var":
        return sq
    if name == "move_std":
        std = oracle.move("move_std", np.asarray(a, dtype=np.float64), window=window, min_count=2, axis=axis)
        with np.errstate(invalid="ignore", divide="ignore"):
            return np.fmax(np.sqrt(sq), sq / std)
    # the pair statistics see only the positions where both inputs are valid
    v = _valid(a, b)
    a_p = np.where(v, np.asarray(a, dtype=np.float64), np.nan)
    b_p = np.where(v, np.asarray(b, dtype=np.float64), np.nan)
    absa, absb = np.abs(a_p), np.abs(b_p)
    cnt = oracle.move("move_sum", v.astype(np.float64), window=window, min_count=0, axis=axis)
    sq = oracle.move("move_sum", absa * absa, window=w2, min_count=0, axis=axis) / np.maximum(cnt - 1, 1)
    sqb = oracle.move("move_sum", absb * absb, window=w2, min_count=0, axis=axis) / np.maximum(cnt - 1, 1)
    if name == "move_cov":
        return np.sqrt(sq * sqb)
    # move_corr
    va = oracle.move("move_var", a_p, window=window, min_count=2, axis=axis)
    vb = oracle.move("move_var", b_p, window=window, min_count=2, axis=axis)
    return np.fmax(1.0, np.fmax(_cond(sq, va), _cond(sqb, vb)))


def exp_bias(a, b, alpha, axis=-1):
    """The bias term 1 - sw2 / sw^2 of the variance family (numbagg/moving_exp.py:142-150)
    over the (pairwise) valid positions: sw = sum of decayed weights, the decayed count
    move_exp_nancount gives, and sw2 the same with every decay squared (alpha' = 1 -
    (1 - alpha)^2).  Where it cancels towards 0 the reference's float64 evaluation
    amplifies every rounding in its running sums by 1 / bias."""
    v = _valid(a, b).astype(np.float64)
    ind = np.where(v > 0, 1.0, np.nan)
    al = alpha if not isinstance(alpha, np.ndarray) else alpha.astype(np.float64)
    al2 = 1.0 - (1.0 - np.asarray(al, dtype=np.float64)) ** 2
    if not isinstance(alpha, np.ndarray):
        al2 = float(al2)
    sw = oracle.move_exp("move_exp_nancount", ind, alpha=al, axis=axis, ext=True)
    sw2 = oracle.move_exp("move_exp_nancount", ind, alpha=al2, axis=axis, ext=True)
    with np.errstate(invalid="ignore", divide="ignore"):
        bias = 1.0 - sw2 / (sw * sw)
    return np.where(np.isfinite(bias) & (bias > 0), bias, np.nan)


def exp_scale(name, a, b, alpha, axis=-1):
    """Natural magnitude of each statistic's rounding: the weighted mean of |x| or x^2;
    for the variance family the result is a biased value divided by the bias term (see
    exp_bias), whose own rounding (~eps absolute) adds |value| * eps / bias, so the scale
    is (mean(x^2) + |value|) / bias; the correlation's bias cancels
    (numbagg/moving_exp.py:319), its scale is the conditioning mean(x^2) / (var * bias)
    of either input's unnormalised weighted variance."""
    a64 = np.asarray(a, dtype=np.float64)
    absa = np.abs(a64)
    if name == "move_exp_nancount":
        return np.ones_like(absa)
    al = alpha if not isinstance(alpha, np.ndarray) else alpha.astype(np.float64)
    if name == "move_exp_nansum":
        return oracle.move_exp("move_exp_nansum", absa, alpha=al, axis=axis)
    if name == "move_exp_nanmean":
        return oracle.move_exp("move_exp_nanmean", absa, alpha=al, axis=axis)
    sq = oracle.move_exp("move_exp_nanmean", absa * absa, alpha=al, axis=axis)
    bias = exp_bias(a, b if name in ("move_exp_nancov", "move_exp_nancorr") else None, alpha, axis)
    amp = np.where(np.isnan(bias), 1.0, 1.0 / np.fmax(bias, 1e-300))
    if name in ("move_exp_nanvar", "move_exp_nanstd"):
        var = np.abs(np.nan_to_num(oracle.move_exp("move_exp_nanvar", a64, alpha=al, axis=axis, ext=True)))
        svar = (sq + var) * amp
        if name == "move_exp_nanvar":
            return svar
        std = np.sqrt(var)
        with np.errstate(invalid="ignore", divide="ignore"):
            return np.fmax(np.sqrt(svar), svar / std)
    # the pair functions see only the positions where both inputs are valid
    v = _valid(a, b)
    a64 = np.where(v, a64, np.nan)
    b64 = np.where(v, np.asarray(b, dtype=np.float64), np.nan)
    absa, absb = np.abs(a64), np.abs(b64)
    sq = oracle.move_exp("move_exp_nanmean", absa * absa, alpha=al, axis=axis)
    sqb = oracle.move_exp("move_exp_nanmean", absb * absb, alpha=al, axis=axis)
    if name == "move_exp_nancov":
        cov = np.abs(np.nan_to_num(oracle.move_exp("move_exp_nancov", a64, b64, alpha=al, axis=axis, ext=True)))
        return (np.sqrt(sq * sqb) + cov) * amp
    va = oracle.move_exp("move_exp_nanvar", a64, alpha=al, axis=axis)
    vb = oracle.move_exp("move_exp_nanvar", b64, alpha=al, axis=axis)
    return np.fmax(1.0, np.fmax(_cond(sq, va), _cond(sqb, vb)) * amp)


# ---- degenerate positions ---------------------------------------------------------------


def _valid(a, b):
    v = ~np.isnan(np.asarray(a, dtype=np.float64))
    if b is not None:
        v &= ~np.isnan(np.asarray(b, dtype=np.float64))
    return v


def move_degenerate(name, a, b, window, axis=-1):
    """move_corr over a window holding a single pair: both variances are 0
    mathematically, the reference's value is the sign of its rounding residue."""
    if name != "move_corr":
        return None
    v = _valid(a, b).astype(np.float64)
    cnt = oracle.move("move_sum", v, window=window, min_count=0, axis=axis)
    return cnt <= 1.5


def exp_degenerate(name, a, b, alpha, min_weight, axis=-1):
    """Positions where the reference's decision rests on rounding noise:
    * variance-like functions while at most one observation has been seen (bias is 0
      mathematically; the reference compares its rounding residue with 0);
    * any function where the running weight equals min_weight to ~1e-12."""
    v = _valid(a, b)
    allow = np.zeros(v.shape, bool)
    if name in ("move_exp_nanvar", "move_exp_nanstd", "move_exp_nancov", "move_exp_nancorr"):
        seen = np.cumsum(np.moveaxis(v, axis, -1), axis=-1)
        allow |= np.moveaxis(seen <= 1, -1, axis)
    al = alpha if not isinstance(alpha, np.ndarray) else alpha.astype(np.float64)
    if isinstance(al, np.ndarray) and al.ndim == 1:
        al_full = np.broadcast_to(np.moveaxis(np.broadcast_to(al, np.moveaxis(v, axis, -1).shape), -1, axis), v.shape)
    else:
        al_full = np.broadcast_to(al, v.shape)
    w_in = np.where(v, al_full, np.nan)
    weight = oracle.move_exp("move_exp_nansum", w_in, alpha=al, axis=axis)
    weight = np.where(np.isnan(weight), 0.0, weight)
    allow |= np.abs(weight - min_weight) <= 1e-12 * max(1.0, abs(min_weight))
    return allow


def move_unresolved(name, a, b, window, k=64, axis=-1):
    """Positions where float64 cannot resolve a window variance that the decision
    rests on: move_std's sqrt of a negative residue (numbagg/moving.py:147-150) and
    move_corr's `var_a * var_b > 0` (numbagg/moving.py:266-272) test a difference of
    two numbers of size mean(x^2), so a true (pairwise) variance within k ulps of
    mean(x^2) makes the NaN decision rounding noise in any float64 evaluation."""
    if name not in ("move_std", "move_var", "move_corr", "move_cov"):
        return None
    v = _valid(a, b)
    res = k * np.finfo(np.float64).eps
    out = np.zeros(v.shape, bool)
    for x in (a, b) if b is not None else (a,):
        xm = np.where(v, np.asarray(x, dtype=np.float64), np.nan)
        var = oracle.move("move_var", xm, window=window, min_count=2, axis=axis, ext=True)
        msq = oracle.move("move_mean", xm * xm, window=window, min_count=1, axis=axis)
        with np.errstate(invalid="ignore"):
            out |= var <= res * msq
    return out


def exp_unresolved(name, a, b, alpha, k=256, axis=-1):
    """The same for the exponentially weighted variance family: a weighted variance
    within k ulps of the weighted mean of x^2 (numbagg/moving_exp.py:145-156,
    :320-335)."""
    if name not in ("move_exp_nanvar", "move_exp_nanstd", "move_exp_nancov", "move_exp_nancorr"):
        return None
    v = _valid(a, b)
    res = k * np.finfo(np.float64).eps
    al = alpha if not isinstance(alpha, np.ndarray) else alpha.astype(np.float64)
    out = np.zeros(v.shape, bool)
    for x in (a, b) if b is not None else (a,):
        xm = np.where(v, np.asarray(x, dtype=np.float64), np.nan)
        var = oracle.move_exp("move_exp_nanvar", xm, alpha=al, axis=axis, ext=True)
        msq = oracle.move_exp("move_exp_nanmean", xm * xm, alpha=al, axis=axis)
        with np.errstate(invalid="ignore"):
            out |= var <= res * msq
    return out
