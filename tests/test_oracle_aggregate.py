"""The static-aggregation oracle pinned to the reference's own expectations, and the
host-side argument checks of ``numbagg_gb300``'s aggregations (no GPU needed).

numbagg's tests compare these functions with numpy's nan-functions
(numbagg/test/test_funcs.py:128-141: nansum/np.nansum, nanmax/np.nanmax,
nanargmin/np.nanargmin, nanargmax/np.nanargmax, nanmin/np.nanmin, nanmean/np.nanmean,
nanstd and nanvar with ddof=1, nancount as a sum of ~isnan) and pin allnan / anynan
on small arrays (numbagg/test/test_funcs.py:255-325).  The same comparisons pin the
oracle here.
"""

import os
import warnings

import numpy as np
import pytest

import numbagg_gb300 as nb
import oracle

COMPARISONS = [
    ("nansum", np.nansum, {}),
    ("nanmax", np.nanmax, {}),
    ("nanargmin", np.nanargmin, {}),
    ("nanargmax", np.nanargmax, {}),
    ("nanmin", np.nanmin, {}),
    ("nanmean", np.nanmean, {}),
    ("nanstd", np.nanstd, {"ddof": 1}),
    ("nanvar", np.nanvar, {"ddof": 1}),
    ("nancount", lambda x, axis=None: np.sum(~np.isnan(x), axis=axis), {}),
]


def _arrays():
    rng = np.random.default_rng(7)
    a = rng.standard_normal((3, 4, 50))
    a[rng.random(a.shape) < 0.2] = np.nan
    yield a
    yield a.astype(np.float32)
    yield np.arange(24, dtype=np.float64).reshape(2, 3, 4)
    yield np.array([1.0, np.nan, -np.inf, 3.0])
    yield np.array([[np.nan, np.nan], [1.0, np.nan]])
    yield rng.integers(-50, 50, size=(5, 7)).astype(np.int32)


def _call(fn):
    try:
        return fn(), None
    except ValueError as err:
        return None, str(err)


@pytest.mark.parametrize("name,numpy_fn,kw", COMPARISONS)
def test_oracle_matches_numpy(name, numpy_fn, kw):
    warnings.simplefilter("ignore")
    for a in _arrays():
        for axis in list(range(-a.ndim, a.ndim)) + [None]:
            got, gerr = _call(lambda: oracle.aggregate(name, a, axis=axis, **kw))
            want, werr = _call(lambda: numpy_fn(a, axis=axis, **kw))
            assert (gerr is None) == (werr is None), (name, a.dtype, axis, gerr, werr)
            if gerr is not None:
                assert gerr == werr or "All-NaN" in gerr
                continue
            np.testing.assert_allclose(np.asarray(got, dtype=np.float64), np.asarray(want, dtype=np.float64),
                                       rtol=1e-5 if a.dtype == np.float32 else 1e-12, equal_nan=True)


def test_oracle_tuple_axes_match_numpy():
    warnings.simplefilter("ignore")
    a = next(_arrays())
    for axis in [(0, 2), (2, 0), (-1, -2), (0,)]:
        np.testing.assert_allclose(oracle.aggregate("nansum", a, axis=axis), np.nansum(a, axis=axis))
        np.testing.assert_allclose(oracle.aggregate("nanvar", a, axis=axis), np.nanvar(a, axis=axis, ddof=1),
                                   rtol=1e-12)


def test_oracle_allnan_anynan_reference_cases():
    assert oracle.aggregate("allnan", np.array([np.nan, np.nan, np.nan]))
    assert oracle.aggregate("allnan", np.array([np.nan]))
    assert not oracle.aggregate("allnan", np.array([1.0, 2.0, 3.0]))
    assert not oracle.aggregate("allnan", np.array([np.nan, 1.0, np.nan]))
    assert not oracle.aggregate("anynan", np.array([1.0, 2.0, 3.0]))
    assert oracle.aggregate("anynan", np.array([np.nan, np.nan]))
    np.testing.assert_array_equal(
        oracle.aggregate("allnan", np.array([[np.nan, np.nan], [1.0, np.nan], [np.nan, np.nan]]), axis=1),
        [True, False, True],
    )
    np.testing.assert_array_equal(
        oracle.aggregate("anynan", np.array([[1.0, 2.0], [1.0, np.nan], [3.0, 4.0]]), axis=1), [False, True, False]
    )


def test_oracle_dtypes_follow_the_reference_loops():
    assert oracle.aggregate("nansum", np.ones(3, np.int32)).dtype == np.int32
    assert oracle.aggregate("nansum", np.ones(3, np.int16)).dtype == np.int32
    assert oracle.aggregate("nansum", np.ones(3, np.float16)).dtype == np.float32
    assert oracle.aggregate("nanmean", np.ones(3, np.int64)).dtype == np.float64
    assert oracle.aggregate("nanmean", np.ones(3, np.int16)).dtype == np.float32
    assert oracle.aggregate("nancount", np.ones(3)).dtype == np.int64
    # integer sums wrap like the int32 loop
    big = np.full(4, 2**30, np.int32)
    assert oracle.aggregate("nansum", big) == np.int32(0)


# ---- host-side checks of the CUDA package (raised before any device work) ----------------


def test_empty_reductions_raise_like_numbagg():
    empty = np.empty((3, 0))
    with pytest.raises(ValueError, match="zero-size array to reduction operation fmax"):
        nb.nanmax(empty, axis=1)
    with pytest.raises(ValueError, match="zero-size array to reduction operation fmin"):
        nb.nanmin(empty, axis=1)
    with pytest.raises(ValueError, match="All-NaN slice encountered"):
        nb.nanargmax(empty, axis=1)
    with pytest.raises(ValueError, match="All-NaN slice encountered"):
        nb.nanargmin(empty, axis=1)


def test_bad_axis_and_dtype_raise():
    a = np.ones((2, 3))
    with pytest.raises(np.exceptions.AxisError):
        nb.nansum(a, axis=2)
    with pytest.raises(ValueError, match="repeated axis"):
        nb.nansum(a, axis=(1, -1))
    with pytest.raises(TypeError):
        nb.nanmean(np.array(["a", "b"]))
    with pytest.raises(TypeError):
        nb.nanvar(a, ddof=1.5)


def test_aggregation_category_list():
    assert nb.count is nb.nancount
    assert {f.__name__ for f in nb.AGGREGATION_FUNCS} >= {
        "allnan", "anynan", "nanargmax", "nanargmin", "nancount", "nanmax", "nanmean", "nanmin", "nanstd",
        "nansum", "nanvar",
    }


# ---- pinned to the reference's own kernel bodies (tests/golden/make_golden.py) -----------

_GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "aggregate_vectors.npz")


def _golden():
    with np.load(_GOLDEN) as z:
        return {k: z[k] for k in z.files}


def test_oracle_matches_reference_bodies_bit_for_bit():
    """numbagg's own funcs.py bodies, run as Python behind a numba stub, against the
    oracle on the same rows: identical values (NaN where NaN), dtypes included."""
    warnings.simplefilter("ignore")
    g = _golden()
    checked = 0
    for key, want in g.items():
        parts = key.split("|")
        if parts[0] != "agg":
            continue
        _, name, inp, extra = parts
        if extra == "rows":
            continue
        a = g[f"agg_in|{inp}"]
        if name in ("nanmax", "nanmin", "nanargmax", "nanargmin"):
            a = a[g[f"agg|{name}|{inp}|rows"]]
            got = oracle.aggregate(name, a, axis=-1)
        elif name in ("nanvar", "nanstd"):
            got = oracle.aggregate(name, a, axis=-1, ddof=int(extra))
        else:
            got = oracle.aggregate(name, a, axis=-1)
        got = np.asarray(got)
        assert got.dtype == want.dtype, (key, got.dtype, want.dtype)
        np.testing.assert_array_equal(got, want, err_msg=key)
        checked += 1
    assert checked >= 60
