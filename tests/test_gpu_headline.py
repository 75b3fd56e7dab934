"""Parity of the kernels the benchmark's workloads actually run, at their shapes.

* Grouped reductions over 64 rows with K = 4,096 and K = 10^6 labels (the headline's
  row count: the row-blocked large-K kernels take 16, 8, 4 or 2 rows per block from
  the row count and K, and three rows never reach those instantiations), a 17-row
  case whose last row block is partial, and a K where eight rows fit one block.
* The rolling matrices at 256 variables, window 500, min_count 400, float32.
* The precision-stress data (1e6 + N(0, 1), correlated pairs, 2% NaN) in plain
  float64, for move_std / move_corr and move_exp_nanmean / nanvar / nancorr, each
  result's error against the extended-precision oracle printed beside the
  reference's own.

Reference loops: numbagg/grouped.py:7-92, :148-176; numbagg/moving_matrix.py:16-201;
numbagg/moving.py:123-151, :223-275; numbagg/moving_exp.py:41-156, :275-335.
"""

import numpy as np
import pytest
import torch

import numbagg_gb300 as nb
import oracle
from tests.parity import (
    F64_TOL,
    assert_bit_equal,
    assert_parity,
    assert_scaled_close,
    exp_degenerate,
    exp_scale,
    exp_unresolved,
    move_degenerate,
    move_scale,
    move_unresolved,
    parity_error,
)

pytestmark = pytest.mark.gpu

HEADLINE_FUNCS = ["group_nansum", "group_nanmean", "group_nanvar", "group_nancount", "group_nanargmax"]


def _group_case(rows, m, K, seed):
    rng = np.random.default_rng(seed)
    values = rng.standard_normal((rows, m))
    values[rng.random(values.shape) < 0.05] = np.nan
    values[:, :64] = np.round(values[:, :64])  # ties for the selections
    labels = rng.integers(0, K, size=m).astype(np.int32)
    labels[rng.random(m) < 0.01] = -1  # skipped labels
    return values, labels


def _group_scale(fname, values, labels, K):
    absv = np.where(np.isnan(values), 0.0, np.abs(values))
    lab = np.where(labels >= 0, labels, K)
    rows = values.shape[0]
    s1 = np.stack([np.bincount(lab, weights=absv[r], minlength=K + 1)[:K] for r in range(rows)])
    s2 = np.stack([np.bincount(lab, weights=absv[r] ** 2, minlength=K + 1)[:K] for r in range(rows)])
    cnt = np.stack([np.bincount(lab, weights=(~np.isnan(values[r])).astype(float), minlength=K + 1)[:K] for r in range(rows)])
    return {
        "group_nansum": s1,
        "group_nanmean": s1 / np.maximum(cnt, 1),
        "group_nanvar": s2 / np.maximum(cnt, 1),
        "group_nanstd": np.sqrt(s2 / np.maximum(cnt, 1)),
        "group_nansum_of_squares": s2,
    }[fname]


def _check_group(fname, values, labels, K, what):
    vt = torch.from_numpy(values).cuda()
    lt = torch.from_numpy(labels).cuda()
    got = getattr(nb, fname)(vt, lt, num_labels=K, axis=-1).cpu().numpy()
    want = oracle.group(fname, values, labels, num_labels=K, axis=-1)
    if fname in ("group_nancount", "group_nanargmax", "group_nanargmin"):
        assert_bit_equal(got, want, what)
    else:
        assert_scaled_close(got, want, _group_scale(fname, values, labels, K), F64_TOL, None, what)


@pytest.mark.parametrize("K", [4096, 1_000_000])
@pytest.mark.parametrize("fname", HEADLINE_FUNCS)
def test_group_headline_rows(fname, K):
    values, labels = _group_case(64, 262_144, K, 41)
    _check_group(fname, values, labels, K, f"{fname} K={K} 64 rows")


@pytest.mark.parametrize("fname", HEADLINE_FUNCS)
def test_group_partial_row_block(fname):
    # 17 rows: with K = 4096 the large-K kernels take 16 rows per block, so the second
    # block holds one row
    values, labels = _group_case(17, 150_001, 4096, 42)
    _check_group(fname, values, labels, 4096, f"{fname} 17 rows")


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int32, np.int64])
@pytest.mark.parametrize("fname", ["group_nanargmax", "group_nanargmin", "group_nanmax", "group_nanmin"])
def test_group_large_k_selection_ties(fname, dtype):
    # K = 200,000 takes the one-pass (key, column) pair updates in L2.  Values from seven
    # levels make nearly every bin a tie that the smallest column must win (signed zeros
    # included, which compare equal), and one label holding a tenth of the columns makes
    # its bins contended, so swaps race and retry.
    rng = np.random.default_rng(45)
    rows, m, K = 8, 400_000, 200_000
    x = rng.integers(-3, 4, size=(rows, m)).astype(dtype)
    if np.issubdtype(dtype, np.floating):
        x[(x == 0) & (rng.random(x.shape) < 0.5)] = -0.0
        x[rng.random(x.shape) < 0.05] = np.nan
    labels = rng.integers(0, K, size=m).astype(np.int32)
    labels[rng.random(m) < 0.1] = 7
    labels[rng.random(m) < 0.01] = -1
    got = getattr(nb, fname)(torch.from_numpy(x).cuda(), torch.from_numpy(labels).cuda(), num_labels=K,
                             axis=-1).cpu().numpy()
    want = oracle.group(fname, x, labels, num_labels=K, axis=-1)
    assert_bit_equal(got, want, f"{fname} {np.dtype(dtype)} K={K}")


@pytest.mark.parametrize("fname", ["group_nanvar", "group_nansum", "group_nanargmax"])
def test_group_eight_rows_per_block(fname):
    # K = 300,000: a variance's 20 bytes per (row, label) fit eight rows in a block
    values, labels = _group_case(64, 131_072, 300_000, 43)
    _check_group(fname, values, labels, 300_000, f"{fname} K=300000")


@pytest.mark.parametrize("fname", ["move_covmatrix", "move_corrmatrix"])
def test_move_matrix_256_vars(fname):
    # X = Z (A / 16)^T: rows drawn from N(0, A A^T / 256); 1% NaN; window 500, min_count 400
    rng = np.random.default_rng(4)
    T, V = 1100, 256
    A = rng.standard_normal((V, V))
    x = (rng.standard_normal((T, V)) @ (A / 16).T).astype(np.float32)
    x[rng.random(x.shape) < 0.01] = np.nan
    got = getattr(nb, fname)(torch.from_numpy(x).cuda(), window=500, min_count=400).cpu().numpy()
    want = oracle.move_matrix(fname, x, window=500, min_count=400)
    ext = oracle.move_matrix(fname, x.astype(np.float64), window=500, min_count=400, ext=True)
    assert got.shape == want.shape == (T, V, V) and got.dtype == np.float32
    # compared in slabs of time to keep the host's temporaries small
    for t0 in range(0, T, 100):
        sl = slice(t0, t0 + 100)
        g, w, e = got[sl], want[sl], ext[sl]
        if fname == "move_covmatrix":
            d = np.abs(np.einsum("tii->ti", np.nan_to_num(e)))
            scale = np.sqrt(d[:, :, None] * d[:, None, :]) + 1e-30
        else:
            scale = np.ones_like(e)
        # both accumulate float32 in float32 (numbagg/moving_matrix.py:149-152), in
        # different orders: 1e-4 of the scale, as for the smaller matrix cases
        assert_parity(g, w, e, scale, 1e-4, None, f"{fname} t={t0}")
    # the first outputs with 400 complete pairs in the window appear near t = 408
    assert np.isnan(got[300]).all() and not np.isnan(got[-1]).all()


def _stress_pair(rows, n, seed):
    rng = np.random.default_rng(seed)
    z1 = rng.standard_normal((rows, n))
    z2 = rng.standard_normal((rows, n))
    a = 1e6 + z1
    b = 1e6 + 0.7 * z1 + np.sqrt(0.51) * z2
    a[rng.random(a.shape) < 0.02] = np.nan
    b[rng.random(b.shape) < 0.02] = np.nan
    return a, b


def _report(what, got, ref, ext):
    fin = ~np.isnan(got) & ~np.isnan(ref) & ~np.isnan(ext)
    rel = lambda x: np.max(np.abs(x[fin] - ext[fin]) / np.maximum(np.abs(ext[fin]), 1e-300)) if fin.any() else 0.0
    print(f"{what}: max relative error vs the extended oracle: gpu {rel(got):.3g}, reference {rel(ref):.3g}")


@pytest.mark.parametrize("window", [5, 252, 10_000])
@pytest.mark.parametrize("fname", ["move_std", "move_corr"])
def test_precision_stress_plain_move(fname, window):
    a, b = _stress_pair(4, 40_000, 3)
    y = b if fname == "move_corr" else None
    mc = max(2, window // 2)
    func = getattr(nb, fname)
    got = (func(a, y, window=window, min_count=mc) if y is not None else func(a, window=window, min_count=mc))
    ref = oracle.move(fname, a, y, window=window, min_count=mc)
    ext = oracle.move(fname, a, y, window=window, min_count=mc, ext=True)
    # where the reference and the extended result disagree on NaN (a variance whose
    # rounding residue in the reference went negative, numbagg/moving.py:147-150), or
    # where the window variance is below what float64 resolves on data of size 1e6,
    # the NaN decision is rounding noise; such positions are allowed and counted
    allow = (np.isnan(ref) != np.isnan(ext)) | move_unresolved(fname, a, y, window)
    deg = move_degenerate(fname, a, y, window)
    if deg is not None:
        allow |= deg
    r = assert_parity(got, ref, ext, move_scale(fname, a, y, window), F64_TOL, allow, f"{fname} w={window}")
    assert r["allowed"] <= 0.01 * r["n"], r
    _report(f"{fname} w={window}", got, ref, ext)
    # the exact window sums make the GPU at least as close to the extended result
    assert r["gpu_vs_ext"] <= max(r["ref_vs_ext"], 1e-14), r


@pytest.mark.parametrize("alpha", [0.5, 0.01, 1e-4])
@pytest.mark.parametrize("fname", ["move_exp_nanmean", "move_exp_nanvar", "move_exp_nancorr"])
def test_precision_stress_plain_exp(fname, alpha):
    a, b = _stress_pair(4, 40_000, 5)
    y = b if fname == "move_exp_nancorr" else None
    func = getattr(nb, fname)
    got = func(a, y, alpha=alpha, min_weight=0) if y is not None else func(a, alpha=alpha, min_weight=0)
    ref = oracle.move_exp(fname, a, y, alpha=alpha, min_weight=0)
    ext = oracle.move_exp(fname, a, y, alpha=alpha, min_weight=0, ext=True)
    allow = exp_degenerate(fname, a, y, alpha, 0.0) | (np.isnan(ref) != np.isnan(ext))
    unresolved = exp_unresolved(fname, a, y, alpha)
    if unresolved is not None:
        allow |= unresolved
    r = assert_parity(got, ref, ext, exp_scale(fname, a, y, alpha), F64_TOL, allow, f"{fname} alpha={alpha}")
    assert r["allowed"] <= 0.01 * r["n"], r
    _report(f"{fname} alpha={alpha}", got, ref, ext)
    info = parity_error(got, ref, ext, exp_scale(fname, a, y, alpha), allow)
    assert info["gpu_vs_ext"] <= max(16 * info["ref_vs_ext"], 1e-12), info
