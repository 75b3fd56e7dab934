"""Ragged batches against numbagg's functions applied series by series (the oracle).

Series of uneven length (including empty ones and ones shorter than the window) sit
back to back in one flat buffer; every result must equal what the per-series call
gives: the same parity bound as the rectangular tests for the plain form, the stated
2e-6 for the FP32-compensated form, bit-exact counts.  RaggedMix replays its captured
graph and must reproduce the direct calls bit for bit.
"""

import numpy as np
import pytest
import torch

import numbagg_gb300 as nb
import oracle
from tests.parity import F64_TOL, assert_parity, exp_degenerate, exp_scale, move_scale, scaled_error

pytestmark = pytest.mark.gpu


def _batch(seed, nseries=40, max_len=9000, p_nan=0.05):
    rng = np.random.default_rng(seed)
    lens = rng.integers(0, max_len, size=nseries)
    lens[:3] = [0, 1, 7]  # empty, single, shorter than the windows
    offsets = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    values = rng.standard_normal(offsets[-1])
    values[rng.random(values.shape) < p_nan] = np.nan
    labels = rng.integers(-1, 70, size=offsets[-1]).astype(np.int32)
    return values, labels, offsets


def _series(x, offsets):
    return [x[offsets[s] : offsets[s + 1]] for s in range(len(offsets) - 1)]


def _dev(values, labels, offsets):
    return (torch.from_numpy(values).cuda(), torch.from_numpy(labels).cuda(), torch.from_numpy(offsets).cuda())


@pytest.mark.parametrize("precision", ["f64", "fp32c"])
@pytest.mark.parametrize("fname", ["move_sum", "move_mean", "move_var", "move_std"])
def test_ragged_move(fname, precision):
    values, labels, offsets = _batch(41)
    v, _, o = _dev(values, labels, offsets)
    for window, mc in ((20, 20), (300, 150)):
        got = getattr(nb.ragged, fname)(v, o, window=window, min_count=mc, precision=precision).cpu().numpy()
        for s, (xs, gs) in enumerate(zip(_series(values, offsets), _series(got, offsets))):
            if xs.size == 0:
                continue
            # a window longer than the series covers it all, like window = len
            w = min(window, xs.size)
            ext = oracle.move(fname, xs[None], window=w, min_count=mc, ext=True)[0]
            r = scaled_error(gs, ext, move_scale(fname, xs[None], None, w)[0])
            assert r["nan_mismatch"] == 0, (fname, s, r)
            assert r["max_err"] <= (F64_TOL if precision == "f64" else 2e-6), (fname, s, window, r)


@pytest.mark.parametrize("precision", ["f64", "fp32c"])
@pytest.mark.parametrize("fname", ["move_exp_nanmean", "move_exp_nanvar", "move_exp_nanstd"])
def test_ragged_move_exp(fname, precision):
    values, labels, offsets = _batch(42, max_len=5000)
    v, _, o = _dev(values, labels, offsets)
    got = getattr(nb.ragged, fname)(v, o, alpha=0.05, precision=precision).cpu().numpy()
    for s, (xs, gs) in enumerate(zip(_series(values, offsets), _series(got, offsets))):
        if xs.size == 0:
            continue
        want = oracle.move_exp(fname, xs[None], alpha=0.05)[0]
        ext = oracle.move_exp(fname, xs[None], alpha=0.05, ext=True)[0]
        scale = exp_scale(fname, xs[None], None, 0.05)[0]
        allow = exp_degenerate(fname, xs[None], None, 0.05, 0.0)[0]
        if precision == "f64":  # the same bar as the rectangular parity tests
            assert_parity(gs, want, ext, scale, F64_TOL, allow, f"{fname} series {s}")
        else:
            r = scaled_error(gs, ext, scale, allow)
            assert r["nan_mismatch"] == 0 and r["max_err"] <= 2e-6, (fname, s, r)


@pytest.mark.parametrize("fname", ["group_nansum", "group_nanmean", "group_nancount"])
def test_ragged_group(fname):
    values, labels, offsets = _batch(43, max_len=20000)
    v, lab, o = _dev(values, labels, offsets)
    got = getattr(nb.ragged, fname)(v, lab, o, num_labels=64).cpu().numpy()
    for s, (xs, ls) in enumerate(zip(_series(values, offsets), _series(labels, offsets))):
        want = oracle.group(fname, xs, ls.astype(np.int64), num_labels=64) if xs.size else None
        if want is None:
            assert (got[s] == 0).all() if fname != "group_nanmean" else np.isnan(got[s]).all()
            continue
        if fname == "group_nancount":
            assert np.array_equal(got[s], want), s
        else:
            scale = np.nanmax(np.abs(want)) if np.isfinite(want).any() else 1.0
            r = scaled_error(got[s], want, scale)
            assert r["nan_mismatch"] == 0 and r["max_err"] <= F64_TOL, (fname, s, r)


def test_ragged_mix_graph_replays_the_direct_calls():
    values, labels, offsets = _batch(44, nseries=300, max_len=30000)
    v, lab, o = _dev(values, labels, offsets)
    mix = nb.ragged.RaggedMix(v, lab, o, window=20, alpha=0.05, num_labels=64)
    mean, std, groups = mix.run()
    torch.cuda.synchronize()
    assert torch.equal(torch.nan_to_num(mean, nan=9.0), torch.nan_to_num(nb.ragged.move_mean(v, o, window=20), nan=9.0))
    assert torch.equal(torch.nan_to_num(std, nan=9.0), torch.nan_to_num(nb.ragged.move_exp_nanstd(v, o, alpha=0.05), nan=9.0))
    assert torch.equal(torch.nan_to_num(groups, nan=9.0), torch.nan_to_num(nb.ragged.group_nanmean(v, lab, o, num_labels=64), nan=9.0))
    # refilled inputs flow through the same graph
    v.mul_(2.0)
    mean2, _, _ = mix.run()
    torch.cuda.synchronize()
    assert torch.equal(torch.nan_to_num(mean2, nan=9.0), torch.nan_to_num(nb.ragged.move_mean(v, o, window=20), nan=9.0))


def _eq(a, b):
    return torch.equal(torch.nan_to_num(a, nan=9.0), torch.nan_to_num(b, nan=9.0))


def test_ragged_plan_many_requests_one_graph():
    values, labels, offsets = _batch(45, nseries=200, max_len=20000)
    v, lab, o = _dev(values, labels, offsets)
    requests = [
        ("move_mean", {"window": 20}),
        ("move_std", {"window": 252, "min_count": 100}),
        ("move_exp_nanmean", {"alpha": 0.3}),
        ("move_exp_nanstd", {"alpha": 0.05}),
        ("group_nansum", {"num_labels": 70}),
        ("group_nancount", {"num_labels": 16}),
    ]
    for precision in ("f64", "fp32c"):
        plan = nb.ragged.RaggedPlan(v, o, requests, labels=lab, precision=precision)
        outs = plan.run()
        torch.cuda.synchronize()
        assert _eq(outs[0], nb.ragged.move_mean(v, o, window=20, precision=precision))
        assert _eq(outs[1], nb.ragged.move_std(v, o, window=252, min_count=100, precision=precision))
        assert _eq(outs[2], nb.ragged.move_exp_nanmean(v, o, alpha=0.3, precision=precision))
        assert _eq(outs[3], nb.ragged.move_exp_nanstd(v, o, alpha=0.05, precision=precision))
        assert _eq(outs[4], nb.ragged.group_nansum(v, lab, o, num_labels=70))
        assert _eq(outs[5], nb.ragged.group_nancount(v, lab, o, num_labels=16))


def test_ragged_plans_over_slices_share_outputs():
    # a batch cut into two slices of series, each its own plan writing into views of one
    # pair of output buffers (how a batch larger than the device's room is streamed)
    values, labels, offsets = _batch(46, nseries=120, max_len=20000)
    v, lab, o = _dev(values, labels, offsets)
    longest = max(int(offsets[60] - offsets[0]), int(offsets[120] - offsets[60]))
    mean_buf = torch.empty(longest, dtype=torch.float64, device="cuda")
    std_buf = torch.empty_like(mean_buf)
    results = []
    for s0, s1 in ((0, 60), (60, 120)):
        e0, e1 = int(offsets[s0]), int(offsets[s1])
        vo = v[e0:e1]
        oo = o[s0 : s1 + 1] - o[s0]
        mix = nb.ragged.RaggedMix(vo, lab[e0:e1], oo, window=20, alpha=0.05, num_labels=70,
                                  outs=[mean_buf[: e1 - e0], std_buf[: e1 - e0], None])
        mean, std, groups = mix.run()
        torch.cuda.synchronize()
        results.append((mean.clone(), std.clone(), groups.clone()))
    full_mean = nb.ragged.move_mean(v, o, window=20)
    full_std = nb.ragged.move_exp_nanstd(v, o, alpha=0.05)
    full_groups = nb.ragged.group_nanmean(v, lab, o, num_labels=70)
    assert _eq(torch.cat([results[0][0], results[1][0]]), full_mean)
    assert _eq(torch.cat([results[0][1], results[1][1]]), full_std)
    assert _eq(torch.cat([results[0][2], results[1][2]]), full_groups)
