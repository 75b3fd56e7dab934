"""Host-side logic that needs no GPU: the ragged module's input checks and its
autotuning cache, and the benchmark's byte accounting and peak / traffic lookups."""

import importlib.util
import json
import os

import numpy as np
import pytest
import torch

from numbagg_gb300 import ragged

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench():
    spec = importlib.util.spec_from_file_location("bench_module", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


# ---- ragged -------------------------------------------------------------------------------


def test_ragged_rejects_host_tensors_and_bad_dtypes():
    values = torch.zeros(10, dtype=torch.float64)
    offsets = torch.tensor([0, 4, 10], dtype=torch.int64)
    with pytest.raises(TypeError, match="values must be a 1-D float64 CUDA tensor"):
        ragged.move_mean(values, offsets, window=3)
    with pytest.raises(TypeError, match="values must be a 1-D float64 CUDA tensor"):
        ragged.group_nansum(values.float(), torch.zeros(10, dtype=torch.int32), offsets, num_labels=2)


def test_ragged_precision_keyword():
    assert ragged._sfx("f64") == "f64"
    assert ragged._sfx("fp32c") == "f64_fp32c"
    with pytest.raises(ValueError, match="precision must be one of"):
        ragged._sfx("fp16")


def test_autotune_shape_buckets():
    k = ragged._shape_key("move_mean", "f64", 20_000, 1_830_000_000, 20, "GB300|sm152|cc103")
    assert k == ragged._shape_key("move_mean", "f64", 30_000, 2_000_000_000, 20, "GB300|sm152|cc103")  # same buckets
    assert k != ragged._shape_key("move_mean", "f64", 40_000, 2_000_000_000, 20, "GB300|sm152|cc103")
    assert k != ragged._shape_key("move_mean", "fp32c", 20_000, 1_830_000_000, 20, "GB300|sm152|cc103")
    assert k != ragged._shape_key("move_mean", "f64", 20_000, 1_830_000_000, 21, "GB300|sm152|cc103")
    # a choice made on one GPU model is not reused on another
    assert k != ragged._shape_key("move_mean", "f64", 20_000, 1_830_000_000, 20, "B200|sm148|cc100")


def test_autotune_cache_round_trip(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    monkeypatch.setattr(ragged, "_CACHE_FILE", str(path))
    monkeypatch.setattr(ragged, "_cache", {"move_mean|f64|s14|n30|w20": 32768})
    ragged._save_cache()
    assert json.loads(path.read_text()) == {"move_mean|f64|s14|n30|w20": 32768}
    monkeypatch.setattr(ragged, "_cache", {})
    ragged._load_cache()
    assert ragged._cache == {"move_mean|f64|s14|n30|w20": 32768}
    # a save merges with what other processes wrote meanwhile, and leaves no temporary
    path.write_text(json.dumps({"other|key": 8192, "move_mean|f64|s14|n30|w20": 1}))
    ragged._save_cache()
    assert json.loads(path.read_text()) == {"other|key": 8192, "move_mean|f64|s14|n30|w20": 32768}
    assert sorted(p.name for p in tmp_path.iterdir()) == ["tune.json"]
    path.write_text("not json")
    monkeypatch.setattr(ragged, "_cache", {})
    ragged._load_cache()  # a corrupt file is ignored
    assert ragged._cache == {}


def test_ragged_requests_are_checked():
    assert ragged.check_request("move_mean", {"window": 20}) == ("move_mean", {"window": 20})
    with pytest.raises(ValueError, match="unknown ragged function"):
        ragged.check_request("move_median", {"window": 3})
    with pytest.raises(TypeError, match="unexpected keywords"):
        ragged.check_request("move_exp_nanmean", {"alpha": 0.1, "window": 3})
    with pytest.raises(TypeError, match="needs"):
        ragged.check_request("group_nanmean", {})


# ---- bench --------------------------------------------------------------------------------


def test_bench_byte_accounting():
    b = _bench()
    rows, cols = 64, 1 << 20
    calls = b.calls_and_bytes(rows, cols)
    assert len(calls) == 19
    keys = [c[0] for c in calls]
    assert len(set(keys)) == 19
    for key, (kind, f, arg), nbytes in calls:
        if kind == "fill":
            assert nbytes == 16 * rows * cols  # read + write
        else:
            assert nbytes == 8 * rows * cols + 4 * cols + 8 * rows * arg  # values + labels + output


def test_bench_peak_and_traffic_lookups(tmp_path, monkeypatch):
    b = _bench()
    monkeypatch.setattr(b, "ROOT", str(tmp_path))
    assert b.measured_peak() == (6800.0, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"hbm_gbs": 6781.8}))
    assert b.measured_peak() == (6781.8, "measured")
    assert b.traffic_for("group_nanvar_K1000000") is None
    (tmp_path / "profiles").mkdir()
    (tmp_path / "profiles" / "traffic.json").write_text(json.dumps({"group_nanvar_K1000000": 123}))
    assert b.traffic_for("group_nanvar_K1000000") == 123


def test_committed_traffic_covers_the_dominant_call():
    with open(os.path.join(ROOT, "profiles", "traffic.json")) as fh:
        data = json.load(fh)
    assert isinstance(data.get("group_nanvar_K1000000"), int)
    assert data["group_nanvar_K1000000"] > 9_169_043_456  # at least the algorithmic bytes


def test_bench_cpu_sample_is_a_prefix_of_the_workload():
    b = _bench()
    rows, cols = 4, 4096
    values = torch.arange(rows * cols, dtype=torch.float64).reshape(rows, cols)
    labels = {K: torch.zeros(cols, dtype=torch.int32) for K in b.KS}
    fill = values.clone()
    v, lab, fl, sc = b.cpu_sample(values, labels, fill, cols)
    assert sc <= cols
    np.testing.assert_array_equal(np.asarray(v), values[:, :sc].numpy())
    assert b.sample_bytes(rows, sc) > 0
    assert str(sc) in b.sample_desc(rows, sc)


def test_in_place_layouts():
    import torch

    from numbagg_gb300 import _host
    from numbagg_gb300.aggregate import middle_inner

    # scans: a non-last axis of a C-contiguous array with enough columns
    t = torch.empty((100, 32768), dtype=torch.float64)
    assert _host.column_layout(t, 0) == (1, 100, 32768)
    assert _host.column_layout(t, 1) is None  # the last axis: the rows kernels
    assert _host.column_layout(torch.empty((3, 50, 11000), dtype=torch.float64), 1) == (3, 50, 11000)
    assert _host.column_layout(torch.empty((100, 7)), 0) is None  # too few columns
    assert _host.column_layout(torch.empty((4096, 100)).T, 0) is None  # not contiguous
    # the in-place kernels need 256 KB of columns per position to beat the copy
    assert _host.column_min(8) == 32768 and _host.column_min(4) == 65536
    assert _host.column_layout(torch.empty((100, 16384), dtype=torch.float64), 0) is None
    assert _host.column_layout(torch.empty((100, 32768), dtype=torch.float32), 0) is None
    assert _host.column_layout(torch.empty((100, 16384), dtype=torch.float64), 0, 2048) == (1, 100, 16384)
    # static aggregations: consecutive middle axes, increasing, not last
    assert middle_inner((4, 40, 50, 64), (1, 2)) == 64
    assert middle_inner((4, 40, 50, 64), (0,)) == 40 * 50 * 64
    assert middle_inner((4, 40, 50, 64), (2, 1)) is None  # order matters for argmax
    assert middle_inner((4, 40, 50, 64), (1, 3)) is None  # not consecutive
    assert middle_inner((4, 40, 50, 64), (2, 3)) is None  # includes the last axis
    assert middle_inner((400, 8), (0,)) is None  # fewer outputs than a warp
    assert middle_inner((5,), ()) is None
    # grouped reductions: consecutive increasing reduced axes, not the last one
    from numbagg_gb300.grouped import group_columns_layout

    assert group_columns_layout((700, 32768), (0,)) == (1, 700, 32768)
    assert group_columns_layout((3, 40, 50, 11000), (1, 2)) == (3, 2000, 11000)
    assert group_columns_layout((3, 40, 50, 11000), (2, 1)) is None  # the labels' order would change
    assert group_columns_layout((3, 40, 50, 11000), (2, 3)) is None  # includes the last axis
    assert group_columns_layout((3, 40, 50, 11000), (0, 2)) is None  # not consecutive
    assert group_columns_layout((700, 4096), (0,)) is None  # too few columns to beat the copy
    assert group_columns_layout((700, 32768), (0,), itemsize=4) is None  # float32 needs twice as many
    assert group_columns_layout((700, 32768), None) is None  # labels over every axis
