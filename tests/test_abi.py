"""The C ABI: the library loads, exports every symbol the header declares, and
rejects bad arguments with status codes before touching a device (CPU only)."""

import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "numbagg_gb300.h")


@pytest.fixture(scope="module")
def lib():
    from numbagg_gb300 import _build, _lib

    if not os.path.exists(_lib.LIB_PATH):
        _build.build()
    return _lib.lib()


def _declared_symbols():
    expanded = subprocess.run(
        ["gcc", "-E", "-P", "-x", "c", HEADER], capture_output=True, text=True, check=True
    ).stdout
    return sorted(set(re.findall(r"\b(nbg_[A-Za-z0-9_]+)\s*\(", expanded)))


def _exported_symbols(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    return sorted({line.split()[-1] for line in out.splitlines() if " T " in line and "nbg_" in line})


def test_header_matches_exports(lib):
    from numbagg_gb300 import _lib

    declared = _declared_symbols()
    assert len(declared) > 100
    exported = _exported_symbols(_lib.LIB_PATH)
    assert declared == exported
    for name in declared:
        assert hasattr(lib, name), name


def test_status_strings(lib):
    assert lib.nbg_version() >= 10000
    assert lib.nbg_status_string(0) == b"ok"
    assert lib.nbg_status_string(3) == b"workspace missing or too small"
    assert lib.nbg_workspace_header_bytes() == 256


def test_invalid_arguments_are_rejected_before_launch(lib):
    null = None
    # negative sizes / window / limit are argument errors, no CUDA call is made
    assert lib.nbg_move_mean_f64(null, null, -1, 10, 3, 3, null, 0, null) == 1
    assert lib.nbg_move_mean_f64(null, null, 1, 10, 0, 3, null, 0, null) == 1
    assert lib.nbg_move_corr_f32(null, null, null, 1, 10, 3, -1, null, 0, null) == 1
    assert lib.nbg_ffill_f64(null, null, 1, 10, -1, null, 0, null) == 1
    assert lib.nbg_move_exp_nanmean_f64(null, null, 0.5, 7, 0.0, null, 1, 10, null, 0, null) == 1
    assert lib.nbg_group_nansum_f64_i32(null, null, null, -1, 10, 4, 1, null, 0, null) == 1
    assert lib.nbg_move_covmatrix_f64(null, null, 1, 10, 3, 0, 1, null) == 1
    assert lib.nbg_move_std_cols_f64(null, null, 1, 10, 4, 0, 3, null) == 1
    assert lib.nbg_move_corr_cols_f32(null, null, null, 1, 10, 4, 3, -1, null) == 1
    assert lib.nbg_move_mean_cols_f64(null, null, 0, 10, 4, 3, 3, null) == 0
    assert lib.nbg_group_nanargmax_cols_i32_i64(null, null, null, 1, -1, 4, 3, 1, null) == 1
    assert lib.nbg_group_nanvar_cols_f32_i32(null, null, null, 0, 10, 4, 3, 1, null) == 0
    assert lib.nbg_group_nansum_cols_f64_i32(null, null, null, 2, 10, 4, 97, 1, null) == 1  # no output
    # empty problems succeed without work
    assert lib.nbg_move_mean_f64(null, null, 0, 10, 3, 3, null, 0, null) == 0
    assert lib.nbg_ffill_f32(null, null, 3, 0, 2, null, 0, null) == 0
    # a scan with work but no workspace reports it
    buf = (ctypes.c_double * 8)()
    assert lib.nbg_move_sum_f64(ctypes.addressof(buf), ctypes.addressof(buf), 1, 8, 2, 1, null, 0, null) == 3


def test_workspace_queries(lib):
    small = lib.nbg_move_workspace_bytes(1, 10)
    big = lib.nbg_move_workspace_bytes(1024, 1 << 20)
    assert 256 < small < big
    assert lib.nbg_fill_workspace_bytes(64, 1 << 24) > lib.nbg_fill_workspace_bytes(64, 1 << 10)
    assert lib.nbg_group_workspace_bytes(0, 4, 1000, 16) >= 4 * 16 * 24
    assert lib.nbg_group_workspace_bytes(99, 4, 1000, 16) == 0
    # in-place grouped column kernels: shared-memory bins of 8, 16 or 24 bytes per
    # (label, column) for 128 columns within 96 KB (numbering of nbg_group_workspace_bytes)
    ids = {"nansum": 0, "nancount": 1, "nanmean": 2, "nanvar": 3, "nanstd": 4, "nanargmax": 6, "nanmax": 8,
           "nanfirst": 10, "nanlast": 11, "nanprod": 12, "nanall": 14}
    want = {"nansum": 96, "nancount": 96, "nanmean": 48, "nanvar": 32, "nanstd": 32, "nanargmax": 48, "nanmax": 48,
            "nanfirst": 48, "nanlast": 96, "nanprod": 96, "nanall": 96}
    for name, fid in ids.items():
        assert lib.nbg_group_cols_max_labels(fid) == want[name], name
    assert lib.nbg_group_cols_max_labels(15) == 0 and lib.nbg_group_cols_max_labels(-1) == 0


@pytest.mark.parametrize("lang,std", [("c", "-std=c99"), ("c++", "-std=c++11")])
def test_header_compiles_standalone(lang, std):
    """A C or C++ host (or a cgo / JNI stub) includes the header with nothing else."""
    cc = "gcc" if lang == "c" else "g++"
    res = subprocess.run([cc, "-fsyntax-only", std, "-Wall", "-Wextra", "-Werror", "-x", lang, HEADER],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
