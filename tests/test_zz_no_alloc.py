"""The allocation-free forward fill, nbg_ffill_f64_noalloc.

It serves callers that may not allocate device memory themselves or through this
library: a host application that owns all GPU memory and lends only the input and
output buffers (a database or stream engine running the fill as a user-defined
function), or a latency-critical path that must not reach cudaMalloc / cudaFree, which
can synchronise the whole device.  Its look-back state lives in a fixed 4 MiB array in
the library's device image instead of a caller-provided workspace.

The test calls it through the C ABI twice in a row on different inputs and checks
each result against the ordinary entry point nbg_ffill_f64 (a fill only selects
values, so the two must agree bit for bit) and that no look-back wait gave up
(nbg_ffill_noalloc_error reads (0, 0)).  It then checks that a problem larger than
the fixed scratch is refused without a launch and that a call after the refusal
still matches the ordinary entry point.  This file is named so that pytest
collects it last; it passes both on its own in a fresh process and after the rest of
the suite.
"""

import ctypes

import numpy as np
import pytest
import torch

from numbagg_gb300 import _lib

pytestmark = pytest.mark.gpu


def _ffill_with_workspace(L, x, limit, stream):
    rows, n = x.shape
    out = torch.empty_like(x)
    nbytes = L.nbg_fill_workspace_bytes(rows, n)
    ws = torch.zeros(nbytes, dtype=torch.uint8, device=x.device)
    assert L.nbg_ffill_f64(x.data_ptr(), out.data_ptr(), rows, n, limit, ws.data_ptr(), ws.numel(), stream) == 0
    return out


def _noalloc_error(L, stream):
    code, tile = ctypes.c_int(-1), ctypes.c_uint(12345)
    assert L.nbg_ffill_noalloc_error(ctypes.byref(code), ctypes.byref(tile), stream) == 0
    return code.value, tile.value


def _check_against_workspace_entry(L, rng, rows, n, limit, what):
    dev = torch.device("cuda", 0)
    stream = _lib.stream_handle(dev)
    x = rng.standard_normal((rows, n))
    x[rng.random(x.shape) < 0.3] = np.nan
    x[0, min(1000, n) : min(30_000, n)] = np.nan  # a NaN run across several tiles
    xt = torch.from_numpy(x).to(dev)
    out = torch.full_like(xt, 7.0)
    status = L.nbg_ffill_f64_noalloc(xt.data_ptr(), out.data_ptr(), rows, n, limit, stream)
    assert status == 0, _lib.STATUS.get(status)
    want = _ffill_with_workspace(L, xt, limit, stream)
    torch.cuda.synchronize()
    got_np, want_np = out.cpu().numpy(), want.cpu().numpy()
    assert np.array_equal(np.isnan(got_np), np.isnan(want_np)), f"{what}: NaN placement"
    keep = ~np.isnan(want_np)
    assert np.array_equal(got_np[keep], want_np[keep]), f"{what}: values"
    assert _noalloc_error(L, stream) == (0, 0), f"{what}: a look-back wait gave up"


def test_noalloc_ffill_matches_workspace_entry_twice():
    L = _lib.lib()
    rng = np.random.default_rng(123)
    for call, (rows, n, limit) in enumerate([(7, 50_001, 3), (3, 200_000, 200_000)]):
        _check_against_workspace_entry(L, rng, rows, n, limit, f"call {call}")


def test_noalloc_ffill_rejects_problems_beyond_its_scratch():
    L = _lib.lib()
    cap = L.nbg_ffill_noalloc_max_scratch_bytes()
    assert cap == 4 << 20
    # 20,000 rows of one 4096-element tile each: more tiles than the 4 MiB holds, so the
    # call is refused before any launch (the buffers are real and of the claimed size)
    rows, n = 20_000, 4096
    assert L.nbg_fill_workspace_bytes(rows, n) > cap
    dev = torch.device("cuda", 0)
    x = torch.zeros((rows, n), dtype=torch.float64, device=dev)
    out = torch.empty_like(x)
    status = L.nbg_ffill_f64_noalloc(x.data_ptr(), out.data_ptr(), rows, n, 5, _lib.stream_handle(dev))
    assert status == 6, _lib.STATUS.get(status)
    assert L.nbg_ffill_f64_noalloc(None, None, -1, 10, 1, None) == 1
    # the refused calls touched nothing: the scratch still serves a call
    _check_against_workspace_entry(L, np.random.default_rng(7), 5, 70_000, 10, "after the refusal")
