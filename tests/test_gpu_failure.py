"""Failure detection on the GPU without a fault: a bounded look-back wait that
nothing satisfies gives up, records NBG_LOOKBACK_TIMEOUT in the workspace header and
returns; the host reads the code back and the CUDA context stays usable."""

import numpy as np
import pytest
import torch

import numbagg_gb300 as nb
from numbagg_gb300 import _lib

pytestmark = pytest.mark.gpu


def test_bounded_wait_reports_timeout_and_context_survives():
    L = _lib.lib()
    dev = torch.device("cuda", 0)
    ws = torch.zeros(1 << 16, dtype=torch.uint8, device=dev)
    stream = _lib.stream_handle(dev)
    assert L.nbg_debug_lookback_timeout(ws.data_ptr(), ws.numel(), 200, stream) == 0
    code, tile = _lib.workspace_error(ws)
    assert code == 4 and tile == 1
    # cleared after reading
    assert _lib.workspace_error(ws) == (0, 0)
    # the context still works
    x = np.random.default_rng(0).standard_normal((2, 1000))
    assert np.isfinite(nb.move_mean(x, window=5)[:, 4:]).all()
    torch.cuda.synchronize()


def test_real_scans_leave_no_error_flag():
    x = torch.randn(16, 500_000, dtype=torch.float64, device="cuda")
    nb.move_mean(x, window=50)
    nb.ffill(x)
    nb.move_exp_nanvar(x, alpha=0.1)
    torch.cuda.synchronize()
    for ws in _lib.workspaces.all_scan():
        assert _lib.workspace_error(ws) == (0, 0)


def test_bad_limit_rejected_on_host():
    with pytest.raises(ValueError):
        nb.ffill(torch.zeros(3, device="cuda"), limit=-1)
