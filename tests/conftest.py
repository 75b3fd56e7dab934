import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_vectors.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")
    config.addinivalue_line("markers", "slow: large sizes")


def pytest_collection_modifyitems(config, items):
    try:
        import torch

        has_gpu = torch.cuda.is_available()
    except Exception:  # pragma: no cover
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def golden():
    with np.load(GOLDEN) as z:
        return {k: z[k] for k in z.files}


def same_values(actual, desired) -> bool:
    """Bit-level equality that treats every NaN as equal and tells +0 from -0."""
    a = np.asarray(actual)
    d = np.asarray(desired)
    if a.shape != d.shape or a.dtype != d.dtype:
        return False
    if a.dtype.kind == "f":
        an, dn = np.isnan(a), np.isnan(d)
        if not np.array_equal(an, dn):
            return False
        keep = ~an
        return bool(
            np.array_equal(a[keep], d[keep]) and np.array_equal(np.signbit(a[keep]), np.signbit(d[keep]))
        )
    return bool(np.array_equal(a, d))
