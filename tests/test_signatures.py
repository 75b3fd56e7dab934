"""numbagg_gb300 accepts every keyword numbagg's public functions accept, with the same
defaults (tests/golden/reference_signatures.json, recorded from numbagg by
tests/golden/make_signatures.py).  Positional array parameters may be named differently;
keywords numbagg passes through to numba (``**kwargs``) are not part of the contract."""

import inspect
import json
import os

import pytest

import numbagg_gb300 as nb

_SIGS = os.path.join(os.path.dirname(__file__), "golden", "reference_signatures.json")
# numbagg functions outside this package's path (not built)
NOT_BUILT = {"nanmedian", "nanquantile"}

with open(_SIGS) as _fh:
    REFERENCE = json.load(_fh)


def test_every_in_scope_function_exists():
    missing = sorted(set(REFERENCE) - NOT_BUILT - {n for n in REFERENCE if hasattr(nb, n)})
    assert missing == []


@pytest.mark.parametrize("name", sorted(set(REFERENCE) - NOT_BUILT))
def test_keywords_and_defaults_match(name):
    ours = inspect.signature(getattr(nb, name)).parameters
    for p in REFERENCE[name]:
        if p["kind"] in ("VAR_POSITIONAL", "VAR_KEYWORD", "POSITIONAL_ONLY"):
            continue
        if p["kind"] == "POSITIONAL_OR_KEYWORD" and p["default"] is None:
            continue  # an input array, passed by position
        q = ours.get(p["name"])
        assert q is not None, f"{name} does not accept {p['name']}="
        default = None if q.default is inspect.Parameter.empty else repr(q.default)
        assert default == p["default"], (name, p["name"], default, p["default"])
