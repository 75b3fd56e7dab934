"""Record numbagg's public call signatures in ``reference_signatures.json``.

numbagg imports behind the same names-only numba stub as ``make_golden.py`` (its
decorators compile lazily), and ``inspect.signature`` of each public function gives the
parameters a caller may pass: their names, kinds and defaults.
``tests/test_signatures.py`` checks that ``numbagg_gb300`` accepts each of them with the
same default.

Usage (needs a numbagg source tree; the GPU machine does not):

    python tests/golden/make_signatures.py /path/to/numbagg-source
"""

from __future__ import annotations

import inspect
import json
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import make_golden  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_signatures.json")


def main() -> None:
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("NUMBAGG_SRC", "")
    if not src or not os.path.isdir(os.path.join(src, "numbagg")):
        sys.exit("usage: make_signatures.py <numbagg source tree>")
    nb = make_golden._import_numbagg(src)
    sigs = {}
    for name in sorted(nb.__all__):
        obj = getattr(nb, name, None)
        if obj is None or isinstance(obj, (list, tuple, str)):
            continue
        try:
            sig = inspect.signature(obj)
        except (TypeError, ValueError):
            continue
        params = []
        for p in sig.parameters.values():
            default = None if p.default is inspect.Parameter.empty else repr(p.default)
            params.append({"name": p.name, "kind": p.kind.name, "default": default})
        sigs[name] = params
    with open(OUT, "w") as fh:
        json.dump(sigs, fh, indent=1, sort_keys=True)
        fh.write("\n")
    print(f"wrote {len(sigs)} signatures to {OUT}")


if __name__ == "__main__":
    main()
