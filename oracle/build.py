"""Build the CPU oracle (test infrastructure only).

Compiles ``nbg_oracle.c`` into ``libnbg_oracle.so`` beside this file with
``-O2 -ffp-contract=off`` (no FMA contraction, like numba without fastmath) and
OpenMP.  Run ``python oracle/build.py`` or call :func:`build`.
"""

from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "nbg_oracle.c")
LIB = os.path.join(HERE, "libnbg_oracle.so")


def build(force: bool = False) -> str:
    newest = max(os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "scan_loops.inc")))
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [
        os.environ.get("CC", "gcc"),
        "-O2",
        "-ffp-contract=off",
        "-fno-fast-math",
        "-fopenmp",
        "-fPIC",
        "-shared",
        "-Wall",
        "-Wno-unknown-pragmas",
        "-o",
        tmp,
        SRC,
        "-lm",
    ]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
