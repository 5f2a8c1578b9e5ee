"""Compile the oracle's C restatement into ``oracle/_build/liboracle.so``.

TEST INFRASTRUCTURE ONLY (see ``oracle/mwdem_oracle.c``).  Called by ``__graft_entry__.build()``
and lazily by ``oracle/oracle.py``.  Flags: ``-ffp-contract=off`` keeps FP32 rounding identical to
the CUDA build, whose narrow-phase translation unit is compiled with ``--fmad=false``.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
SOURCES = [HERE / "mwdem_oracle.c"]
HEADERS = [HERE / "narrow_impl.h"]
LIB = BUILD / "liboracle.so"
CFLAGS = ["-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
          "-Wall", "-Wno-unused-function"]


def build(force: bool = False) -> Path:
    BUILD.mkdir(parents=True, exist_ok=True)
    newest = max(p.stat().st_mtime for p in SOURCES + HEADERS + [Path(__file__)])
    if not force and LIB.exists() and LIB.stat().st_mtime >= newest:
        return LIB
    tmp = LIB.with_suffix(".so.tmp%d" % os.getpid())
    subprocess.run(["gcc", *CFLAGS, *map(str, SOURCES), "-o", str(tmp), "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
