"""Build ``libmwdem.so`` in-tree (``mwdiem_gb300/_build/``) with nvcc for sm_103a.

Every translation unit is compiled with ``--fmad=false`` and IEEE division/square root: the narrow
phase reproduces the reference kernel's rounding operation by operation, and the host parts of the
library (which derive the contact-law constants) are compiled with ``-ffp-contract=off`` for the
same reason.  Translation units compile in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
BUILD = HERE / "_build"
INCLUDE = HERE.parent / "include"
LIB = BUILD / "libmwdem.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-std=c++17",
           "-Xcompiler", "-fPIC,-ffp-contract=off", "-diag-suppress", "1444", f"-I{INCLUDE}"]
SOURCES = ["narrow.cu", "integrate.cu", "broad.cu", "capi.cu", "probe.cu", "noalloc.cu", "adjoint.cu", "reduce.cu", "inlet.cu"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _deps():
    return [CSRC / s for s in SOURCES] + list(CSRC.glob("*.cuh")) + [INCLUDE / "mwdem.h", Path(__file__)]


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _deps())


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and up_to_date():
        return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    cc = nvcc()

    def one(src):
        obj = BUILD / (Path(src).stem + ".o")
        cmd = [cc, *ARCH, *NVFLAGS, "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(one, SOURCES))
    objs = [str(o) for o, _ in results]
    tmp = LIB.with_suffix(".so.tmp%d" % os.getpid())
    r = subprocess.run([cc, *ARCH, "-shared", *objs, "-o", str(tmp)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        for _, log in results:
            print(log)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose="-v" in sys.argv))
