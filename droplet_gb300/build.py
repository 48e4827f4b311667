"""Build libdroplet_gb300.so in-tree with nvcc for sm_103a (GB300).

Each .cu file is compiled on its own (in parallel) with the flags its
arithmetic needs, then the objects are linked into one shared library next to
this file. The FP64 plain-form files are compiled with --fmad=false so that
no multiply-add is contracted (their results are bitwise those of the FP64
restatement); the reduced-precision files keep contraction on.

Usage: ``python -m droplet_gb300.build [--force] [-v]``
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libdroplet_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ARCH + [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-Xcompiler", "-fPIC",
    "-Xcompiler", "-ffp-contract=off",
    f"-I{INCLUDE}",
    "--expt-relaxed-constexpr",
]

# per-file arithmetic flags
EXACT = ["--fmad=false", "-prec-div=true", "-prec-sqrt=true"]
FAST = ["--fmad=true"]
SOURCES = {
    "dl_api.cu": EXACT,
    "step_fp64.cu": EXACT,
    "spectral.cu": EXACT,
    "layout.cu": EXACT,
    "reduce.cu": EXACT,
    "reduce_static.cu": EXACT,
    "energy.cu": EXACT,
    "step_fast.cu": FAST,
    "step_push.cu": FAST,
    "adjoint.cu": FAST,
    "labels.cu": FAST,
    "ceiling.cu": FAST,
}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libdroplet_gb300.so")


def _deps() -> list:
    out = [os.path.join(INCLUDE, "droplet_gb300.h"), __file__]
    for fn in os.listdir(CSRC):
        if fn.endswith((".cu", ".cuh", ".h")):
            out.append(os.path.join(CSRC, fn))
    return out


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def _compile(nvcc: str, src: str, flags: list, verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src).replace(".cu", ".o"))
    cmd = [nvcc] + COMMON + flags + (["-Xptxas", "-v"] if verbose else []) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose:
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile and link; returns the path of the shared library."""
    if not force and up_to_date():
        return LIB
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    srcs = [(os.path.join(CSRC, fn), fl) for fn, fl in SOURCES.items()]
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(nvcc, s[0], s[1], verbose), srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcufft"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
