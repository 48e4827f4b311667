"""ctypes wrapper of the C oracle (liboracle.so). TEST INFRASTRUCTURE ONLY.

``OracleDroplet`` has the methods of ``droplet_gb300.solver.Droplet`` so a
test can drive the GPU library and the oracle through the same calls.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

from droplet_gb300 import _abi
from droplet_gb300.solver import _HandleAPI, _ptr

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP, -ffp-contract=off)."""
    args = ["make", "-s", "-C", HERE]
    if force:
        args.append("-B")
    r = subprocess.run(args, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB_PATH


def load() -> C.CDLL:
    global _lib
    with _lock:
        if _lib is None:
            build()
            lib = C.CDLL(LIB_PATH, mode=C.RTLD_LOCAL)
            _abi.declare(lib, "orc")
            _lib = lib
        return _lib


def set_threads(n: int) -> None:
    load().orc_set_threads(int(n))


def get_threads() -> int:
    return int(load().orc_get_threads())


class OracleDroplet(_HandleAPI):
    """FP64 CPU restatement with the Droplet interface (form is always FP64)."""

    prefix = "orc"

    def __init__(self, params, shape, form=None, single_phase=False):
        super().__init__(load(), params, shape, form)
        self.single_phase = bool(single_phase)
        if single_phase:
            self._lib.orc_set_single.argtypes = [C.c_void_p, C.c_int]
            self._call("set_single", 1)

    def get_force(self):
        out = [np.empty(self.shape3) for _ in range(3)]
        self._call("get_force", *[_ptr(a) for a in out])
        return out

    def compute_spectral_force(self):
        self._call("compute_spectral_force")
        return self.get_force()
