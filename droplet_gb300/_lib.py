"""Loader of the in-tree CUDA library libdroplet_gb300.so.

There is no CPU fallback: if the library is missing or cannot be loaded the
import of the solver fails with an error that says so.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import _abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libdroplet_gb300.so")

_lock = threading.Lock()
_lib = None


class DropletError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, status: int, what: str, detail: str = ""):
        self.status = status
        text = _abi.STATUS_TEXT.get(status, f"status {status}")
        super().__init__(f"{what}: {text}" + (f" ({detail})" if detail else ""))


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load (building first if needed) the CUDA library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            if not build_if_missing:
                raise RuntimeError(f"{LIB_PATH} is missing: run `python -m droplet_gb300.build`")
            from . import build as _build

            _build.build()
        lib = C.CDLL(LIB_PATH, mode=C.RTLD_LOCAL)
        _abi.declare(lib, "dl")
        _lib = lib
        return lib
