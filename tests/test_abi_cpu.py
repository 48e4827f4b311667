"""The C-ABI library builds, loads without a GPU, and exports exactly the
entry points include/droplet_gb300.h declares (no compute calls here)."""
import ctypes as C
import os
import re

from droplet_gb300 import _abi, _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    text = open(os.path.join(ROOT, "include", "droplet_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dl_[a-z0-9_]+)\s*\(", text)))


def test_header_symbol_list_is_complete():
    assert header_functions() == sorted(_abi.HEADER_SYMBOLS)


def test_library_loads_and_exports_every_header_symbol():
    lib = _lib.load()
    for name in header_functions():
        assert hasattr(lib, name), name
    assert lib.dl_version() >= 100
    assert lib.dl_status_string(_abi.DL_ERR_NAN) == b"NaN/Inf detected"


def test_bad_arguments_are_rejected_without_touching_the_gpu():
    lib = _lib.load()
    h = C.c_void_p()
    p = _abi.DLParams()
    # null params / out pointer, tiny domain, unknown form: all rejected before any CUDA call
    assert lib.dl_create(None, 8, 8, 8, 64, C.byref(h)) == _abi.DL_ERR_ARG
    assert lib.dl_create(C.byref(p), 8, 8, 8, 64, None) == _abi.DL_ERR_ARG
    assert lib.dl_create(C.byref(p), 2, 8, 8, 64, C.byref(h)) == _abi.DL_ERR_ARG
    assert lib.dl_create(C.byref(p), 8, 8, 8, 7, C.byref(h)) == _abi.DL_ERR_UNSUPPORTED
    assert lib.dl_step(None, 1) == _abi.DL_ERR_ARG
    assert lib.dl_destroy(None) == _abi.DL_ERR_ARG
