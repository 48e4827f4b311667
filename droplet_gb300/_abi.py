"""ctypes mirror of include/droplet_gb300.h (structs, constants, prototypes).

The same structs are used by the GPU library and by the oracle's CPU
library, whose entry points have identical signatures (``dl_*`` / ``orc_*``).
"""
from __future__ import annotations

import ctypes as C

DL_OK = 0
DL_ERR_ARG = -1
DL_ERR_CUDA = -2
DL_ERR_ALLOC = -3
DL_ERR_NAN = -4
DL_ERR_TIMEOUT = -5
DL_ERR_STATE = -6
DL_ERR_UNSUPPORTED = -7

STATUS_TEXT = {
    DL_OK: "ok",
    DL_ERR_ARG: "bad argument",
    DL_ERR_CUDA: "CUDA error",
    DL_ERR_ALLOC: "allocation failed",
    DL_ERR_NAN: "NaN/Inf detected",
    DL_ERR_TIMEOUT: "device wait timed out",
    DL_ERR_STATE: "call out of order",
    DL_ERR_UNSUPPORTED: "unsupported option for this form",
}

DL_FORM_FP64 = 64
DL_FORM_FP32 = 32
DL_FORM_FP16 = 16
DL_SINGLE_PHASE = 0x100

DL_FORCE_NONE = 0
DL_FORCE_STATIC = 1
DL_FORCE_SPECTRAL = 2

DL_VISC_MINMAX = 0
DL_VISC_FIXED = 1

DL_REDUCE_STATIC_MAX_BLOCKS = 1216
DL_REDUCE_STATIC_SCRATCH_BYTES = 253144


class DLParams(C.Structure):
    _fields_ = [
        ("ds", C.c_double),
        ("tauf", C.c_double),
        ("kappaf", C.c_double),
        ("kappag", C.c_double),
        ("phi1", C.c_double),
        ("phi2", C.c_double),
        ("a", C.c_double),
        ("b", C.c_double),
        ("T", C.c_double),
        ("nu1", C.c_double),
        ("nu2", C.c_double),
        ("Anu", C.c_double),
        ("Cs", C.c_double),
        ("delta", C.c_double),
        ("wall_u", C.c_double * 3),
        ("eps", C.c_double),
        ("wall_start", C.c_int64),
        ("visc_mode", C.c_int32),
        ("les", C.c_int32),
        ("walls", C.c_int32),
        ("kc", C.c_int32),
    ]


class DLDiag(C.Structure):
    _fields_ = [
        ("phi_sum", C.c_double),
        ("p_sum", C.c_double),
        ("mom", C.c_double * 3),
        ("ke", C.c_double),
        ("diss", C.c_double),
        ("vol_count", C.c_double),
        ("vol_smooth", C.c_double),
        ("phi_min", C.c_double),
        ("phi_max", C.c_double),
        ("p_in", C.c_double),
        ("n_in", C.c_double),
        ("p_out", C.c_double),
        ("n_out", C.c_double),
        ("w_sum", C.c_double),
        ("w_x", C.c_double * 3),
        ("w_xx", C.c_double * 6),
        ("step", C.c_int64),
        ("nan_flag", C.c_int32),
        ("pad_", C.c_int32),
    ]

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            if name == "pad_":
                continue
            v = getattr(self, name)
            out[name] = list(v) if hasattr(v, "__len__") else v
        return out


class DLEnergyDiag(C.Structure):
    _fields_ = [("psi_sum", C.c_double), ("mu_sum", C.c_double), ("grad_sq_sum", C.c_double),
                ("spectrum_sum", C.c_double), ("nbins", C.c_int64), ("step", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class DLProfileStats(C.Structure):
    _fields_ = [
        ("main_ms", C.c_double),
        ("total_ms", C.c_double),
        ("main_launches", C.c_int64),
        ("timed_launches", C.c_int64),
        ("launches", C.c_int64),
    ]


_dp = C.POINTER(C.c_double)
_vp = C.c_void_p


def declare(lib: C.CDLL, prefix: str) -> None:
    """Attach argtypes/restype for the handle API under ``prefix`` (dl / orc)."""
    h = _vp
    sig = {
        "create": [C.POINTER(DLParams), C.c_int, C.c_int, C.c_int] + ([C.c_int] if prefix == "dl" else []) + [C.POINTER(_vp)],
        "destroy": [h],
        "set_fields": [h, _dp, _dp, _dp, _dp, _dp],
        "init_equilibrium": [h],
        "set_force": [h, C.c_int, _dp, _dp, _dp],
        "step": [h, C.c_int],
        "get_fields": [h, _dp, _dp, _dp, _dp, _dp],
        "get_populations": [h, _dp, _dp],
        "set_populations": [h, _dp, _dp],
        "set_step": [h, C.c_int64],
        "get_step": [h, C.POINTER(C.c_int64)],
        "get_minmax": [h, _dp, _dp],
    }
    for name, args in sig.items():
        fn = getattr(lib, f"{prefix}_{name}")
        fn.argtypes = args
        fn.restype = C.c_int
    if prefix == "dl":
        lib.dl_version.argtypes = []
        lib.dl_version.restype = C.c_int
        lib.dl_status_string.argtypes = [C.c_int]
        lib.dl_status_string.restype = C.c_char_p
        lib.dl_set_stream.argtypes = [h, _vp]
        lib.dl_set_stream.restype = C.c_int
        lib.dl_reduce.argtypes = [h, C.POINTER(DLDiag)]
        lib.dl_reduce.restype = C.c_int
        lib.dl_fp64_ceiling.argtypes = [h, C.POINTER(C.c_double)]
        lib.dl_fp64_ceiling.restype = C.c_int
        lib.dl_pull_ceiling.argtypes = [h, C.c_int, C.POINTER(C.c_double)]
        lib.dl_pull_ceiling.restype = C.c_int
        lib.dl_energy.argtypes = [h, C.POINTER(DLEnergyDiag), C.c_void_p, C.c_int64]
        lib.dl_energy.restype = C.c_int
        lib.dl_get_minmax_async.argtypes = [h, _vp]
        lib.dl_get_minmax_async.restype = C.c_int
        lib.dl_set_minmax_mirror.argtypes = [h, _vp, C.c_int64]
        lib.dl_set_minmax_mirror.restype = C.c_int
        lib.dl_host_alloc.argtypes = [C.c_int64, C.POINTER(_vp)]
        lib.dl_host_alloc.restype = C.c_int
        lib.dl_host_free.argtypes = [_vp]
        lib.dl_host_free.restype = C.c_int
        lib.dl_reduce_static.argtypes = [h, C.c_int, C.POINTER(DLDiag)]
        lib.dl_reduce_static.restype = C.c_int
        lib.dl_sync.argtypes = [h]
        lib.dl_sync.restype = C.c_int
        lib.dl_last_error.argtypes = [h, C.c_char_p, C.c_int]
        lib.dl_last_error.restype = C.c_int
        lib.dl_profile.argtypes = [h, C.c_int]
        lib.dl_profile.restype = C.c_int
        lib.dl_profile_read.argtypes = [h, C.POINTER(DLProfileStats)]
        lib.dl_profile_read.restype = C.c_int
        lib.dl_set_option.argtypes = [h, C.c_char_p, C.c_int64]
        lib.dl_set_option.restype = C.c_int
        lib.dl_get_option.argtypes = [h, C.c_char_p, C.POINTER(C.c_int64)]
        lib.dl_get_option.restype = C.c_int
        lib.dl_label_droplets.argtypes = [h, C.c_int, _vp, C.POINTER(C.c_int64), _dp, C.c_int64]
        lib.dl_label_droplets.restype = C.c_int
        lib.dl_state_floats.argtypes = [h, C.POINTER(C.c_int64)]
        lib.dl_state_floats.restype = C.c_int
        lib.dl_save_state.argtypes = [h, _vp]
        lib.dl_save_state.restype = C.c_int
        lib.dl_adjoint_state_floats.argtypes = [h, C.POINTER(C.c_int64)]
        lib.dl_adjoint_state_floats.restype = C.c_int
        lib.dl_save_adjoint_state.argtypes = [h, _vp]
        lib.dl_save_adjoint_state.restype = C.c_int
        lib.dl_load_state.argtypes = [h, _vp]
        lib.dl_load_state.restype = C.c_int
        lib.dl_adjoint_begin.argtypes = [h, _vp]
        lib.dl_adjoint_begin.restype = C.c_int
        lib.dl_adjoint_step.argtypes = [h, _vp, C.c_int64]
        lib.dl_adjoint_step.restype = C.c_int
        lib.dl_adjoint_init.argtypes = [h, _vp, _vp]
        lib.dl_adjoint_init.restype = C.c_int
        lib.dl_adjoint_grads.argtypes = [h, _dp]
        lib.dl_adjoint_grads.restype = C.c_int
        lib.dl_batch_create.argtypes = [C.POINTER(DLParams), C.POINTER(C.c_int), C.c_int, C.c_int, C.POINTER(_vp)]
        lib.dl_batch_create.restype = C.c_int
        lib.dl_batch_member.argtypes = [_vp, C.c_int, C.POINTER(_vp)]
        lib.dl_batch_member.restype = C.c_int
        lib.dl_batch_set_stream.argtypes = [_vp, _vp]
        lib.dl_batch_set_stream.restype = C.c_int
        lib.dl_batch_step.argtypes = [_vp, C.c_int]
        lib.dl_batch_step.restype = C.c_int
        lib.dl_batch_set_option.argtypes = [_vp, C.c_char_p, C.c_int64]
        lib.dl_batch_set_option.restype = C.c_int
        lib.dl_batch_get_option.argtypes = [_vp, C.c_char_p, C.POINTER(C.c_int64)]
        lib.dl_batch_get_option.restype = C.c_int
        lib.dl_batch_destroy.argtypes = [_vp]
        lib.dl_batch_destroy.restype = C.c_int
    else:
        lib.orc_get_force.argtypes = [h, _dp, _dp, _dp]
        lib.orc_get_force.restype = C.c_int
        lib.orc_compute_spectral_force.argtypes = [h]
        lib.orc_compute_spectral_force.restype = C.c_int
        lib.orc_set_threads.argtypes = [C.c_int]
        lib.orc_set_threads.restype = C.c_int
        lib.orc_get_threads.argtypes = []
        lib.orc_get_threads.restype = C.c_int


# Every symbol include/droplet_gb300.h declares (checked by the CPU test suite).
HEADER_SYMBOLS = [
    "dl_version",
    "dl_status_string",
    "dl_create",
    "dl_destroy",
    "dl_set_stream",
    "dl_set_fields",
    "dl_init_equilibrium",
    "dl_set_force",
    "dl_step",
    "dl_get_fields",
    "dl_get_populations",
    "dl_set_populations",
    "dl_set_step",
    "dl_get_step",
    "dl_get_minmax",
    "dl_get_minmax_async",
    "dl_set_minmax_mirror",
    "dl_host_alloc",
    "dl_host_free",
    "dl_reduce",
    "dl_reduce_static",
    "dl_energy",
    "dl_pull_ceiling",
    "dl_fp64_ceiling",
    "dl_sync",
    "dl_last_error",
    "dl_profile",
    "dl_profile_read",
    "dl_set_option",
    "dl_get_option",
    "dl_label_droplets",
    "dl_state_floats",
    "dl_save_state",
    "dl_load_state",
    "dl_adjoint_state_floats",
    "dl_save_adjoint_state",
    "dl_adjoint_begin",
    "dl_adjoint_step",
    "dl_adjoint_init",
    "dl_adjoint_grads",
    "dl_batch_create",
    "dl_batch_member",
    "dl_batch_set_stream",
    "dl_batch_step",
    "dl_batch_set_option",
    "dl_batch_get_option",
    "dl_batch_destroy",
]
