"""droplet_gb300: GB300-native D3Q15 two-phase droplet lattice-Boltzmann step.

The hot path (one time step of the reference's Inamuro free-energy droplet
code, nakano-gendai/droplet program/lbm_drop_xy.f90) runs as hand-written
CUDA for sm_103a in libdroplet_gb300.so, driven through a thin ctypes C-ABI
(include/droplet_gb300.h).
"""
from .params import Params, kappag_from_sigma, sigma_from_kappag, static_vortex_force  # noqa: F401
from . import init_fields  # noqa: F401

__version__ = "0.1.0"


def __getattr__(name):
    # the solver loads the CUDA library lazily, so importing the package
    # (e.g. for parameters or initial fields) needs no GPU
    if name in ("Droplet", "DropletError", "FORM_FP64", "FORM_FP32", "FORM_FP16",
                "FORCE_NONE", "FORCE_STATIC", "FORCE_SPECTRAL"):
        from . import solver, _lib

        if name == "DropletError":
            return _lib.DropletError
        return getattr(solver, name)
    raise AttributeError(name)
