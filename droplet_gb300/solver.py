"""Python host interface of the droplet step (the drop-in for the Fortran
main loop of program/lbm_drop_xy.f90:756-868).

A :class:`Droplet` owns one whole resident domain. Its methods map onto the
reference's main-loop phases:

=========================  ===================================================
reference (lbm_drop_xy)    here
=========================  ===================================================
ini, :131-252              ``set_fields`` + ``init_equilibrium``
ini_op, :254-285           ``init_equilibrium`` (tau_g range phi1..phi2)
externalforce, :668-693    ``set_force(FORCE_STATIC, fx, fy, fz)``
loop body, :830-840        ``step(n)``
output, :695-719           ``get_fields``
outputfg, :721-743         ``get_populations``
precursor read, :789-823   ``set_populations``
=========================  ===================================================

Arrays are NumPy float64 with shape (nz, ny, nx) (x fastest, the Fortran
order of phi_procs(x,y,z)); populations have shape (nz, ny, nx, 15), the
direction index fastest like f_procs(1:15,x,y,z).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._lib import DropletError, load
from .params import Params

FORM_FP64 = _abi.DL_FORM_FP64
FORM_FP32 = _abi.DL_FORM_FP32
FORM_FP16 = _abi.DL_FORM_FP16
FORCE_NONE = _abi.DL_FORCE_NONE
FORCE_STATIC = _abi.DL_FORCE_STATIC
FORCE_SPECTRAL = _abi.DL_FORCE_SPECTRAL

_dp = C.POINTER(C.c_double)


def _as_f64(a, shape, name):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.shape != shape:
        if a.size != int(np.prod(shape)):
            raise ValueError(f"{name}: expected shape {shape}, got {a.shape}")
        a = a.reshape(shape)
    return a


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


class _HandleAPI:
    """Shared implementation over a C library exposing ``<prefix>_*`` entry
    points with the signatures of include/droplet_gb300.h."""

    prefix = "dl"

    def __init__(self, lib, params: Params, shape, form: int | None):
        nx, ny, nz = (int(v) for v in shape)
        self.nx, self.ny, self.nz = nx, ny, nz
        self.params = params
        self.form = form
        self._lib = lib
        self._cparams = params.to_c()
        h = C.c_void_p()
        args = [C.byref(self._cparams), nx, ny, nz]
        if self.prefix == "dl":
            args.append(int(form))
        args.append(C.byref(h))
        self._h = None
        self._call("create", *args, handle=False)
        self._h = h

    # ---- plumbing ------------------------------------------------------------
    @property
    def shape3(self):
        return (self.nz, self.ny, self.nx)

    @property
    def n_sites(self) -> int:
        return self.nx * self.ny * self.nz

    def _detail(self) -> str:
        return ""

    def _call(self, name, *args, handle=True):
        fn = getattr(self._lib, f"{self.prefix}_{name}")
        rc = fn(self._h, *args) if handle else fn(*args)
        if rc != 0:
            raise DropletError(rc, f"{self.prefix}_{name}", self._detail() if handle else "")
        return rc

    def close(self):
        if getattr(self, "_h", None) is not None:
            getattr(self._lib, f"{self.prefix}_destroy")(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- the main-loop phases ---------------------------------------------------
    def set_fields(self, phi, u1, u2, u3, p):
        arrs = [_as_f64(a, self.shape3, n) for a, n in zip((phi, u1, u2, u3, p), ("phi", "u1", "u2", "u3", "p"))]
        self._keep = arrs
        self._call("set_fields", *[_ptr(a) for a in arrs])

    def init_equilibrium(self):
        self._call("init_equilibrium")

    def set_force(self, mode: int, fx=None, fy=None, fz=None):
        if mode == FORCE_STATIC:
            arrs = [_as_f64(a, self.shape3, n) for a, n in zip((fx, fy, fz), ("fx", "fy", "fz"))]
            self._call("set_force", int(mode), *[_ptr(a) for a in arrs])
        else:
            self._call("set_force", int(mode), None, None, None)

    def step(self, n: int = 1):
        self._call("step", int(n))

    def get_fields(self) -> dict:
        out = {k: np.empty(self.shape3, dtype=np.float64) for k in ("phi", "u1", "u2", "u3", "p")}
        return self.get_fields_into(out)

    def get_fields_into(self, out: dict) -> dict:
        """Download into caller-owned C-contiguous float64 arrays (e.g. pinned)."""
        for k in ("phi", "u1", "u2", "u3", "p"):
            a = out[k]
            if a.dtype != np.float64 or not a.flags.c_contiguous or a.size != self.n_sites:
                raise ValueError(f"{k}: need a C-contiguous float64 array of {self.n_sites} values")
        self._call("get_fields", *[_ptr(out[k]) for k in ("phi", "u1", "u2", "u3", "p")])
        return out

    def get_populations(self):
        f = np.empty(self.shape3 + (15,), dtype=np.float64)
        g = np.empty(self.shape3 + (15,), dtype=np.float64)
        self._call("get_populations", _ptr(f), _ptr(g))
        return f, g

    def set_populations(self, f, g):
        shape = self.shape3 + (15,)
        f = _as_f64(f, shape, "f")
        g = _as_f64(g, shape, "g")
        self._call("set_populations", _ptr(f), _ptr(g))

    @property
    def step_count(self) -> int:
        v = C.c_int64()
        self._call("get_step", C.byref(v))
        return int(v.value)

    @step_count.setter
    def step_count(self, n: int):
        self._call("set_step", C.c_int64(int(n)))

    def minmax(self):
        mn, mx = C.c_double(), C.c_double()
        self._call("get_minmax", C.byref(mn), C.byref(mx))
        return float(mn.value), float(mx.value)

    def minmax_async(self, pinned_ptr: int):
        """Enqueue the copy of (phi_min, phi_max) into two pinned host doubles
        at pinned_ptr; read them once the stream has passed this point."""
        self._call("get_minmax_async", C.c_void_p(int(pinned_ptr)))

    def set_minmax_mirror(self, pinned_ptr: int, nslots: int = 2):
        """Have every step write its (phi_min, phi_max) into 2 nslots pinned
        host doubles at pinned_ptr: the step that takes the step counter to n
        fills slot n % nslots once its launch completes. pinned_ptr 0 turns the
        mirror off."""
        self._call("set_minmax_mirror", C.c_void_p(int(pinned_ptr) or None), C.c_int64(int(nslots)))


class Droplet(_HandleAPI):
    """Whole-domain droplet state resident on the current CUDA device."""

    prefix = "dl"

    def __init__(self, params: Params, shape, form: int = FORM_FP64, single_phase: bool = False):
        """single_phase: the g-only step of the precursor turbulence program
        (program/lbm_iht_xy.f90), DL_SINGLE_PHASE; phi is then not a field."""
        self.single_phase = bool(single_phase)
        super().__init__(load(), params, shape, int(form) | (_abi.DL_SINGLE_PHASE if single_phase else 0))
        self.form = int(form)

    def _detail(self) -> str:
        if getattr(self, "_h", None) is None:
            return ""
        buf = C.create_string_buffer(512)
        self._lib.dl_last_error(self._h, buf, 512)
        return buf.value.decode(errors="replace")

    def set_stream(self, stream_ptr: int):
        """Run this handle's work on a cudaStream_t given as an integer."""
        self._call("set_stream", C.c_void_p(int(stream_ptr)))

    def sync(self):
        self._call("sync")

    def reduce(self) -> dict:
        d = _abi.DLDiag()
        self._call("reduce", C.byref(d))
        return d.as_dict()

    def energy(self, nbins: int | None = None):
        """In-situ energy diagnostics (dl_energy): dict of the free-energy sums
        and, unless nbins == 0, the kinetic-energy spectrum (nbins defaults to
        the reference's nx/2 + 1 bins)."""
        nb = self.nx // 2 + 1 if nbins is None else int(nbins)
        spec = np.zeros(max(nb, 1), dtype=np.float64)
        d = _abi.DLEnergyDiag()
        self._call("energy", C.byref(d), _ptr(spec) if nb > 0 else None, C.c_int64(nb))
        out = d.as_dict()
        out["spectrum"] = spec[:nb].copy()
        return out

    def pull_ceiling(self, repeats: int = 20) -> float:
        """GB/s of the step's pull pattern without arithmetic (dl_pull_ceiling);
        overwrites the next-step population buffer."""
        v = C.c_double()
        self._call("pull_ceiling", int(repeats), C.byref(v))
        return float(v.value)

    def fp64_ceiling(self) -> float:
        """Measured FP64 FMA throughput of this GPU, TFLOP/s (dl_fp64_ceiling)."""
        v = C.c_double()
        self._call("fp64_ceiling", C.byref(v))
        return float(v.value)

    def reduce_static(self, nblocks: int = 0) -> dict:
        """The diagnostics of reduce() through dl_reduce_static, which
        allocates no device memory (fixed scratch inside the library, shared
        per device: calls on one device must not overlap)."""
        d = _abi.DLDiag()
        self._call("reduce_static", int(nblocks), C.byref(d))
        return d.as_dict()

    def label_droplets(self, connectivity: int = 14, labels: bool = False, max_volumes: int = 100000):
        """Droplets = periodic connected components of phi >= (phi1+phi2)/2.
        Returns (volumes sorted decreasing, labels array or None)."""
        n = C.c_int64()
        vols = np.zeros(max_volumes, dtype=np.float64)
        lab = np.empty(self.shape3, dtype=np.int32) if labels else None
        self._call("label_droplets", int(connectivity), lab.ctypes.data_as(C.c_void_p) if labels else None,
                   C.byref(n), _ptr(vols), C.c_int64(max_volumes))
        return vols[: min(int(n.value), max_volumes)].copy(), lab

    def profile(self, enable: bool = True, every: int = 1):
        """Bracket every ``every``-th launch with CUDA events (and reset the
        counters); ``enable`` False stops."""
        self._call("profile", int(every) if enable else 0)

    def set_option(self, key: str, value: int):
        """Launch-shape knob of the fused kernel (e.g. "lz")."""
        self._call("set_option", key.encode(), C.c_int64(int(value)))

    def get_option(self, key: str) -> int:
        v = C.c_int64()
        self._call("get_option", key.encode(), C.byref(v))
        return int(v.value)

    def profile_read(self) -> dict:
        s = _abi.DLProfileStats()
        self._call("profile_read", C.byref(s))
        return {k: getattr(s, k) for k, _ in s._fields_}
