"""Batched ensembles: many independent droplet domains (uneven sizes, their
own parameters and seeds) stepped together: by default each member takes its
own one-launch steps on one of up to 16 streams forked from the ensemble's
stream (the blocks of many members fill the GPU together); option
"persistent" = 1 runs one persistent launch per step over all members instead,
with pairs of steps replayed from a captured CUDA graph.

The reference's analogues are replica groups of MPI ranks
(program/lbm_omp_drop.f90:149-166) and a sequential loop over cases
(program/lbm_drop_iht_xy_many.f90:1211).
"""
from __future__ import annotations

import ctypes as C

from . import _abi
from ._lib import DropletError, load
from .solver import Droplet, FORM_FP32


class _Member(Droplet):
    """A member handle owned by its ensemble (not destroyed on close)."""

    def __init__(self, lib, handle, params, shape, form, persistent):  # noqa: D401 - bypass Droplet.__init__
        nx, ny, nz = (int(v) for v in shape)
        self.nx, self.ny, self.nz = nx, ny, nz
        self.params = params
        self.form = form
        self._lib = lib
        self._cparams = params.to_c()
        self._h = handle
        self._persistent = persistent  # callable: is the ensemble in its persistent mode?

    def close(self):
        self._h = None

    def step(self, n: int = 1):
        """A member may step on its own while the ensemble steps its members'
        own launches (the default); the persistent launch needs them in step."""
        if self._persistent():
            raise DropletError(_abi.DL_ERR_STATE, "member step", "members step through Ensemble.step")
        super().step(n)


class Ensemble:
    """Members step together; member ``m`` is ``ens.members[m]`` (a Droplet
    view: set_fields, init_equilibrium, set_force, get_fields, reduce ...)."""

    def __init__(self, params_list, shapes, form: int = FORM_FP32):
        if len(params_list) != len(shapes) or not params_list:
            raise ValueError("one parameter set per member shape")
        self._lib = load()
        n = len(params_list)
        cps = (_abi.DLParams * n)(*[p.to_c() for p in params_list])
        dims = (C.c_int * (3 * n))(*[int(v) for s in shapes for v in s])
        b = C.c_void_p()
        rc = self._lib.dl_batch_create(cps, dims, n, int(form), C.byref(b))
        if rc != 0:
            raise DropletError(rc, "dl_batch_create")
        self._b = b
        self.form = form
        self.members = []
        for m in range(n):
            h = C.c_void_p()
            self._chk(self._lib.dl_batch_member(b, m, C.byref(h)), "dl_batch_member")
            self.members.append(_Member(self._lib, h, params_list[m], shapes[m], form,
                                        lambda: bool(self.get_option("persistent"))))

    def _chk(self, rc, what):
        if rc != 0:
            detail = self.members[0]._detail() if getattr(self, "members", None) else ""
            raise DropletError(rc, what, detail)

    @property
    def n_sites(self) -> int:
        return sum(m.n_sites for m in self.members)

    def step(self, n: int = 1):
        self._chk(self._lib.dl_batch_step(self._b, int(n)), "dl_batch_step")

    def set_stream(self, stream_ptr: int):
        self._chk(self._lib.dl_batch_set_stream(self._b, C.c_void_p(int(stream_ptr))), "dl_batch_set_stream")

    def set_option(self, key: str, value: int):
        self._chk(self._lib.dl_batch_set_option(self._b, key.encode(), C.c_int64(int(value))), "dl_batch_set_option")

    def get_option(self, key: str) -> int:
        v = C.c_int64()
        self._chk(self._lib.dl_batch_get_option(self._b, key.encode(), C.byref(v)), "dl_batch_get_option")
        return int(v.value)

    def profile(self, enable: bool = True, every: int = 1):
        for m in self.members:
            m.profile(enable, every)

    def profile_read(self) -> dict:
        """Launch counts and event-timed durations summed over the members (the
        persistent mode counts its launches on member 0; with concurrent member
        launches the summed durations exceed the wall time)."""
        tot = None
        for m in self.members:
            s = m.profile_read()
            tot = dict(s) if tot is None else {k: tot[k] + s[k] for k in tot}
        return tot

    def sync(self):
        for m in self.members:
            m.sync()

    def close(self):
        if getattr(self, "_b", None) is not None:
            for m in self.members:
                m.close()
            self._lib.dl_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
