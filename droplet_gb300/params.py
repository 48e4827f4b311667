"""Physical parameters of the droplet step, mirroring the reference's
``module globals`` (program/lbm_drop_xy.f90:10-59; the forced-turbulence
variant program/lbm_drop_iht_xy.f90:38-72; the LES variant
program/LES_drop_xy.f90:41-43; the wall prototype
prototype_program/two-phase/drop8_mpi.f90:50-74).

The reference fixes these as compile-time ``parameter`` constants; here they
are one plain struct passed through the C-ABI.
"""
from __future__ import annotations

import dataclasses
import math

from . import _abi

#: D3Q15 lattice, program/lbm_drop_xy.f90:70-84 (directions 0..14 = reference 1..15)
CX = (0, 1, 0, 0, -1, 0, 0, 1, -1, 1, 1, -1, 1, -1, -1)
CY = (0, 0, 1, 0, 0, -1, 0, 1, 1, -1, 1, -1, -1, 1, -1)
CZ = (0, 0, 0, 1, 0, 0, -1, 1, 1, 1, -1, -1, -1, -1, 1)
E = (2.0 / 9.0,) + (1.0 / 9.0,) * 6 + (1.0 / 72.0,) * 8
H = (1.0,) + (0.0,) * 14
F = (-7.0 / 3.0,) + (1.0 / 3.0,) * 6 + (1.0 / 24.0,) * 8
OPPOSITE = (0, 4, 5, 6, 1, 2, 3, 11, 12, 13, 14, 7, 8, 9, 10)


def kappag_from_sigma(sigma: float) -> float:
    """Surface-tension parameter from sigma with the reference's Laplace-law
    fit sigma = 1.7039 kappag**0.9991 (program/lbm_drop_xy.f90:51)."""
    return (sigma / 1.7039) ** (1.0 / 0.9991)


def sigma_from_kappag(kappag: float) -> float:
    """Inverse of :func:`kappag_from_sigma`."""
    return 1.7039 * kappag ** 0.9991


@dataclasses.dataclass
class Params:
    """Parameters of one droplet simulation (reference names)."""

    ds: float = 1.0
    tauf: float = 0.7
    kappaf: float = 0.01
    kappag: float = 1.0e-3
    phi1: float = 2.211
    phi2: float = 4.895
    a: float = 9.0 / 49.0
    b: float = 2.0 / 21.0
    T: float = 0.55
    nu1: float = 0.1
    nu2: float = 0.1
    Anu: float = 0.0
    Cs: float = 0.0
    delta: float = 0.0
    wall_u: tuple = (0.0, 0.0, 0.0)
    eps: float = 0.0
    wall_start: int = 1
    visc_mode: int = _abi.DL_VISC_MINMAX
    les: bool = False
    walls: bool = False
    kc: int = 3

    # ---- derived quantities ------------------------------------------------
    @property
    def taug_bulk(self) -> float:
        """tau_g of phase 1 without eddy viscosity: 0.5 + 3 nu1/ds + 2/3 Anu."""
        return 0.5 + 3.0 * self.nu1 / self.ds + 2.0 / 3.0 * self.Anu

    @property
    def mobility(self) -> float:
        """Gamma = (tau_f - 1/2) ds sum_i F_i c_ix^2 = (tau_f - 1/2) ds: the
        implicit mobility of Inamuro's model (sum_i F_i c_ix^2 = 1)."""
        return (self.tauf - 0.5) * self.ds

    @property
    def sigma(self) -> float:
        return sigma_from_kappag(self.kappag)

    def to_c(self) -> _abi.DLParams:
        c = _abi.DLParams()
        for f in dataclasses.fields(self):
            v = getattr(self, f.name)
            if f.name == "wall_u":
                c.wall_u = (_abi.C.c_double * 3)(*[float(x) for x in v])
            elif f.name in ("les", "walls", "visc_mode", "kc", "wall_start"):
                setattr(c, f.name, int(v))
            else:
                setattr(c, f.name, float(v))
        return c

    def replace(self, **kw) -> "Params":
        return dataclasses.replace(self, **kw)

    # ---- the reference's own parameter sets --------------------------------
    @classmethod
    def lbm_drop_xy(cls) -> "Params":
        """Values of program/lbm_drop_xy.f90:31-59 (vortex-forced droplet)."""
        Re, eta, Ca = 0.01, 1.0, 10.0
        D_vortex, D_ratio, umax = 127.5, 0.375, 0.0001
        nu1 = umax * D_vortex * D_ratio / Re
        sigma = nu1 * umax / Ca
        return cls(tauf=0.7, kappaf=0.01, kappag=kappag_from_sigma(sigma), nu1=nu1, nu2=eta * nu1)

    @classmethod
    def lbm_drop_iht_xy(cls, We: float = 20.0, D: float = 70.0) -> "Params":
        """Values of program/lbm_drop_iht_xy.f90:38-72 (forced-turbulence droplet)."""
        nu1 = 0.001
        sigma = (9.15e-10) ** (2.0 / 3.0) * D ** (5.0 / 3.0) / We
        return cls(tauf=0.7, kappaf=0.06, kappag=sigma / 2.95e-3, phi1=0.2638, phi2=0.4031,
                   a=1.0, b=1.0, T=0.293, nu1=nu1, nu2=nu1, eps=nu1 ** 3 / 1.0 ** 4, kc=3)


def static_vortex_force(nx: int, ny: int, nz: int, umax: float = 0.0001, D_vortex: float = 127.5,
                        Re: float = 0.01):
    """Body force of externalforce, program/lbm_drop_xy.f90:668-693:
    Fx = 2 pi^2 U^2/(D Re) sin(kw x) cos(kw z), Fy = 0,
    Fz = -2 pi^2 U^2/(D Re) cos(kw x) sin(kw z), kw = pi / D."""
    import numpy as np

    pi = math.acos(-1.0)
    kw = pi / D_vortex
    x = np.arange(nx, dtype=np.float64)[None, None, :]
    z = np.arange(nz, dtype=np.float64)[:, None, None]
    amp = 2.0 * pi * pi * umax * umax / (D_vortex * Re)
    fx = amp * np.sin(kw * x) * np.cos(kw * z) * np.ones((nz, ny, nx))
    fz = -amp * np.cos(kw * x) * np.sin(kw * z) * np.ones((nz, ny, nx))
    fy = np.zeros((nz, ny, nx))
    return fx, fy, fz
