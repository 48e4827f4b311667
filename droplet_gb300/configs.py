"""The benchmark workloads: synthetic, seeded inputs with the sizes and
physics of the five measurement cases. The reference publishes no benchmark
and its inputs (precursor turbulence files) are not available, so every
field here is generated from a seed.

Parameter mapping onto the reference's own parameter set
(program/lbm_drop_xy.f90:31-59):
  * phi is Inamuro's index function (phi1 = 2.211, phi2 = 4.895, van der
    Waals a = 9/49, b = 2/21, T = 0.55); "phi in [-1, 1]" is the map
    phi~ = 2 (phi - phi1)/(phi2 - phi1) - 1 (init_fields.phi_tilde);
  * the mobility is not a free parameter of the model: it is
    Gamma = (tau_f - 1/2) ds (Params.mobility), set through tau_f;
  * kappa = kappaf; kappag follows from the surface tension through the
    reference's Laplace-law fit sigma = 1.7039 kappag**0.9991 (:51), with
    sigma from the capillary number Ca = (2U/H) nu R / sigma of the shear
    prototype (prototype_program/two-phase/drop8_mpi.f90:57-58) or from the
    Weber number We = u'^2 D / sigma in turbulence;
  * density and viscosity ratios are 1 (nu2 = nu1, eta = 1).
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import init_fields
from .params import Params, kappag_from_sigma
from . import _abi


@dataclasses.dataclass
class Workload:
    name: str
    params: Params
    shape: tuple          # (nx, ny, nz)
    form: int
    steps: int
    fields: dict          # phi, u1, u2, u3, p with shape (nz, ny, nx)
    force_mode: int
    seed: int
    notes: str = ""
    single_phase: bool = False  # the g-only precursor step (DL_SINGLE_PHASE)

    @property
    def n_sites(self) -> int:
        nx, ny, nz = self.shape
        return nx * ny * nz


def shear_droplet(n: int = 64, radius: float = 12.0, U: float = 0.05, Ca: float = 0.3, tauf: float = 1.0,
                  taug: float = 0.8, kappaf: float = 0.01, width: float = 2.0,
                  form: int = _abi.DL_FORM_FP64, steps: int = 2000) -> Workload:
    """Single droplet in planar Couette shear between walls at z = 0 and
    z = n-1 moving with -U and +U in x; initial linear shear profile."""
    shape = (n, n, n)
    nu = (taug - 0.5) / 3.0
    H = float(n - 1)
    sigma = (2.0 * U / H) * nu * radius / Ca
    P = Params.lbm_drop_xy().replace(tauf=tauf, nu1=nu, nu2=nu, kappaf=kappaf, kappag=kappag_from_sigma(sigma),
                                     walls=True, wall_u=(U, 0.0, 0.0), wall_start=1)
    c = (n - 1) / 2.0
    phi = init_fields.tanh_droplets(shape, P, [(c, c, c)], [radius], width=width)
    f = init_fields.fields(phi, init_fields.couette_u(shape, U))
    return Workload(f"shear_droplet_{n}^3", P, shape, form, steps, f, _abi.DL_FORCE_NONE, 0,
                    f"Ca={Ca} sigma={sigma:.4g} R={radius}")


def config1() -> Workload:
    """64^3 FP64 shear droplet, R = 12, walls +-0.05, tau_g = 0.8, tau_f = 1.0,
    kappaf = 0.01, Ca = 0.3, 2000 steps (deterministic)."""
    return shear_droplet()


def forced_turbulence(n: int = 128, centers=None, radius: float = 16.0, We: float = 5.0, urms: float = 0.01,
                      taug: float = 0.52, Cs: float = 0.1, eps: float = 1e-6, kc: int = 3, seed: int = 1,
                      form: int = _abi.DL_FORM_FP32, steps: int = 5000, width: float = 2.0) -> Workload:
    """Periodic box with Smagorinsky LES and constant-injection band forcing;
    random-phase solenoidal initial velocity on 1 <= |k| <= 2 from ``seed``."""
    shape = (n, n, n)
    nu = (taug - 0.5) / 3.0
    if centers is None:
        c = (n - 1) / 2.0
        centers = [(c, c, c)]
    D = 2.0 * radius
    sigma = urms * urms * D / We
    P = Params.lbm_drop_xy().replace(tauf=0.7, nu1=nu, nu2=nu, kappaf=0.01, kappag=kappag_from_sigma(sigma),
                                     les=True, Cs=Cs, delta=1.0, eps=eps, kc=kc)
    phi = init_fields.tanh_droplets(shape, P, centers, [radius] * len(centers), width=width)
    u = init_fields.random_solenoidal(shape, seed, kmin=1.0, kmax=2.0, urms=urms)
    f = init_fields.fields(phi, *u)
    return Workload(f"forced_turbulence_{n}^3", P, shape, form, steps, f, _abi.DL_FORCE_SPECTRAL, seed,
                    f"We={We} sigma={sigma:.4g} urms={urms} eps={eps}")


def config2(form: int = _abi.DL_FORM_FP32) -> Workload:
    """128^3 FP32 forced turbulence, one droplet R = 16, LES Cs = 0.1,
    tau_g = 0.52, eps = 1e-6, 5000 steps."""
    return forced_turbulence(form=form)


def place_droplets(n: int, count: int, radius: float, seed: int, margin: float = 2.0):
    """Seeded non-overlapping droplet centres in a periodic box."""
    rng = np.random.default_rng(seed)
    centers = []
    tries = 0
    while len(centers) < count:
        tries += 1
        if tries > 100000:
            raise RuntimeError("could not place droplets")
        c = rng.uniform(0, n, size=3)
        ok = True
        for d in centers:
            dd = np.abs(c - np.asarray(d))
            dd = np.minimum(dd, n - dd)
            if np.sqrt((dd * dd).sum()) < 2 * radius + 2 * margin:
                ok = False
                break
        if ok:
            centers.append(tuple(float(v) for v in c))
    return centers


def config3(seed: int = 3) -> Workload:
    """256^3 FP16-storage forced turbulence with 8 seed-placed droplets R = 12,
    3000 steps."""
    centers = place_droplets(256, 8, 12.0, seed)
    w = forced_turbulence(n=256, centers=centers, radius=12.0, seed=seed, form=_abi.DL_FORM_FP16, steps=3000)
    w.name = "forced_turbulence_8drops_256^3"
    return w


def ensemble_members(n_members: int = 64, seed: int = 4, sizes=(48, 64, 96), webers=(2.0, 5.0, 10.0, 20.0),
                     urms: float = 0.01, form: int = _abi.DL_FORM_FP32):
    """Members of the batched ensemble: grid L drawn uniformly from ``sizes``,
    droplet radius 0.15 L at the centre plus a uniform offset within +-4
    cells, Weber number drawn from ``webers``, its own forcing-phase seed.
    Physics as the forced-turbulence case (LES, band forcing)."""
    rng = np.random.default_rng(seed)
    out = []
    for m in range(n_members):
        L = int(rng.choice(sizes))
        We = float(rng.choice(webers))
        off = rng.uniform(-4.0, 4.0, size=3)
        c = (L - 1) / 2.0
        mseed = int(rng.integers(0, 2**31 - 1))
        w = forced_turbulence(n=L, centers=[tuple(c + off)], radius=0.15 * L, We=We, urms=urms, seed=mseed,
                              form=form, steps=2000)
        w.name = f"member{m}_L{L}_We{We:g}"
        out.append(w)
    return out


def config4(n_members: int = 64, seed: int = 4):
    """64 FP32 members, L in {48, 64, 96}, R = 0.15 L, We in {2, 5, 10, 20},
    offsets within +-4 cells, 2000 steps."""
    return ensemble_members(n_members=n_members, seed=seed)


def config5(n: int = 96) -> Workload:
    """Adjoint workload: 96^3 shear droplet (config-1 physics), R = 18,
    walls +-0.04, FP32, 500 steps; loss = deformation at the final step."""
    return shear_droplet(n=n, radius=18.0 * n / 96.0, U=0.04, form=_abi.DL_FORM_FP32, steps=500)


def precursor(n: int = 256, form: int = _abi.DL_FORM_FP32, steps: int = 2000, nu: float = 0.001, kc: int = 3,
              eta: float = 1.0) -> Workload:
    """Single-phase forced turbulence, the precursor program
    program/lbm_iht_xy.f90: nu = 0.001, band forcing on 1 <= |k| < kc = 3 with
    eps = nu^3 / eta^4 (Kolmogorov scale eta = 1 ds, :31-34), started from its
    Taylor-Green-like field (ini, :238-243): u1 = -A cos(kx) sin(kz),
    u3 = A sin(kx) cos(kz), p = 1/3 - A^2/4 (cos 2kx + cos 2kz), A = 1e-4."""
    shape = (n, n, n)
    eps = nu ** 3 / eta ** 4
    P = Params.lbm_drop_xy().replace(nu1=nu, nu2=nu, kappaf=0.0, kappag=0.0, eps=eps, kc=kc,
                                     visc_mode=_abi.DL_VISC_FIXED)
    x, y, z = init_fields.grid(shape)
    k = 2.0 * np.pi / n
    A = 1e-4
    u1 = -A * np.cos(k * x) * np.sin(k * z)
    u3 = A * np.sin(k * x) * np.cos(k * z)
    p = 1.0 / 3.0 - A * A / 4.0 * (np.cos(2.0 * k * x) + np.cos(2.0 * k * z))
    f = init_fields.fields(np.full(shape[::-1], P.phi1), u1, np.zeros_like(u1), u3, p)
    return Workload(f"precursor_turbulence_{n}^3", P, shape, form, steps, f, _abi.DL_FORCE_SPECTRAL, 0,
                    f"single phase, nu={nu} eps={eps:.3g} kc={kc}", single_phase=True)


WORKLOADS = {"config1": config1, "config2": config2, "config3": config3, "config4": config4, "config5": config5,
             "precursor": precursor}
