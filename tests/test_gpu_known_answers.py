"""Physics known answers of the reference's equations, run through the GPU
forms (the reference ships no golden vectors, so these pin behaviour beyond
the oracle's few-step parity):

* Laplace law: a droplet relaxed in a periodic box has
  dp = p_in - p_out = 2 sigma / R with the reference's fit
  sigma = 1.7039 kappag^0.9991 (program/lbm_drop_xy.f90:51, where it is
  inverted to set kappag). Measured with dl_reduce's inside/outside means and
  R from the smooth volume; tolerance 3 %.
* Static vortex forcing (externalforce, program/lbm_drop_xy.f90:668-693):
  the forced Taylor-Green mode relaxes to the Stokes amplitude
  U0 = A / (2 nu kw^2); tolerance 0.5 % after 6000 steps (about 12 viscous
  times), pattern correlation with the force above 0.99999, and no flow
  across the forcing plane beyond the form's storage rounding (|u2| below
  1e-9, 1e-6, 1e-4 of U0 for FP64, FP32, FP16 storage).
"""
import math

import numpy as np
import pytest

from droplet_gb300 import Params, init_fields, _abi
from droplet_gb300.params import static_vortex_force
from droplet_gb300.solver import Droplet, FORM_FP64, FORM_FP32, FORM_FP16

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("form,kappag", [(FORM_FP64, 2e-3), (FORM_FP32, 2e-3), (FORM_FP32, 5e-4),
                                         (FORM_FP16, 2e-3)])
def test_laplace_law(form, kappag):
    n = 64
    shape = (n, n, n)
    P = Params.lbm_drop_xy().replace(kappag=kappag, nu1=0.1, nu2=0.1, tauf=0.7)
    phi = init_fields.tanh_droplets(shape, P, [(n / 2 - 0.5, n / 2 - 0.5, n / 2 - 0.5)], [12.0], width=2.0)
    g = Droplet(P, shape, form)
    g.set_fields(**init_fields.fields(phi))
    g.init_equilibrium()
    g.step(4000)
    d = g.reduce()
    assert d["nan_flag"] == 0 and d["n_in"] > 0 and d["n_out"] > 0
    dp = d["p_in"] / d["n_in"] - d["p_out"] / d["n_out"]
    R = (3.0 * d["vol_smooth"] / (4.0 * math.pi)) ** (1.0 / 3.0)
    sigma = dp * R / 2.0
    fit = 1.7039 * kappag ** 0.9991
    assert abs(sigma / fit - 1.0) < 0.03, (sigma, fit, R)


@pytest.mark.parametrize("form", [FORM_FP64, FORM_FP32, FORM_FP16])
@pytest.mark.parametrize("single_phase", [False, True])
def test_static_vortex_steady_state(form, single_phase):
    U, D, Re, nu = 0.01, 32.0, 1.0, 0.1
    nx, ny, nz = 64, 4, 64
    fx, fy, fz = static_vortex_force(nx, ny, nz, umax=U, D_vortex=D, Re=Re)
    amp = 2.0 * math.pi ** 2 * U * U / (D * Re)
    kw = math.pi / D
    U0 = amp / (2.0 * nu * kw * kw)
    # uniform phi: constant viscosity (the min/max interpolation would divide 0 by 0)
    P = Params.lbm_drop_xy().replace(nu1=nu, nu2=nu, visc_mode=_abi.DL_VISC_FIXED)
    g = Droplet(P, (nx, ny, nz), form, single_phase=single_phase)
    g.set_fields(**init_fields.fields(np.full((nz, ny, nx), P.phi1)))
    g.init_equilibrium()
    g.set_force(_abi.DL_FORCE_STATIC, fx, fy, fz)
    g.step(6000)
    f = g.get_fields()
    u1 = f["u1"]
    assert np.isfinite(u1).all()
    assert abs(np.abs(u1).max() / U0 - 1.0) < 5e-3, np.abs(u1).max() / U0
    corr = float((u1 * fx).sum() / math.sqrt((u1 ** 2).sum() * (fx ** 2).sum()))
    assert corr > 0.99999, corr
    assert np.abs(f["u2"]).max() < {FORM_FP64: 1e-9, FORM_FP32: 1e-6, FORM_FP16: 1e-4}[form] * U0
