"""dl_energy on the GPU against the NumPy restatements of enesupe_cal
(program/turbulence_hit_xy.f90:588-645) and of the free-energy and
chemical-potential sums (program/energy_budget.f90:998-1023), evaluated on
the fields the handle holds (relative 1e-10 for the spectrum, whose FP64
atomics add in no fixed order; 1e-12 for the sums)."""
import numpy as np
import pytest

from droplet_gb300 import Params, init_fields
from droplet_gb300 import _abi
from droplet_gb300.solver import Droplet, FORM_FP16, FORM_FP32, FORM_FP64
from oracle import np_energy

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("form", [FORM_FP64, FORM_FP32, FORM_FP16])
@pytest.mark.parametrize("shape", [(24, 20, 16), (17, 12, 15)])
def test_energy_matches_numpy(form, shape):
    nx, ny, nz = shape
    P = Params.lbm_drop_xy().replace(tauf=0.8, nu1=0.1, nu2=0.1, kappag=2e-3)
    phi = init_fields.tanh_droplets(shape, P, [(nx / 2, ny / 2, nz / 2)], [min(shape) / 4], width=1.5)
    u = init_fields.random_solenoidal(shape, 7, kmin=1.0, kmax=3.0, urms=0.01)
    g = Droplet(P, shape, form)
    g.set_fields(**init_fields.fields(phi, *u))
    g.init_equilibrium()
    g.step(3)
    f = g.get_fields()
    nb = max(shape)
    d = g.energy(nb)
    ref = np_energy.spectrum(f["u1"], f["u2"], f["u3"], nb)
    scale = ref.max()
    assert np.allclose(d["spectrum"], ref, rtol=1e-10, atol=1e-12 * scale)
    assert np.isclose(d["spectrum_sum"], ref.sum(), rtol=1e-10)
    psi, mu, gsq = np_energy.free_energy_sums(P, f["phi"])
    assert np.isclose(d["psi_sum"], psi, rtol=1e-12)
    assert np.isclose(d["mu_sum"], mu, rtol=1e-12, atol=1e-12 * abs(psi))
    assert np.isclose(d["grad_sq_sum"], gsq, rtol=1e-11)
    d0 = g.energy(0)
    assert d0["nbins"] == 0 and np.isclose(d0["psi_sum"], psi, rtol=1e-12)
