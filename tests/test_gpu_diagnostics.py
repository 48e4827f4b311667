"""Whole-domain diagnostics of dl_reduce on the GPU against NumPy
restatements evaluated on the fields the handle holds, for every form: the
second moments of w = (phi - phi1)/(phi2 - phi1) that the deformation D is
built from (prototype_program/two-phase/drop8_mpi.f90:812-970 in its 3-D
form), and the dissipation 2 nu(phi) S:S (program/energy_budget.f90:1494).
Then the reference's own mid-plane measure (break_up3, restated in
droplet_gb300.diagnostics) on the fields of a sheared droplet stepped on the
GPU, against the same measure on the oracle's fields.

Tolerances: the device sums are FP64 over terms formed from the stored
fields; they agree with NumPy to 1e-12 relative to the sum of the terms'
magnitudes (moments) and 1e-9 relative (dissipation, whose gradient the FP32
and FP16 forms form in FP32 as their step does: 2e-6 relative there)."""
import numpy as np
import pytest

from droplet_gb300 import Params, configs, diagnostics, init_fields
from droplet_gb300.adjoint import deformation_from_diag
from droplet_gb300.solver import Droplet, FORM_FP16, FORM_FP32, FORM_FP64
from oracle import np_energy, pyoracle

pytestmark = pytest.mark.gpu

FORMS = [FORM_FP64, FORM_FP32, FORM_FP16]


def stepped(form, shape=(40, 32, 28), steps=6):
    P = Params.lbm_drop_xy().replace(tauf=0.8, nu1=0.1, nu2=0.05, kappag=2e-3)
    nx, ny, nz = shape
    phi = init_fields.tanh_droplets(shape, P, [(15.3, 17.0, 13.6)], [7.0], width=1.5)
    u = init_fields.random_solenoidal(shape, 5, kmin=1.0, kmax=3.0, urms=0.02)
    g = Droplet(P, shape, form)
    g.set_fields(**init_fields.fields(phi, *u))
    g.init_equilibrium()
    g.step(steps)
    return P, g


@pytest.mark.parametrize("form", FORMS)
def test_deformation_moments_match_numpy(form):
    P, g = stepped(form)
    d = g.reduce()
    f = g.get_fields()
    ref = np_energy.second_moments(P, f["phi"])
    n = f["phi"].size
    wmax = float(np.abs((f["phi"] - P.phi1) / (P.phi2 - P.phi1)).max())
    ext = float(max(g.nx, g.ny, g.nz))
    assert d["w_sum"] == pytest.approx(ref["w_sum"], rel=0, abs=1e-12 * n * wmax)
    np.testing.assert_allclose(d["w_x"], ref["w_x"], rtol=0, atol=1e-12 * n * wmax * ext)
    np.testing.assert_allclose(d["w_xx"], ref["w_xx"], rtol=0, atol=1e-12 * n * wmax * ext * ext)
    # the deformation built from the device moments equals the one from the fields
    D_dev, _ = deformation_from_diag(d, P.phi1, P.phi2)
    D_np = diagnostics.deformation_from_moments(ref)
    assert D_dev == pytest.approx(D_np, rel=0, abs=1e-9)
    g.close()


@pytest.mark.parametrize("form", FORMS)
def test_dissipation_matches_numpy(form):
    P, g = stepped(form)
    d = g.reduce()
    f = g.get_fields()
    ref = np_energy.dissipation_sum(P, f["u1"], f["u2"], f["u3"], f["phi"])
    rel = 1e-9 if form == FORM_FP64 else 2e-6
    assert d["diss"] == pytest.approx(ref, rel=rel)
    g.close()


@pytest.mark.parametrize("form", FORMS)
def test_midplane_deformation_of_gpu_fields(form):
    """A droplet in Couette shear (walls +-0.04 in x), 32^3, 300 steps: the
    mid-plane D of the GPU fields against the mid-plane D of the oracle's
    fields (the FP64 form: identical; FP32/FP16: within 2e-4); the droplet
    has deformed (D > 0.01), and the 3-D D of the device moments agrees
    with the 3-D D of the downloaded fields."""
    w = configs.shear_droplet(n=32, radius=8.0, U=0.04, Ca=0.3, steps=300)
    g = Droplet(w.params, w.shape, form)
    o = pyoracle.OracleDroplet(w.params, w.shape)
    for s in (g, o):
        s.set_fields(**w.fields)
        s.init_equilibrium()
        s.step(w.steps)
    fg, fo = g.get_fields(), o.get_fields()
    Dg = diagnostics.deformation_midplane(fg["phi"], w.params.phi1)
    Do = diagnostics.deformation_midplane(fo["phi"], w.params.phi1)
    assert abs(Do) > 0.01
    if form == FORM_FP64:
        assert Dg == Do
    else:
        assert abs(Dg - Do) <= 2e-4, (Dg, Do)
    D3_dev, _ = deformation_from_diag(g.reduce(), w.params.phi1, w.params.phi2)
    D3_np = diagnostics.deformation_from_moments(np_energy.second_moments(w.params, fg["phi"]))
    assert D3_dev == pytest.approx(D3_np, rel=0, abs=1e-9)
    g.close()
    o.close()
