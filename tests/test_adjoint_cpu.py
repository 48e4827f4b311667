"""The analytic gradient of the deformation loss against torch autograd (CPU)."""
import numpy as np
import torch

from droplet_gb300 import Params, init_fields
from droplet_gb300.adjoint import deformation_and_grad
from oracle import torch_ref


def test_deformation_gradient_matches_autograd():
    P = Params.lbm_drop_xy()
    shape = (20, 18, 16)
    nx, ny, nz = shape
    x, y, z = init_fields.grid(shape)
    r = ((x - 9.3) / 6.0) ** 2 + ((y - 8.6) / 4.0) ** 2 + ((z - 7.7) / 3.5) ** 2
    pt = np.tanh((1.0 - np.sqrt(r)) * 2.0)
    phi = init_fields.phi_from_tilde(P, pt)
    D, g = deformation_and_grad(phi, P.phi1, P.phi2)
    t = torch.tensor(phi, dtype=torch.float64, requires_grad=True)
    Dt = torch_ref.deformation(P, t)
    Dt.backward()
    assert abs(D - Dt.item()) < 1e-12
    assert np.abs(g - t.grad.numpy()).max() <= 1e-9 * np.abs(g).max()


def _torch_steps(P, f, nsteps, spectral):
    T = lambda a: torch.tensor(a, dtype=torch.float64)  # noqa: E731
    u0 = [T(f["u1"]), T(f["u2"]), T(f["u3"])]
    feq, geq = torch_ref.equilibria(P, T(f["phi"]), u0, T(f["p"]), P.kappaf, P.kappag)
    F, G = feq, geq
    U = torch.tensor(P.wall_u[0], dtype=torch.float64)
    for _ in range(nsteps):
        F, G = torch_ref.step(P, F, G, P.kappaf, P.kappag, P.tauf, U, 0.5 + 3.0 * P.nu1 / P.ds, spectral)
    return torch_ref.moments(F, G)


def test_torch_reference_band_force_equals_the_oracle():
    """The differentiable reference's band force (torch.fft on the band) equals
    the C oracle's separable-DFT restatement of externalforce on the same u."""
    from droplet_gb300 import configs
    from oracle import pyoracle

    w = configs.forced_turbulence(n=16, radius=3.0, urms=0.01, taug=0.6, steps=3, form=32)
    o = pyoracle.OracleDroplet(w.params, w.shape)
    o.set_fields(**w.fields)
    o.init_equilibrium()
    o.set_force(2)
    ref = o.compute_spectral_force()
    F = torch_ref.band_force(w.params, [torch.tensor(w.fields[k]) for k in ("u1", "u2", "u3")])
    for c in range(3):
        assert np.abs(F[c].numpy() - ref[c]).max() <= 1e-12 * np.abs(ref[c]).max()


def test_torch_reference_steps_equal_the_oracle():
    """Three steps of the differentiable reference against the C oracle: forced
    turbulence (Smagorinsky LES and the band force) and the shear droplet with
    viscosity ratio 3 in the fixed-range mode; FP64 both, different summation
    orders (agreement to 1e-12)."""
    from droplet_gb300 import _abi, configs
    from oracle import pyoracle

    cases = []
    w = configs.forced_turbulence(n=12, radius=3.0, urms=0.01, taug=0.6, steps=3, form=32)
    cases.append((w, w.params, True))
    w2 = configs.shear_droplet(n=12, radius=3.0, U=0.04, steps=3, form=32)
    cases.append((w2, w2.params.replace(nu2=3.0 * w2.params.nu1, visc_mode=_abi.DL_VISC_FIXED), False))
    for w, P, spectral in cases:
        o = pyoracle.OracleDroplet(P, w.shape)
        o.set_fields(**w.fields)
        o.init_equilibrium()
        if spectral:
            o.set_force(_abi.DL_FORCE_SPECTRAL)
        o.step(3)
        ref = o.get_fields()
        phi, u, p = _torch_steps(P, w.fields, 3, spectral)
        assert np.abs(phi.numpy() - ref["phi"]).max() <= 1e-12
        for c, k in enumerate(("u1", "u2", "u3")):
            assert np.abs(u[c].numpy() - ref[k]).max() <= 1e-12
