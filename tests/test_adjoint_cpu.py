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
