"""Host diagnostics (no GPU): deformation from the second-moment tensor and the
reference's mid-plane inertia-tensor measure on analytic shapes."""
import math

import numpy as np

from droplet_gb300 import Params, diagnostics, init_fields


def ellipsoid_phi(shape, P, c, axes):
    nx, ny, nz = shape
    x, y, z = init_fields.grid(shape)
    r = ((x - c[0]) / axes[0]) ** 2 + ((y - c[1]) / axes[1]) ** 2 + ((z - c[2]) / axes[2]) ** 2
    return np.where(r <= 1.0, P.phi2, P.phi1)


def moments_dict(phi, P):
    nz, ny, nx = phi.shape
    x, y, z = init_fields.grid((nx, ny, nz))
    w = (phi - P.phi1) / (P.phi2 - P.phi1)
    return {
        "w_sum": w.sum(),
        "w_x": [(w * x).sum(), (w * y).sum(), (w * z).sum()],
        "w_xx": [(w * x * x).sum(), (w * y * y).sum(), (w * z * z).sum(), (w * x * y).sum(), (w * x * z).sum(),
                 (w * y * z).sum()],
    }


def test_deformation_sphere_is_zero_and_spheroid_matches_axes():
    P = Params.lbm_drop_xy()
    shape = (64, 64, 64)
    d0 = diagnostics.deformation_from_moments(moments_dict(ellipsoid_phi(shape, P, (31.5, 31.5, 31.5), (12, 12, 12)), P))
    assert abs(d0) < 1e-3
    a, b = 16.0, 10.0
    d1 = diagnostics.deformation_from_moments(moments_dict(ellipsoid_phi(shape, P, (31.5, 31.5, 31.5), (a, b, b)), P))
    assert abs(d1 - (a - b) / (a + b)) < 0.01


def test_midplane_deformation_of_tilted_ellipse():
    """Ellipse in the x-z plane with axes 15 and 9 rotated by 30 degrees."""
    P = Params.lbm_drop_xy()
    nx, ny, nz = 80, 9, 80
    x = np.arange(nx)[None, :] - 39.5
    z = np.arange(nz)[:, None] - 39.5
    t = math.radians(30)
    xr = x * math.cos(t) + z * math.sin(t)
    zr = -x * math.sin(t) + z * math.cos(t)
    inside = (xr / 15.0) ** 2 + (zr / 9.0) ** 2 <= 1.0
    phi = np.full((nz, ny, nx), P.phi1)
    phi[:, ny // 2, :] = np.where(inside, P.phi2, P.phi1)
    D = diagnostics.deformation_midplane(phi, P.phi1)
    assert abs(abs(D) - (15 - 9) / (15 + 9)) < 0.02


def test_laplace_pressure_and_volume():
    d = {"p_in": 10.0, "n_in": 5.0, "p_out": 3.0, "n_out": 3.0, "vol_count": 7.0, "vol_smooth": 6.5}
    assert diagnostics.laplace_pressure(d) == 2.0 - 1.0
    assert diagnostics.volume(d) == {"count": 7.0, "smooth": 6.5}
