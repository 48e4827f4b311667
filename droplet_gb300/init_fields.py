"""Initial conditions for the droplet step (host side, NumPy).

``sharp_sphere`` is the reference's own initial condition (ini,
program/lbm_drop_xy.f90:224-242). The others build the synthetic inputs of
the benchmark workloads: tanh-profile droplets, the linear Couette profile
between the moving walls, and a seeded random-phase solenoidal velocity field
(the reference reads a precursor turbulence file instead, which is not
available; program/lbm_drop_xy.f90:789-823).

All arrays have shape (nz, ny, nx).
"""
from __future__ import annotations

import numpy as np

from .params import Params


def grid(shape):
    nx, ny, nz = shape
    z, y, x = np.meshgrid(np.arange(nz, dtype=np.float64), np.arange(ny, dtype=np.float64),
                          np.arange(nx, dtype=np.float64), indexing="ij")
    return x, y, z


def sharp_sphere(shape, params: Params, center, diameter: float):
    """phi = phi2 inside the sphere |x - c| <= D/2, phi1 outside; u = 0; p = 1/3
    (program/lbm_drop_xy.f90:229-240)."""
    x, y, z = grid(shape)
    ds = params.ds
    xc, yc, zc = center
    dif = (x * ds - xc) ** 2 + (y * ds - yc) ** 2 + (z * ds - zc) ** 2
    phi = np.where(dif <= (0.5 * diameter) ** 2, params.phi2, params.phi1)
    zeros = np.zeros_like(phi)
    return dict(phi=phi, u1=zeros.copy(), u2=zeros.copy(), u3=zeros.copy(), p=np.full_like(phi, 1.0 / 3.0))


def phi_tilde(params: Params, phi):
    """The presentation map phi~ = 2 (phi - phi1)/(phi2 - phi1) - 1 in [-1, 1]."""
    return 2.0 * (np.asarray(phi) - params.phi1) / (params.phi2 - params.phi1) - 1.0


def phi_from_tilde(params: Params, pt):
    return params.phi1 + (params.phi2 - params.phi1) * (np.asarray(pt) + 1.0) / 2.0


def tanh_droplets(shape, params: Params, centers, radii, width: float = 2.0):
    """phi~ = max_k tanh((R_k - |x - c_k|)/width), mapped back to phi.
    Distances are taken with periodic wrap."""
    nx, ny, nz = shape
    x, y, z = grid(shape)
    pt = np.full((nz, ny, nx), -1.0)
    for c, r in zip(centers, radii):
        dx = np.abs(x - c[0]); dx = np.minimum(dx, nx - dx)
        dy = np.abs(y - c[1]); dy = np.minimum(dy, ny - dy)
        dz = np.abs(z - c[2]); dz = np.minimum(dz, nz - dz)
        d = np.sqrt(dx * dx + dy * dy + dz * dz)
        pt = np.maximum(pt, np.tanh((r - d) / width))
    return phi_from_tilde(params, pt)


def couette_u(shape, wall_u: float):
    """Linear profile u_x(z) = U (2 z/(nz-1) - 1) between the bottom wall
    (-U at z = 0) and the top wall (+U at z = nz-1)."""
    nx, ny, nz = shape
    z = np.arange(nz, dtype=np.float64)
    prof = wall_u * (2.0 * z / (nz - 1) - 1.0)
    return np.broadcast_to(prof[:, None, None], (nz, ny, nx)).copy()


def random_solenoidal(shape, seed: int, kmin: float = 1.0, kmax: float = 2.0, urms: float = 0.01):
    """Seeded random-phase velocity field with energy on kmin <= |k| <= kmax,
    projected onto divergence-free modes and scaled to the given rms speed."""
    nx, ny, nz = shape
    rng = np.random.default_rng(seed)
    kx = np.fft.fftfreq(nx, 1.0 / nx)[None, None, :]
    ky = np.fft.fftfreq(ny, 1.0 / ny)[None, :, None]
    kz = np.fft.fftfreq(nz, 1.0 / nz)[:, None, None]
    kk = np.sqrt(kx * kx + ky * ky + kz * kz)
    band = (kk >= kmin) & (kk <= kmax)
    comps = []
    for _ in range(3):
        amp = rng.standard_normal((nz, ny, nx)) + 1j * rng.standard_normal((nz, ny, nx))
        comps.append(np.where(band, amp, 0.0))
    # solenoidal projection: u_hat - k (k . u_hat)/|k|^2
    k2 = np.where(kk > 0, kk * kk, 1.0)
    kdotu = kx * comps[0] + ky * comps[1] + kz * comps[2]
    comps = [comps[0] - kx * kdotu / k2, comps[1] - ky * kdotu / k2, comps[2] - kz * kdotu / k2]
    u = [np.real(np.fft.ifftn(c)) for c in comps]
    rms = np.sqrt(np.mean(u[0] ** 2 + u[1] ** 2 + u[2] ** 2) / 3.0)
    scale = urms / rms if rms > 0 else 0.0
    return [np.ascontiguousarray(c * scale) for c in u]


def fields(phi, u1=None, u2=None, u3=None, p=None):
    """Bundle fields with zero velocity and p = 1/3 defaults (ini's values)."""
    phi = np.ascontiguousarray(phi, dtype=np.float64)
    z = np.zeros_like(phi)
    return dict(phi=phi,
                u1=z.copy() if u1 is None else np.ascontiguousarray(u1, dtype=np.float64),
                u2=z.copy() if u2 is None else np.ascontiguousarray(u2, dtype=np.float64),
                u3=z.copy() if u3 is None else np.ascontiguousarray(u3, dtype=np.float64),
                p=np.full_like(phi, 1.0 / 3.0) if p is None else np.ascontiguousarray(p, dtype=np.float64))
