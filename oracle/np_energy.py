"""NumPy restatements of the in-situ energy diagnostics (checkers of
dl_energy). TEST INFRASTRUCTURE ONLY.

* spectrum: enesupe_cal, program/turbulence_hit_xy.f90:588-645, with
  u_hat = FFT(u)/N (fft_r2c, :725-730) and the signed wavenumbers of the function judge
  (:739-746): over k1 in [0,nx), k2 in [0,ny), k3 in [0,nz/2],
  E[int(|k|)] += 0.5 (|u1_hat|^2 + |u2_hat|^2 + |u3_hat|^2) (1 if k3 == 0 else 2).
* free energy: free_energy_cal (program/energy_budget.f90:1012-1023) and
  chemical_potencial_cal (:998-1010) with the 14-neighbour Laplacian of
  various_cal (program/lbm_drop_xy.f90:608-613).
Fields have shape (nz, ny, nx).
"""
from __future__ import annotations

import numpy as np

from .np_oracle import CR, shifted


def signed(k, n):
    return np.where(k >= n // 2 + 1, k - n, k)


def spectrum(u1, u2, u3, nbins):
    nz, ny, nx = u1.shape
    N = nx * ny * nz
    e2 = sum(np.abs(np.fft.fftn(u)) ** 2 for u in (u1, u2, u3)) / float(N) ** 2  # [k3][k2][k1]
    k3 = np.arange(nz // 2 + 1)
    e2 = e2[: nz // 2 + 1]
    K3, K2, K1 = np.meshgrid(k3, np.arange(ny), np.arange(nx), indexing="ij")
    s1, s2, s3 = signed(K1, nx), signed(K2, ny), signed(K3, nz)
    kidx = np.sqrt((s1 * s1 + s2 * s2 + s3 * s3).astype(np.float64)).astype(np.int64)
    w = np.where(K3 == 0, 1.0, 2.0)
    v = 0.5 * e2 * w
    keep = kidx < nbins
    return np.bincount(kidx[keep].ravel(), weights=v[keep].ravel(), minlength=nbins)[:nbins]


def free_energy_sums(P, phi):
    lap = -(14.0 * phi)
    g = [np.zeros_like(phi) for _ in range(3)]
    for i in range(1, 15):
        v = shifted(phi, i)
        lap = lap + v
        for a in range(3):
            g[a] = g[a] + CR[i][a] * v
    lap = lap / (5.0 * P.ds * P.ds)
    omb = 1.0 - P.b * phi
    lg = np.log(phi / omb)
    psi = phi * P.T * lg - P.a * phi * phi
    mu = (P.T * lg + P.T / omb - 2.0 * P.a * phi) - P.kappag * lap
    gsq = (g[0] * g[0] + g[1] * g[1] + g[2] * g[2]) / (10.0 * P.ds) ** 2
    return float(psi.sum()), float(mu.sum()), float(gsq.sum())


def dissipation_sum(P, u1, u2, u3, phi):
    """Sum over sites of 2 nu(phi) S:S (program/energy_budget.f90:1494), with
    grad u from the 14-neighbour stencil of various_cal
    (program/lbm_drop_xy.f90:615-633) and nu(phi) linear in
    w = (phi - phi1)/(phi2 - phi1) between nu1 and nu2."""
    u = (u1, u2, u3)
    G = [[np.zeros_like(u1) for _ in range(3)] for _ in range(3)]  # G[a][b] = d u_b / d x_a
    for i in range(1, 15):
        for b in range(3):
            v = shifted(u[b], i)
            for a in range(3):
                if CR[i][a] != 0.0:
                    G[a][b] = G[a][b] + CR[i][a] * v
    gd = 10.0 * P.ds
    G = [[G[a][b] / gd for b in range(3)] for a in range(3)]
    ss = sum(G[a][a] * G[a][a] for a in range(3))
    for a, b in ((0, 1), (0, 2), (1, 2)):
        s = 0.5 * (G[a][b] + G[b][a])
        ss = ss + 2.0 * s * s
    w = (phi - P.phi1) / (P.phi2 - P.phi1)
    nu = P.nu1 + w * (P.nu2 - P.nu1)
    return float((2.0 * nu * ss).sum())


def second_moments(P, phi):
    """w_sum, w_x (x, y, z) and w_xx (xx, yy, zz, xy, xz, yz) of
    w = (phi - phi1)/(phi2 - phi1) over the sites, coordinates = site indices."""
    nz, ny, nx = phi.shape
    z, y, x = np.meshgrid(np.arange(nz, dtype=np.float64), np.arange(ny, dtype=np.float64),
                          np.arange(nx, dtype=np.float64), indexing="ij")
    w = (phi - P.phi1) / (P.phi2 - P.phi1)
    return {"w_sum": float(w.sum()),
            "w_x": [float((w * x).sum()), float((w * y).sum()), float((w * z).sum())],
            "w_xx": [float((w * x * x).sum()), float((w * y * y).sum()), float((w * z * z).sum()),
                     float((w * x * y).sum()), float((w * x * z).sum()), float((w * y * z).sum())]}
