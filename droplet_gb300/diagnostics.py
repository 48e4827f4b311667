"""Droplet diagnostics on the host, from the FP64 sums of ``dl_reduce`` or from
downloaded fields.

* :func:`deformation_from_moments` -- the 3-D deformation D of the droplet
  from the second-moment tensor of w = (phi - phi1)/(phi2 - phi1) = (1+phi~)/2:
  D = (sqrt(l_max) - sqrt(l_min)) / (sqrt(l_max) + sqrt(l_min)) with l the
  eigenvalues of the covariance of w.
* :func:`deformation_midplane` -- the reference's own measure, break_up3 of
  prototype_program/two-phase/drop8_mpi.f90:812-970: centroid and inertia
  tensor on the plane y = y_mid with weight phi - phi1, eigenvalues by the same
  cyclic Jacobi rotation (pivot = largest off-diagonal, stop when every
  off-diagonal is below 1e-6), L = 2 sqrt(I_3 / sum w), B = 2 sqrt(I_1 / sum w)
  taken from the unsorted diagonal, D = (L - B)/(L + B).
* :func:`laplace_pressure` -- p inside minus p outside the droplet.
"""
from __future__ import annotations

import math

import numpy as np


def _moments(d: dict):
    w = d["w_sum"]
    m = np.array(d["w_x"]) / w
    xx, yy, zz, xy, xz, yz = d["w_xx"]
    S = np.array([[xx, xy, xz], [xy, yy, yz], [xz, yz, zz]]) / w
    return w, m, S - np.outer(m, m)


def deformation_from_moments(d: dict) -> float:
    """D from the covariance of w (keys w_sum, w_x, w_xx of dl_reduce)."""
    _, _, C = _moments(d)
    lam = np.linalg.eigvalsh(C)
    a, b = math.sqrt(max(lam[-1], 0.0)), math.sqrt(max(lam[0], 0.0))
    return (a - b) / (a + b)


def centroid(d: dict):
    _, m, _ = _moments(d)
    return m


def deformation_midplane(phi: np.ndarray, phi1: float, y_mid: int | None = None) -> float:
    """break_up3 (drop8_mpi.f90:812-970) on phi with shape (nz, ny, nx)."""
    nz, ny, nx = phi.shape
    yi = ny // 2 if y_mid is None else int(y_mid)
    w = phi[:, yi, :] - phi1          # (nz, nx)
    X = np.arange(nx, dtype=np.float64)[None, :]
    Z = np.arange(nz, dtype=np.float64)[:, None]
    Y = float(yi)
    ws = w.sum()
    xg = (X * w).sum() / ws
    yg = Y
    zg = (Z * w).sum() / ws
    dx, dy, dz = X - xg, Y - yg, Z - zg
    xx = (w * dx * dx).sum()
    yy = (w * dy * dy).sum()
    zz = (w * dz * dz).sum()
    xy = (w * dx * dy).sum()
    yz = (w * dy * dz).sum()
    zx = (w * dz * dx).sum()
    A = np.array([[yy + zz, -xy, -zx], [-xy, xx + zz, -yz], [-zx, -yz, xx + yy]], dtype=np.float64)
    for _ in range(100):
        mx = abs(A[0, 1])
        p, q = 0, 1
        for j in range(1, 3):
            for i in range(0, j):
                if abs(A[i, j]) > mx:
                    mx = abs(A[i, j])
                    p, q = i, j
        if A[p, p] - A[q, q] == 0.0:
            theta = 0.25 * math.pi * (1.0 if A[p, q] >= 0 else -1.0)
        else:
            theta = 0.5 * math.atan(2.0 * A[p, q] / (A[p, p] - A[q, q]))
        W = np.eye(3)
        W[p, p] = math.cos(theta)
        W[p, q] = -math.sin(theta)
        W[q, p] = math.sin(theta)
        W[q, q] = math.cos(theta)
        A = W.T @ A @ W
        if all(abs(A[i, j]) < 1e-6 for j in range(3) for i in range(j + 1, 3)):
            break
    L = 2.0 * math.sqrt(max(A[2, 2], 0.0) / ws)
    B = 2.0 * math.sqrt(max(A[0, 0], 0.0) / ws)
    return (L - B) / (L + B)


def laplace_pressure(d: dict) -> float:
    """Mean p where w > 0.95 minus mean p where w < 0.05 (keys p_in, n_in, p_out, n_out)."""
    if d["n_in"] <= 0 or d["n_out"] <= 0:
        return float("nan")
    return d["p_in"] / d["n_in"] - d["p_out"] / d["n_out"]


def volume(d: dict) -> dict:
    """Droplet volume as a site count (phi above the mid value) and as sum w."""
    return {"count": d["vol_count"], "smooth": d["vol_smooth"]}
