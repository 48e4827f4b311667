"""Differentiable PyTorch restatement of the droplet step. TEST INFRASTRUCTURE ONLY.

Used as the "plain PyTorch autodiff reference" for the hand-written adjoint:
the same physics as the C oracle (program/lbm_drop_xy.f90:421-666 with the
moving-wall bounce-back of prototype_program/two-phase/drop8_mpi.f90:642-674
and, when P.les, the Smagorinsky tau_g of program/LES_drop_xy.f90:481-502,
663-690; a viscosity ratio in the fixed-range mode),
written with torch.roll so that autograd differentiates it, in FP64. It does
not follow the reference's evaluation order (it is not a parity restatement);
its job is gradients.

Fields have shape (nz, ny, nx); populations (15, nz, ny, nx).
"""
from __future__ import annotations

import torch

CX = (0, 1, 0, 0, -1, 0, 0, 1, -1, 1, 1, -1, 1, -1, -1)
CY = (0, 0, 1, 0, 0, -1, 0, 1, 1, -1, 1, -1, -1, 1, -1)
CZ = (0, 0, 0, 1, 0, 0, -1, 1, 1, 1, -1, -1, -1, -1, 1)
E = [2.0 / 9.0] + [1.0 / 9.0] * 6 + [1.0 / 72.0] * 8
H = [1.0] + [0.0] * 14
F = [-7.0 / 3.0] + [1.0 / 3.0] * 6 + [1.0 / 24.0] * 8
BOT = ((3, 6), (7, 11), (8, 12), (9, 13), (14, 10))   # (incoming, source) at z = 0
TOP = ((6, 3), (10, 14), (11, 7), (12, 8), (13, 9))   # at z = nz - 1


def nb(a, i, sign=+1):
    """a at x + sign * c_i (periodic)."""
    return torch.roll(a, shifts=(-sign * CZ[i], -sign * CY[i], -sign * CX[i]), dims=(0, 1, 2))


def equilibria(P, phi, u, p, kf, kg):
    """feq_i, geq_i (lists of 15 fields) from phi, u = (u1, u2, u3), p."""
    lap = -14.0 * phi
    for i in range(1, 15):
        lap = lap + nb(phi, i)
    lap = lap / (5.0 * P.ds * P.ds)
    grad = []
    for al in range(3):
        s = torch.zeros_like(phi)
        for i in range(1, 15):
            c = (CX, CY, CZ)[al][i]
            if c:
                s = s + c * nb(phi, i)
        grad.append(s / (10.0 * P.ds))
    gsq = grad[0] ** 2 + grad[1] ** 2 + grad[2] ** 2
    p0 = phi * P.T / (1.0 - P.b * phi) - P.a * phi * phi
    A = p0 - kf * phi * lap - kf / 6.0 * gsq
    usq = u[0] ** 2 + u[1] ** 2 + u[2] ** 2
    feq, geq = [], []
    for i in range(15):
        c = (CX[i], CY[i], CZ[i])
        cu = c[0] * u[0] + c[1] * u[1] + c[2] * u[2]
        cg = c[0] * grad[0] + c[1] * grad[1] + c[2] * grad[2]
        cGc = 4.5 * cg * cg - 1.5 * (c[0] ** 2 + c[1] ** 2 + c[2] ** 2) * gsq
        feq.append(H[i] * phi + F[i] * A + 3.0 * E[i] * phi * cu + E[i] * kf * cGc)
        geq.append(E[i] * (3.0 * p + 3.0 * cu + 4.5 * cu * cu - 1.5 * usq) + E[i] * kg * cGc)
    return feq, geq


def moments(f, g):
    phi = sum(f)
    p = sum(g) / 3.0
    u = [sum(c[i] * g[i] for i in range(15) if c[i]) for c in (CX, CY, CZ)]
    return phi, u, p


def taug_field(P, phi, u, frozen_visc=False):
    """tau_g = 1/2 + 3 (nu(phi) + nu_t)/ds: nu(phi) = nu1 + (phi - phi1)(nu2 -
    nu1)/(phi2 - phi1) (the fixed-range mode, program/lbm_drop_xy.f90:254-285),
    nu_t the Smagorinsky term when P.les. frozen_visc: no gradient through
    nu(phi) (tests use it to show that its adjoint matters)."""
    ph = phi.detach() if frozen_visc else phi
    nu = P.nu1 + (ph - P.phi1) / (P.phi2 - P.phi1) * (P.nu2 - P.nu1)
    if P.les:
        nu = nu + (les_taug(P, u) - 0.5) * P.ds / 3.0 - P.nu1
    return 0.5 + 3.0 * nu / P.ds


def les_taug(P, u):
    """tau_g = 1/2 + 3 (nu1 + nu_t)/ds, nu_t = (Cs delta)^2 sqrt(2 S:S), S the
    symmetric part of d u_a / d x_b from the 14-neighbour stencil."""
    G = [[None] * 3 for _ in range(3)]
    for a in range(3):
        for b in range(3):
            s = torch.zeros_like(u[a])
            for i in range(1, 15):
                c = (CX, CY, CZ)[b][i]
                if c:
                    s = s + c * nb(u[a], i)
            G[a][b] = s / (10.0 * P.ds)
    acc = torch.zeros_like(u[0])
    for a in range(3):
        for b in range(3):
            acc = acc + (0.5 * (G[a][b] + G[b][a])) ** 2
    nut = (P.Cs * P.delta) ** 2 * torch.sqrt((2.0 * acc).clamp_min(1e-300))
    return 0.5 + 3.0 * (P.nu1 + nut) / P.ds


def band_force(P, u):
    """Constant-injection band forcing (program/lbm_drop_iht_xy.f90:722-842):
    u_hat = FFT(u)/N on the band 1 <= |k|^2 < kc^2, E = sum 0.5 |u_hat|^2 over
    the band (the full spectrum, which the reference's half spectrum with
    weights min(2, k3+1) equals), F = (0.5 eps / E) times the band-passed u."""
    nz, ny, nx = u[0].shape
    N = nx * ny * nz
    kz = torch.fft.fftfreq(nz, d=1.0 / nz).view(nz, 1, 1)
    ky = torch.fft.fftfreq(ny, d=1.0 / ny).view(1, ny, 1)
    kx = torch.fft.fftfreq(nx, d=1.0 / nx).view(1, 1, nx)
    kk = kx * kx + ky * ky + kz * kz
    mask = ((kk >= 1) & (kk < P.kc * P.kc)).to(torch.float64)
    uh = [torch.fft.fftn(c) / N * mask for c in u]
    E = 0.5 * sum((h.real ** 2 + h.imag ** 2).sum() for h in uh)
    coef = 0.5 * P.eps / E
    return [coef * torch.fft.ifftn(h).real * N for h in uh]


def step(P, f, g, kf, kg, tauf, U, taug, spectral=False, frozen_visc=False):
    """One time step at viscosity ratio 1: tau_g constant, or from the
    Smagorinsky strain when P.les; with spectral, the band force of the
    step's u at the source. U: top-wall x velocity (tensor); the bottom wall
    moves with -U. spectral="frozen" applies the force with no gradient
    through it (tests use it to show that its adjoint matters)."""
    phi, u, p = moments(f, g)
    feq, geq = equilibria(P, phi, u, p, kf, kg)
    if P.les or P.nu2 != P.nu1:
        taug = taug_field(P, phi, u, frozen_visc)
    fn = [nb(f[i] - (f[i] - feq[i]) / tauf, i, -1) for i in range(15)]
    if spectral:
        F = band_force(P, u)
        if spectral == "frozen":
            F = [c.detach() for c in F]
        gn = [nb(g[i] - (g[i] - geq[i]) / taug + 3.0 * P.ds * E[i] * (CX[i] * F[0] + CY[i] * F[1] + CZ[i] * F[2]),
                 i, -1) for i in range(15)]
    else:
        gn = [nb(g[i] - (g[i] - geq[i]) / taug, i, -1) for i in range(15)]
    if P.walls:
        Uv = (U, 0.0, 0.0)
        gb = list(gn)
        for i, j in BOT:
            w = 6.0 * E[j] * ((-Uv[0]) * CX[j] + (-Uv[1]) * CY[j] + (-Uv[2]) * CZ[j])
            gb[i] = torch.cat([(gn[j][:1] - w), gn[i][1:]], dim=0)
        for i, j in TOP:
            w = 6.0 * E[j] * (Uv[0] * CX[j] + Uv[1] * CY[j] + Uv[2] * CZ[j])
            gb[i] = torch.cat([gn[i][:-1], (gn[j][-1:] - w)], dim=0)
        gn = gb
    return fn, gn


def deformation(P, phi):
    """D from the covariance of w = (phi - phi1)/(phi2 - phi1)."""
    nz, ny, nx = phi.shape
    w = (phi - P.phi1) / (P.phi2 - P.phi1)
    z, y, x = torch.meshgrid(torch.arange(nz, dtype=phi.dtype), torch.arange(ny, dtype=phi.dtype),
                             torch.arange(nx, dtype=phi.dtype), indexing="ij")
    X = torch.stack([x, y, z]).reshape(3, -1)
    wf = w.reshape(-1)
    W = wf.sum()
    m = (X * wf).sum(dim=1) / W
    S = (X * wf) @ X.T / W
    C = S - torch.outer(m, m)
    lam = torch.linalg.eigvalsh(C)
    a, b = torch.sqrt(lam[-1]), torch.sqrt(lam[0])
    return (a - b) / (a + b)


def run_loss(P, phi0, u0, p0, kf, kg, tauf, U, taug, nsteps, spectral=False, frozen_visc=False):
    """Initialise at equilibrium from (phi0, u0, p0) and return D after nsteps."""
    feq, geq = equilibria(P, phi0, u0, p0, kf, kg)
    f, g = feq, geq
    for _ in range(nsteps):
        f, g = step(P, f, g, kf, kg, tauf, U, taug, spectral, frozen_visc)
    phi, _, _ = moments(f, g)
    return deformation(P, phi)
