"""Second, independent restatement of the reference step in vectorised NumPy.
TEST INFRASTRUCTURE ONLY.

It exists to pin the C oracle: both are written from the Fortran, in its
evaluation order (left-to-right, x**2 as x*x, the i = 1..15 accumulation
order, divisions kept), and NumPy's element-wise ufuncs never fuse a
multiply-add, so on small grids the two must agree bit for bit.

Sources: program/lbm_drop_xy.f90:421-666 (various_cal, gphi_cal,
equilibrium_cal, fg_cal, physics), program/LES_drop_xy.f90:481-502,655-690
(Smagorinsky tau_g), prototype_program/two-phase/drop8_mpi.f90:642-674
(moving-wall bounce-back of g).

Fields have shape (nz, ny, nx); populations (15, nz, ny, nx).
"""
from __future__ import annotations

import numpy as np

# program/lbm_drop_xy.f90:70-84
CX = (0, 1, 0, 0, -1, 0, 0, 1, -1, 1, 1, -1, 1, -1, -1)
CY = (0, 0, 1, 0, 0, -1, 0, 1, 1, -1, 1, -1, -1, 1, -1)
CZ = (0, 0, 0, 1, 0, 0, -1, 1, 1, 1, -1, -1, -1, -1, 1)
E = [2.0 / 9.0] + [1.0 / 9.0] * 6 + [1.0 / 72.0] * 8
H = [1.0] + [0.0] * 14
F = [-7.0 / 3.0] + [1.0 / 3.0] * 6 + [1.0 / 24.0] * 8
CR = [[float(CX[i]), float(CY[i]), float(CZ[i])] for i in range(15)]


def shifted(a, i, sign=+1):
    """a evaluated at x + sign*c_i with periodic wrap (the glue halo)."""
    return np.roll(a, shift=(-sign * CZ[i], -sign * CY[i], -sign * CX[i]), axis=(0, 1, 2))


class NumpyStep:
    def __init__(self, P, fields):
        self.P = P
        self.phi = fields["phi"].astype(np.float64).copy()
        self.u = [fields["u1"].astype(np.float64).copy(), fields["u2"].astype(np.float64).copy(),
                  fields["u3"].astype(np.float64).copy()]
        self.p = fields["p"].astype(np.float64).copy()
        self.force = [np.zeros_like(self.phi) for _ in range(3)]
        self.phi_min, self.phi_max = P.phi1, P.phi2
        self.n = 0
        self.f = None
        self.g = None

    # various_cal, :590-640
    def various(self):
        P, phi = self.P, self.phi
        p0 = phi * P.T / (1.0 - P.b * phi) - P.a * (phi * phi)
        lap = -(14.0 * phi)
        for i in range(1, 15):
            lap = lap + shifted(phi, i)
        lap = lap / (5.0 * (P.ds * P.ds))
        grad = []
        gu = [[None] * 3 for _ in range(3)]  # gu[a][al] = d u_a / d x_al
        for al in range(3):
            s = np.zeros_like(phi)
            t = [np.zeros_like(phi) for _ in range(3)]
            for i in range(1, 15):
                s = s + CR[i][al] * shifted(phi, i)
                for c in range(3):
                    t[c] = t[c] + CR[i][al] * shifted(self.u[c], i)
            grad.append(s / (10.0 * P.ds))
            for c in range(3):
                gu[c][al] = t[c] / (10.0 * P.ds)
        return p0, lap, grad, gu

    # gphi_cal, :642-666
    @staticmethod
    def gphi(grad):
        gsq = (grad[0] * grad[0] + grad[1] * grad[1]) + grad[2] * grad[2]
        G = [[None] * 3 for _ in range(3)]  # G[al][be]
        for be in range(3):
            for al in range(3):
                kr = 1.0 if al == be else 0.0
                G[al][be] = 4.5 * grad[al] * grad[be] - 1.5 * gsq * kr
        return G

    def taug(self, gu):
        P = self.P
        if P.visc_mode == 1:
            mn, mx = P.phi1, P.phi2
        else:
            mn, mx = self.phi_min, self.phi_max
        nu = (self.phi - mn) / (mx - mn) * (P.nu2 - P.nu1) + P.nu1
        nue = np.zeros_like(self.phi)
        if P.les:
            acc = np.zeros_like(self.phi)
            for be in range(3):
                for al in range(3):
                    st = 0.5 * (gu[al][be] + gu[be][al])
                    acc = acc + st * st
            nue = P.Cs * P.Cs * P.delta * P.delta * np.sqrt(2.0 * acc)
        return 0.5 + 3.0 * (nu + nue) / P.ds + (2.0 / 3.0) * P.Anu

    # equilibrium_cal, :421-476
    def equilibria(self, p0, lap, grad, gu, G):
        P = self.P
        u1, u2, u3 = self.u
        phi, p = self.phi, self.p
        feq, geq = [], []
        for i in range(15):
            cr = CR[i]
            ftemp = np.zeros_like(phi)
            gtemp = np.zeros_like(phi)
            for be in range(3):
                for al in range(3):
                    ftemp = ftemp + (gu[be][al] + gu[al][be]) * cr[al] * cr[be]
                    gtemp = gtemp + G[al][be] * cr[al] * cr[be]
            fe = (H[i] * phi
                  + F[i] * (p0 - P.kappaf * phi * lap
                            - P.kappaf / 6.0 * (grad[0] * grad[0] + grad[1] * grad[1] + grad[2] * grad[2]))
                  + E[i] * phi * 3.0 * (cr[0] * u1 + cr[1] * u2 + cr[2] * u3)
                  + E[i] * P.kappaf * gtemp)
            cu = u1 * cr[0] + u2 * cr[1] + u3 * cr[2]
            ge = (E[i] * (3.0 * p + 3.0 * cu + 4.5 * (cu * cu)
                          - 1.5 * (u1 * u1 + u2 * u2 + u3 * u3) + P.Anu * P.ds * ftemp)
                  + E[i] * P.kappag * gtemp)
            feq.append(fe)
            geq.append(ge)
        return feq, geq

    def init_equilibrium(self):
        p0, lap, grad, gu = self.various()
        self.f, self.g = self.equilibria(p0, lap, grad, gu, self.gphi(grad))
        self.phi_min, self.phi_max = self.P.phi1, self.P.phi2

    def step(self, nsteps=1):
        for _ in range(nsteps):
            self._step()

    def _step(self):
        P = self.P
        n = self.n + 1
        p0, lap, grad, gu = self.various()
        G = self.gphi(grad)
        tg = self.taug(gu)
        feq, geq = self.equilibria(p0, lap, grad, gu, G)
        fn, gn = [], []
        fx, fy, fz = self.force
        for i in range(15):
            fs, gs = shifted(self.f[i], i, -1), shifted(self.g[i], i, -1)
            fn.append(fs - (fs - shifted(feq[i], i, -1)) / P.tauf)
            gn.append(gs - (gs - shifted(geq[i], i, -1)) / shifted(tg, i, -1)
                      + 3.0 * P.ds * E[i] * (CR[i][0] * shifted(fx, i, -1) + CR[i][1] * shifted(fy, i, -1)
                                            + CR[i][2] * shifted(fz, i, -1)))
        if P.walls:
            U = list(P.wall_u) if n >= P.wall_start else [0.0, 0.0, 0.0]
            for i, j in ((3, 6), (7, 11), (8, 12), (9, 13), (14, 10)):
                gn[i][0] = gn[j][0] - 6.0 * E[j] * ((-U[0]) * CR[j][0] + (-U[1]) * CR[j][1] + (-U[2]) * CR[j][2])
            for i, j in ((6, 3), (10, 14), (11, 7), (12, 8), (13, 9)):
                gn[i][-1] = gn[j][-1] - 6.0 * E[j] * (U[0] * CR[j][0] + U[1] * CR[j][1] + U[2] * CR[j][2])
        self.f, self.g = fn, gn
        phi = np.zeros_like(self.phi)
        p = np.zeros_like(self.phi)
        u = [np.zeros_like(self.phi) for _ in range(3)]
        for i in range(15):
            phi = phi + fn[i]
            p = p + gn[i] / 3.0
            for c in range(3):
                u[c] = u[c] + CR[i][c] * gn[i]
        self.phi, self.p, self.u = phi, p, u
        mn, mx = P.phi2, P.phi1
        for v in phi.reshape(-1):
            if v > mx:
                mx = v
            elif v < mn:
                mn = v
        self.phi_min, self.phi_max = float(mn), float(mx)
        self.n = n

    def fields(self):
        return dict(phi=self.phi, u1=self.u[0], u2=self.u[1], u3=self.u[2], p=self.p)

    def populations(self):
        """f, g with shape (nz, ny, nx, 15) like the C-ABI."""
        return np.stack(self.f, axis=-1), np.stack(self.g, axis=-1)


class SinglePhaseStep:
    """The single-phase step of the precursor turbulence program
    program/lbm_iht_xy.f90: equilibrium_cal (:532-559), g_cal (:561-590) and
    physics (:592-654), in the reference's evaluation order. tau_g is
    1/2 + 3 (nu + nu_t)/ds with nu_t = 0 (the program's Cs = 0, :21-22)."""

    def __init__(self, nu, fields, ds=1.0):
        self.nu, self.ds = nu, ds
        self.u = [fields["u1"].astype(np.float64).copy(), fields["u2"].astype(np.float64).copy(),
                  fields["u3"].astype(np.float64).copy()]
        self.p = fields["p"].astype(np.float64).copy()
        self.force = [np.zeros_like(self.p) for _ in range(3)]
        self.g = None

    # equilibrium_cal, :532-559
    def equilibria(self):
        u1, u2, u3 = self.u
        p = self.p
        geq = []
        for i in range(15):
            cu = u1 * float(CX[i]) + u2 * float(CY[i]) + u3 * float(CZ[i])
            geq.append(E[i] * (3.0 * p + 3.0 * cu + 4.5 * (cu * cu) - 1.5 * (u1 * u1 + u2 * u2 + u3 * u3)))
        return geq

    # ini, :270
    def init_equilibrium(self):
        self.g = self.equilibria()

    def step(self, nsteps=1):
        for _ in range(nsteps):
            self._step()

    def _step(self):
        taug = 0.5 + 3.0 * (self.nu + 0.0) / self.ds  # physics :649
        geq = self.equilibria()
        fx, fy, fz = self.force
        gn = []
        # g_cal, :573-582
        for i in range(15):
            gs = shifted(self.g[i], i, -1)
            gn.append(gs - (gs - shifted(geq[i], i, -1)) / taug
                      + 3.0 * self.ds * E[i] * (float(CX[i]) * shifted(fx, i, -1) + float(CY[i]) * shifted(fy, i, -1)
                                                + float(CZ[i]) * shifted(fz, i, -1)))
        # physics, :613-625
        p = np.zeros_like(self.p)
        u = [np.zeros_like(self.p) for _ in range(3)]
        for i in range(15):
            p = p + gn[i] / 3.0
            u[0] = u[0] + float(CX[i]) * gn[i]
            u[1] = u[1] + float(CY[i]) * gn[i]
            u[2] = u[2] + float(CZ[i]) * gn[i]
        self.g, self.p, self.u = gn, p, u

    def fields(self):
        return dict(u1=self.u[0], u2=self.u[1], u3=self.u[2], p=self.p)

    def populations(self):
        return np.stack(self.g, axis=-1)
