"""CPU pins of the energy-diagnostics checker (oracle/np_energy.py): a single
Fourier mode lands in its shell, and the bins add up to the Parseval energy
(plus the reference's double count of the k3 = nz/2 plane for even nz)."""
import numpy as np

from droplet_gb300 import Params, init_fields
from oracle import np_energy


def test_single_mode_in_its_shell():
    nz, ny, nx = 8, 10, 12
    x = np.arange(nx)[None, None, :] * np.ones((nz, ny, nx))
    u1 = np.cos(2 * np.pi * 3 * x / nx)
    z = np.zeros_like(u1)
    E = np_energy.spectrum(u1, z, z, nx // 2 + 1)
    assert abs(E[3] - 0.25) < 1e-14 and abs(E.sum() - E[3]) < 1e-14


def test_bins_sum_to_parseval_odd_nz():
    rng = np.random.default_rng(1)
    u = [rng.standard_normal((9, 8, 10)) for _ in range(3)]
    E = np_energy.spectrum(*u, 64)
    assert np.isclose(E.sum(), 0.5 * np.mean(u[0] ** 2 + u[1] ** 2 + u[2] ** 2), rtol=1e-12)


def test_even_nz_counts_the_nyquist_plane_twice():
    rng = np.random.default_rng(2)
    u = [rng.standard_normal((8, 6, 10)) for _ in range(3)]
    E = np_energy.spectrum(*u, 64)
    N = u[0].size
    nyq = sum(np.abs(np.fft.fftn(v)[4]) ** 2 for v in u).sum() / N ** 2 * 0.5
    assert np.isclose(E.sum(), 0.5 * np.mean(u[0] ** 2 + u[1] ** 2 + u[2] ** 2) + nyq, rtol=1e-12)


def test_free_energy_of_uniform_phase():
    P = Params.lbm_drop_xy()
    phi = np.full((4, 5, 6), P.phi2)
    psi, mu, gsq = np_energy.free_energy_sums(P, phi)
    lg = np.log(P.phi2 / (1 - P.b * P.phi2))
    assert np.isclose(psi, 120 * (P.phi2 * P.T * lg - P.a * P.phi2 ** 2))
    assert np.isclose(mu, 120 * (P.T * lg + P.T / (1 - P.b * P.phi2) - 2 * P.a * P.phi2))
    assert gsq == 0.0
