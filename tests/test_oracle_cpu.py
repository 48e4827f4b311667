"""CPU tests of the oracle (no GPU): the C restatement against an independent
NumPy restatement (bitwise), against an FFT evaluation of the forcing, and
against physical known answers. The reference ships no tests or golden
vectors, so these pins replace them."""
import ctypes as C

import numpy as np
import pytest

from droplet_gb300 import Params, init_fields
from droplet_gb300 import _abi
from oracle import np_oracle, pyoracle


def small_case(shape=(10, 9, 8), seed=0, **kw):
    """A droplet plus a smooth random velocity; cheap enough for NumPy."""
    base = dict(tauf=0.8, nu1=0.1, nu2=0.1, kappag=2e-3)
    base.update(kw)
    P = Params.lbm_drop_xy().replace(**base)
    nx, ny, nz = shape
    phi = init_fields.tanh_droplets(shape, P, [(nx / 2 - 0.3, ny / 2 + 0.2, nz / 2)], [2.5], width=1.5)
    rng = np.random.default_rng(seed)
    u = [0.01 * rng.standard_normal((nz, ny, nx)) for _ in range(3)]
    f = init_fields.fields(phi, *u)
    f["p"] = f["p"] + 1e-3 * rng.standard_normal((nz, ny, nx))
    return P, f


def run_both(P, f, shape, nsteps, force=None):
    o = pyoracle.OracleDroplet(P, shape)
    o.set_fields(**f)
    o.init_equilibrium()
    n = np_oracle.NumpyStep(P, f)
    n.init_equilibrium()
    if force is not None:
        o.set_force(_abi.DL_FORCE_STATIC, *force)
        n.force = [np.asarray(a, dtype=np.float64) for a in force]
    o.step(nsteps)
    n.step(nsteps)
    return o, n


def test_abi_struct_sizes_match_header():
    lib = pyoracle.load()
    lib.orc_abi_sizes.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_int)]
    a, b = C.c_int(), C.c_int()
    assert lib.orc_abi_sizes(C.byref(a), C.byref(b)) == 0
    assert a.value == C.sizeof(_abi.DLParams)
    assert b.value == C.sizeof(_abi.DLDiag)


@pytest.mark.parametrize("case", ["plain", "walls", "les_force", "anu_minmax_eta"])
def test_c_oracle_equals_numpy_restatement_bitwise(case):
    shape = (10, 9, 8)
    nx, ny, nz = shape
    force = None
    if case == "plain":
        P, f = small_case(shape)
    elif case == "walls":
        P, f = small_case(shape, walls=True, wall_u=(0.03, 0.01, 0.0), wall_start=3)
    elif case == "les_force":
        P, f = small_case(shape, les=True, Cs=0.17, delta=1.0)
        force = [1e-4 * np.sin(np.arange(nx) * 0.7)[None, None, :] * np.ones((nz, ny, nx)),
                 1e-4 * np.cos(np.arange(ny) * 0.4)[None, :, None] * np.ones((nz, ny, nx)),
                 np.full((nz, ny, nx), -2e-5)]
    else:
        P, f = small_case(shape, Anu=0.05, nu2=0.2)
    o, n = run_both(P, f, shape, 6, force)
    fo = o.get_fields()
    fn = n.fields()
    for k in ("phi", "u1", "u2", "u3", "p"):
        assert np.array_equal(fo[k], fn[k]), k
    po, go = o.get_populations()
    pn, gn = n.populations()
    assert np.array_equal(po, pn)
    assert np.array_equal(go, gn)
    assert o.minmax() == (n.phi_min, n.phi_max)


def test_minmax_scan_quirk_first_site_minimum():
    """All phi above phi1 with the first site the smallest: the reference's
    if/else-if scan never counts that site for the minimum."""
    P = Params.lbm_drop_xy().replace(nu2=0.2, tauf=0.8)
    shape = (6, 5, 4)
    nx, ny, nz = shape
    rng = np.random.default_rng(3)
    phi = P.phi1 + 0.2 + 0.01 * rng.random((nz, ny, nx))
    phi.reshape(-1)[0] = P.phi1 + 0.1
    f = init_fields.fields(phi)
    o, n = run_both(P, f, shape, 1)
    assert o.minmax() == (n.phi_min, n.phi_max)


def test_phi_conserved_to_roundoff():
    shape = (16, 16, 16)
    P = Params.lbm_drop_xy().replace(tauf=1.0, nu1=0.1, nu2=0.1, kappag=1e-3)
    phi = init_fields.tanh_droplets(shape, P, [(7.5, 7.5, 7.5)], [5.0])
    f = init_fields.fields(phi, init_fields.couette_u(shape, 0.02))
    o = pyoracle.OracleDroplet(P, shape)
    o.set_fields(**f)
    o.init_equilibrium()
    s0 = o.get_fields()["phi"].sum()
    o.step(50)
    s1 = o.get_fields()["phi"].sum()
    assert abs(s1 - s0) / s0 < 1e-13


def _fft_force(u, kc, eps):
    """The forcing of program/lbm_drop_iht_xy.f90:722-842 with NumPy's FFT."""
    nz, ny, nx = u[0].shape
    N = nx * ny * nz
    uh = [np.fft.rfftn(c, axes=(2, 1, 0)) / N for c in u]  # halves axis 0 (z), shape (nz/2+1, ny, nx)
    kz = np.arange(nz // 2 + 1)[:, None, None]
    ky = np.fft.fftfreq(ny, 1.0 / ny)[None, :, None]
    kx = np.fft.fftfreq(nx, 1.0 / nx)[None, None, :]
    kk = kx * kx + ky * ky + kz * kz
    band = (kk >= 1) & (kk < kc * kc)
    w = np.minimum(2.0, kz + 1.0)
    E = np.sum(0.5 * (np.abs(uh[0]) ** 2 + np.abs(uh[1]) ** 2 + np.abs(uh[2]) ** 2) * w * band)
    coef = 0.5 * eps / E
    return [np.fft.irfftn(np.where(band, coef * c, 0.0), s=(nx, ny, nz), axes=(2, 1, 0)) * N for c in uh]


def test_spectral_force_equals_fft_evaluation():
    shape = (16, 12, 20)
    nx, ny, nz = shape
    P = Params.lbm_drop_xy().replace(eps=1e-6, kc=3)
    u = init_fields.random_solenoidal(shape, seed=5, kmin=1, kmax=4, urms=0.02)
    f = init_fields.fields(np.full((nz, ny, nx), P.phi1), *u)
    o = pyoracle.OracleDroplet(P, shape)
    o.set_fields(**f)
    got = o.compute_spectral_force()
    ref = _fft_force(u, P.kc, P.eps)
    scale = max(np.abs(r).max() for r in ref)
    for g, r in zip(got, ref):
        assert np.abs(g - r).max() <= 1e-12 * scale


def test_spectral_force_injects_eps():
    """sum F.u / N = eps by construction (the constant-injection property)."""
    shape = (16, 16, 16)
    P = Params.lbm_drop_xy().replace(eps=3e-6, kc=3)
    u = init_fields.random_solenoidal(shape, seed=1, kmin=1, kmax=5, urms=0.02)
    o = pyoracle.OracleDroplet(P, shape)
    o.set_fields(**init_fields.fields(np.full(u[0].shape, P.phi1), *u))
    F = o.compute_spectral_force()
    power = sum((a * b).sum() for a, b in zip(F, u)) / u[0].size
    assert abs(power - P.eps) / P.eps < 1e-10


def test_uniform_phi_minmax_mode_matches_restatement():
    """With a uniform phi the reference's min/max range can collapse to one
    value, making nu = 0/0 * (nu2-nu1) + nu1 NaN; whether it does depends on
    the sign of the round-off in sum f. Both restatements must agree,
    NaNs included."""
    shape = (6, 6, 6)
    P = Params.lbm_drop_xy().replace(tauf=0.8)
    f = init_fields.fields(np.full((6, 6, 6), P.phi1))
    o, n = run_both(P, f, shape, 3)
    fo, fn = o.get_fields(), n.fields()
    for k in ("phi", "u1", "u2", "u3", "p"):
        assert np.array_equal(fo[k], fn[k], equal_nan=True), k


def test_couette_profile_is_linear():
    """Moving walls +-U with no droplet: steady linear u_x(z)."""
    shape = (4, 4, 16)
    nz = 16
    U = 0.02
    P = Params.lbm_drop_xy().replace(tauf=0.8, nu1=0.1, nu2=0.1, visc_mode=_abi.DL_VISC_FIXED, walls=True,
                                     wall_u=(U, 0.0, 0.0), wall_start=1)
    o = pyoracle.OracleDroplet(P, shape)
    o.set_fields(**init_fields.fields(np.full((nz, 4, 4), P.phi1)))
    o.init_equilibrium()
    o.step(4000)
    ux = o.get_fields()["u1"][:, 0, 0]
    z = np.arange(nz)
    a, b = np.polyfit(z, ux, 1)
    resid = ux - (a * z + b)
    assert np.abs(resid).max() < 1e-3 * U
    assert abs(ux[0] + ux[-1]) < 1e-6 * U  # antisymmetric
    assert 0.8 * U < ux[-1] <= 1.05 * U


def test_taylor_green_decay_rate():
    """Shear wave u_x = U sin(2 pi y / L) decays as exp(-nu k^2 t)."""
    L = 32
    shape = (4, L, 4)
    nu = 0.1
    P = Params.lbm_drop_xy().replace(tauf=0.8, nu1=nu, nu2=nu, visc_mode=_abi.DL_VISC_FIXED)
    k = 2 * np.pi / L
    y = np.arange(L)
    U = 1e-3
    u1 = np.broadcast_to((U * np.sin(k * y))[None, :, None], (4, L, 4)).copy()
    o = pyoracle.OracleDroplet(P, shape)
    o.set_fields(**init_fields.fields(np.full((4, L, 4), P.phi1), u1))
    o.init_equilibrium()
    t = 300
    o.step(t)
    a = o.get_fields()["u1"][0, :, 0]
    amp = np.sum(a * np.sin(k * y)) / np.sum(np.sin(k * y) ** 2)
    expect = U * np.exp(-nu * k * k * t)
    assert abs(amp / expect - 1.0) < 0.02


def single_phase_params(**kw):
    """The two-phase parameters that reduce the g update to the precursor's
    single-phase step: no interface terms, one viscosity, fixed range."""
    base = dict(kappaf=0.0, kappag=0.0, nu1=0.02, nu2=0.02, Anu=0.0, visc_mode=_abi.DL_VISC_FIXED)
    base.update(kw)
    return Params.lbm_drop_xy().replace(**base)


@pytest.mark.parametrize("forced", [False, True])
def test_single_phase_restatement_equals_c_oracle_g_update(forced):
    """program/lbm_iht_xy.f90's g-only step (NumPy restatement) equals the C
    oracle's g update with kappaf = kappag = Anu = 0 and nu2 = nu1, bit for
    bit: p, u and g."""
    shape = (10, 9, 8)
    nx, ny, nz = shape
    P = single_phase_params()
    rng = np.random.default_rng(5)
    u = [0.02 * rng.standard_normal((nz, ny, nx)) for _ in range(3)]
    f = init_fields.fields(np.full((nz, ny, nx), P.phi1), *u)
    f["p"] = f["p"] + 1e-3 * rng.standard_normal((nz, ny, nx))
    force = None
    if forced:
        force = [1e-4 * np.sin(np.arange(nx) * 0.7)[None, None, :] * np.ones((nz, ny, nx)),
                 np.full((nz, ny, nx), 3e-5),
                 1e-4 * np.cos(np.arange(nz) * 0.5)[:, None, None] * np.ones((nz, ny, nx))]
    o = pyoracle.OracleDroplet(P, shape)
    o.set_fields(**f)
    o.init_equilibrium()
    s = np_oracle.SinglePhaseStep(P.nu1, f, ds=P.ds)
    s.init_equilibrium()
    if force is not None:
        o.set_force(_abi.DL_FORCE_STATIC, *force)
        s.force = [np.asarray(a, dtype=np.float64) for a in force]
    o.step(7)
    s.step(7)
    fo, fs = o.get_fields(), s.fields()
    for k in ("u1", "u2", "u3", "p"):
        assert np.array_equal(fo[k], fs[k]), k
    assert np.array_equal(o.get_populations()[1], s.populations())


@pytest.mark.parametrize("forced", [False, True])
def test_c_single_phase_mode_equals_numpy_restatement(forced):
    """The C oracle's own single-phase mode (the CPU baseline of the precursor
    workload) against the NumPy restatement of program/lbm_iht_xy.f90."""
    shape = (10, 9, 8)
    nx, ny, nz = shape
    P = single_phase_params(eps=1e-6, kc=3)
    rng = np.random.default_rng(9)
    u = [0.02 * rng.standard_normal((nz, ny, nx)) for _ in range(3)]
    f = init_fields.fields(np.full((nz, ny, nx), P.phi1), *u)
    o = pyoracle.OracleDroplet(P, shape, single_phase=True)
    o.set_fields(**f)
    o.init_equilibrium()
    s = np_oracle.SinglePhaseStep(P.nu1, f, ds=P.ds)
    s.init_equilibrium()
    if forced:
        force = [1e-4 * np.sin(np.arange(nx) * 0.7)[None, None, :] * np.ones((nz, ny, nx)),
                 np.full((nz, ny, nx), 3e-5),
                 1e-4 * np.cos(np.arange(nz) * 0.5)[:, None, None] * np.ones((nz, ny, nx))]
        o.set_force(_abi.DL_FORCE_STATIC, *force)
        s.force = force
    o.step(5)
    s.step(5)
    fo, fs = o.get_fields(), s.fields()
    for k in ("u1", "u2", "u3", "p"):
        assert np.array_equal(fo[k], fs[k]), k
    assert np.array_equal(o.get_populations()[1], s.populations())
