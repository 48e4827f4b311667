"""Small and odd domain sizes (x below and above one 32-wide tile, y not a
multiple of the 8-row tile, z shorter than a block's z range) through every
form: FP64 bit for bit against the oracle, FP32 / FP16 within the stated
tolerances (phi~ and u), and the populations round-tripped through the host."""
import numpy as np
import pytest

from droplet_gb300 import DropletError, Params, init_fields
from droplet_gb300 import _abi
from droplet_gb300.solver import Droplet, FORM_FP16, FORM_FP32, FORM_FP64
from oracle import pyoracle

pytestmark = pytest.mark.gpu

SHAPES = [(7, 5, 3), (33, 9, 5), (3, 17, 4), (64, 3, 3)]
TOL = {FORM_FP32: (2e-5, 2e-6), FORM_FP16: (1e-3, 1e-4)}


def case(shape, les, spectral):
    nx, ny, nz = shape
    P = Params.lbm_drop_xy().replace(tauf=0.8, nu1=0.1, nu2=0.1, kappag=2e-3)
    if les:
        P = P.replace(les=True, Cs=0.1, delta=1.0)
    if spectral:
        P = P.replace(eps=1e-6, kc=2)
    rng = np.random.default_rng(nx * 100 + ny * 10 + nz)
    phi = init_fields.tanh_droplets(shape, P, [(nx / 2, ny / 2, nz / 2)], [max(1.2, min(shape) / 3)], width=1.0)
    f = init_fields.fields(phi, *[0.01 * rng.standard_normal(phi.shape) for _ in range(3)])
    return P, f


def run(sim, f, spectral, steps):
    sim.set_fields(**f)
    sim.init_equilibrium()
    sim.set_force(_abi.DL_FORCE_SPECTRAL if spectral else _abi.DL_FORCE_NONE)
    sim.step(steps)
    return sim.get_fields()


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("les,spectral", [(False, False), (True, False), (True, True)])
@pytest.mark.parametrize("form", [FORM_FP64, FORM_FP32, FORM_FP16])
def test_odd_sizes_track_oracle(shape, les, spectral, form):
    if spectral and shape[2] < 4:
        pytest.skip("the kc = 2 band needs nz >= 4")
    P, f = case(shape, les, spectral)
    o = run(pyoracle.OracleDroplet(P, shape), f, spectral, 6)
    g = Droplet(P, shape, form)
    a = run(g, f, spectral, 6)
    span = P.phi2 - P.phi1
    if form == FORM_FP64:
        for k in ("phi", "u1", "u2", "u3", "p"):
            if spectral:
                assert np.abs(a[k] - o[k]).max() <= 1e-13 * max(1.0, np.abs(o[k]).max()), k
            else:
                assert np.array_equal(a[k], o[k]), k
    else:
        tphi, tu = TOL[form]
        assert 2 * np.abs(a["phi"] - o["phi"]).max() / span <= tphi
        assert max(np.abs(a[k] - o[k]).max() for k in ("u1", "u2", "u3")) <= tu
    # populations out and back in give the same next step
    fa, ga = g.get_populations()
    h = Droplet(P, shape, form)
    h.set_populations(fa, ga)
    h.set_force(_abi.DL_FORCE_SPECTRAL if spectral else _abi.DL_FORCE_NONE)
    h.step_count = g.step_count
    g.step(1)
    h.step(1)
    b, c = g.get_fields(), h.get_fields()
    for k in ("phi", "u1", "u2", "u3", "p"):
        assert np.abs(b[k] - c[k]).max() <= (1e-12 if form == FORM_FP64 else 2e-3 * max(1e-3, np.abs(b[k]).max())), k


def test_spectral_force_refused_on_a_domain_too_small_for_the_band():
    P, f = case((7, 5, 3), False, True)
    g = Droplet(P, (7, 5, 3), FORM_FP32)
    g.set_fields(**f)
    with pytest.raises(DropletError):
        g.set_force(_abi.DL_FORCE_SPECTRAL)
