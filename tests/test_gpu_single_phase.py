"""The single-phase step (DL_SINGLE_PHASE: the g-only precursor step of
program/lbm_iht_xy.f90) on the GPU against the C oracle run with the
parameters that reduce its g update to that step (kappaf = kappag = Anu = 0,
nu2 = nu1, fixed viscosity range): bit for bit in the FP64 form, within
stated tolerances in the FP32 and FP16 forms."""
import numpy as np
import pytest

from droplet_gb300 import DropletError, Params, init_fields
from droplet_gb300 import _abi
from droplet_gb300.solver import Droplet, FORM_FP16, FORM_FP32, FORM_FP64
from oracle import pyoracle

pytestmark = pytest.mark.gpu

U_FIELDS = ("u1", "u2", "u3", "p")


def case(kind, shape, seed=3):
    nx, ny, nz = shape
    P = Params.lbm_drop_xy().replace(kappaf=0.0, kappag=0.0, nu1=0.02, nu2=0.02, Anu=0.0,
                                     visc_mode=_abi.DL_VISC_FIXED)
    rng = np.random.default_rng(seed)
    u = [0.02 * rng.standard_normal((nz, ny, nx)) for _ in range(3)]
    f = init_fields.fields(np.full((nz, ny, nx), P.phi1), *u)
    f["p"] = f["p"] + 1e-3 * rng.standard_normal((nz, ny, nx))
    mode, force = _abi.DL_FORCE_NONE, None
    if kind == "static_force":
        mode = _abi.DL_FORCE_STATIC
        force = [1e-4 * np.sin(np.arange(nx) * 0.7)[None, None, :] * np.ones((nz, ny, nx)),
                 np.full((nz, ny, nx), 3e-5),
                 1e-4 * np.cos(np.arange(nz) * 0.5)[:, None, None] * np.ones((nz, ny, nx))]
    elif kind == "spectral":
        P = P.replace(eps=1e-6, kc=3)
        mode = _abi.DL_FORCE_SPECTRAL
    elif kind == "walls":
        P = P.replace(walls=True, wall_u=(0.03, 0.0, 0.0), wall_start=2)
    return P, f, mode, force


def start(sim, f, mode, force):
    sim.set_fields(**f)
    sim.init_equilibrium()
    if force is not None:
        sim.set_force(mode, *force)
    else:
        sim.set_force(mode)


def run(kind, form, shape, steps, pipeline=0):
    P, f, mode, force = case(kind, shape)
    g = Droplet(P, shape, form, single_phase=True)
    if form != FORM_FP64:
        g.set_option("pipeline", pipeline)
    o = pyoracle.OracleDroplet(P, shape)
    start(g, f, mode, force)
    start(o, f, mode, force)
    g.step(steps)
    o.step(steps)
    return P, g, o


@pytest.mark.parametrize("kind", ["plain", "static_force", "spectral", "walls"])
def test_fp64_single_phase_bitwise(kind):
    shape = (24, 20, 16)
    P, g, o = run(kind, FORM_FP64, shape, 12)
    a, b = g.get_fields(), o.get_fields()
    for k in U_FIELDS:
        if kind == "spectral":  # the band DFT sums in a different order on the device
            assert np.abs(a[k] - b[k]).max() <= 1e-13, k
        else:
            assert np.array_equal(a[k], b[k]), (k, np.abs(a[k] - b[k]).max())
    assert np.all(a["phi"] == P.phi1)
    if kind != "spectral":
        fa, ga = g.get_populations()
        assert np.array_equal(ga, o.get_populations()[1])
        assert not fa.any()


@pytest.mark.parametrize("pipeline", [0, 1])
@pytest.mark.parametrize("form,tol_u,tol_p", [(FORM_FP32, 2e-6, 2e-6), (FORM_FP16, 1e-4, 1e-4)])
@pytest.mark.parametrize("kind", ["plain", "static_force", "spectral", "walls"])
def test_fast_single_phase_tracks_oracle(form, tol_u, tol_p, kind, pipeline):
    """40 x 20 x 16 (x not a multiple of the 32-wide tile), 30 steps, both
    kernel variants; absolute tolerances on u and p."""
    shape = (40, 20, 16)
    P, g, o = run(kind, form, shape, 30, pipeline)
    a, b = g.get_fields(), o.get_fields()
    eu = max(np.abs(a[k] - b[k]).max() for k in ("u1", "u2", "u3"))
    ep = np.abs(a["p"] - b["p"]).max()
    assert eu <= tol_u and ep <= tol_p, (eu, ep)
    assert np.all(a["phi"] == P.phi1)


def test_single_phase_refusals():
    shape = (16, 16, 16)
    P, f, mode, force = case("plain", shape)
    with pytest.raises(DropletError):
        Droplet(P.replace(les=True, Cs=0.1, delta=1.0), shape, FORM_FP32, single_phase=True)
    g = Droplet(P, shape, FORM_FP32, single_phase=True)
    start(g, f, mode, force)
    with pytest.raises(DropletError):
        g.label_droplets()
    g.step(2)
    d = g.reduce()
    assert d["nan_flag"] == 0 and d["phi_min"] == d["phi_max"] == P.phi1
