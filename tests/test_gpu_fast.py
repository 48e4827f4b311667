"""GPU accuracy of the reduced-precision forms (FP32 arithmetic; FP32 or FP16
population storage) against the FP64 oracle, through the C-ABI.

Tolerances (stated per test) are in the presentation map
phi~ = 2 (phi - phi1)/(phi2 - phi1) - 1, i.e. relative to phi2 - phi1,
and absolute for u and p."""
import numpy as np
import pytest

from droplet_gb300 import Params, init_fields, configs
from droplet_gb300 import _abi
from droplet_gb300.solver import Droplet, FORM_FP64, FORM_FP32, FORM_FP16
from oracle import pyoracle

pytestmark = pytest.mark.gpu

FIELDS = ("phi", "u1", "u2", "u3", "p")


def make_case(case, shape, seed=11):
    nx, ny, nz = shape
    P = Params.lbm_drop_xy().replace(tauf=0.8, nu1=0.1, nu2=0.1, kappag=2e-3)
    rng = np.random.default_rng(seed)
    phi = init_fields.tanh_droplets(shape, P, [(nx / 2 - 0.3, ny / 2 + 0.2, nz / 2)], [min(shape) / 4], width=1.5)
    u = [0.01 * rng.standard_normal((nz, ny, nx)) for _ in range(3)]
    f = init_fields.fields(phi, *u)
    force = None
    mode = _abi.DL_FORCE_NONE
    if case == "walls":
        P = P.replace(walls=True, wall_u=(0.03, 0.01, 0.0), wall_start=4)
    elif case == "les_static_force":
        P = P.replace(les=True, Cs=0.17, delta=1.0)
        force = [1e-4 * np.sin(np.arange(nx) * 0.7)[None, None, :] * np.ones((nz, ny, nx)),
                 1e-4 * np.cos(np.arange(ny) * 0.4)[None, :, None] * np.ones((nz, ny, nx)),
                 np.full((nz, ny, nx), -2e-5)]
        mode = _abi.DL_FORCE_STATIC
    elif case == "spectral_les":
        P = P.replace(les=True, Cs=0.1, delta=1.0, eps=1e-6, kc=3)
        mode = _abi.DL_FORCE_SPECTRAL
    elif case == "spectral_kc4":
        # more band modes than the in-kernel synthesis holds: separate launches
        P = P.replace(eps=1e-6, kc=4)
        mode = _abi.DL_FORCE_SPECTRAL
    elif case == "eta":
        P = P.replace(nu2=0.05)
    return P, f, mode, force


def start(sim, f, mode, force):
    sim.set_fields(**f)
    sim.init_equilibrium()
    if mode == _abi.DL_FORCE_STATIC:
        sim.set_force(mode, *force)
    else:
        sim.set_force(mode)


def errors(P, a, b):
    span = P.phi2 - P.phi1
    return {
        "phi": np.abs(a["phi"] - b["phi"]).max() / span,
        "u": max(np.abs(a[k] - b[k]).max() for k in ("u1", "u2", "u3")),
        "p": np.abs(a["p"] - b["p"]).max(),
    }


@pytest.mark.parametrize("form,tol_phi,tol_u", [(FORM_FP32, 2e-5, 2e-6), (FORM_FP16, 1e-3, 1e-4)])
@pytest.mark.parametrize("case", ["plain", "walls", "les_static_force", "spectral_les", "spectral_kc4", "eta"])
def test_fast_form_tracks_oracle(form, tol_phi, tol_u, case):
    """30 steps on a ragged 40 x 20 x 16 grid (x not a multiple of the 32-wide
    tile); tolerances: FP32 2e-5 in phi~, 2e-6 in u; FP16 storage 1e-3, 1e-4."""
    shape = (40, 20, 16)
    P, f, mode, force = make_case(case, shape)
    g = Droplet(P, shape, form)
    o = pyoracle.OracleDroplet(P, shape)
    start(g, f, mode, force)
    start(o, f, mode, force)
    g.step(30)
    o.step(30)
    e = errors(P, g.get_fields(), o.get_fields())
    assert e["phi"] <= tol_phi, e
    assert e["u"] <= tol_u, e
    assert e["p"] <= tol_u, e
    assert g.step_count == 30


@pytest.mark.parametrize("form", [FORM_FP32, FORM_FP16])
def test_init_equilibrium_populations_match_oracle(form):
    shape = (32, 16, 12)
    P, f, mode, force = make_case("plain", shape)
    g = Droplet(P, shape, form)
    o = pyoracle.OracleDroplet(P, shape)
    start(g, f, mode, force)
    start(o, f, mode, force)
    fg, gg = g.get_populations()
    fo, go = o.get_populations()
    tol = 1e-6 if form == FORM_FP32 else 2e-4
    assert np.abs(fg - fo).max() <= tol
    assert np.abs(gg - go).max() <= tol


@pytest.mark.parametrize("form", [FORM_FP32, FORM_FP16])
def test_populations_roundtrip(form):
    shape = (32, 16, 12)
    P, f, mode, force = make_case("walls", shape)
    o = pyoracle.OracleDroplet(P, shape)
    start(o, f, mode, force)
    o.step(3)
    fo, go = o.get_populations()
    g = Droplet(P, shape, form)
    g.set_populations(fo, go)
    fg, gg = g.get_populations()
    tol = 1e-6 if form == FORM_FP32 else 2e-4
    assert np.abs(fg - fo).max() <= tol and np.abs(gg - go).max() <= tol
    e = errors(P, g.get_fields(), o.get_fields())
    assert e["phi"] <= 1e-6 and e["u"] <= 1e-6 and e["p"] <= 1e-6, e


@pytest.mark.parametrize("form", [FORM_FP32, FORM_FP16])
def test_fast_form_conserves_phi(form):
    """sum phi drifts only by rounding: relative 1e-6 (FP32) / 1e-4 (FP16) after 200 steps."""
    shape = (32, 32, 32)
    P, f, mode, force = make_case("plain", shape)
    g = Droplet(P, shape, form)
    start(g, f, mode, force)
    s0 = g.reduce()["phi_sum"]
    g.step(200)
    d = g.reduce()
    assert d["nan_flag"] == 0
    tol = 1e-6 if form == FORM_FP32 else 1e-4
    assert abs(d["phi_sum"] - s0) / s0 <= tol


def test_fp32_shear_droplet_64cube_500_steps_against_fp64():
    """The shear workload (walls +-0.05, 64^3) in FP32 against the plain FP64
    form on the GPU (itself bitwise equal to the oracle): phi~ within 1e-4,
    u within 1e-5 after 500 steps."""
    w = configs.config1()
    out = {}
    for form in (FORM_FP64, FORM_FP32):
        g = Droplet(w.params, w.shape, form)
        start(g, w.fields, w.force_mode, None)
        g.step(500)
        out[form] = g.get_fields()
    e = errors(w.params, out[FORM_FP32], out[FORM_FP64])
    assert e["phi"] <= 1e-4 and e["u"] <= 1e-5, e


def test_fast_form_profile_counts_launches():
    shape = (32, 16, 16)
    P, f, mode, force = make_case("plain", shape)
    g = Droplet(P, shape, FORM_FP32)
    start(g, f, mode, force)
    g.profile(True)
    g.step(7)
    s = g.profile_read()
    assert s["main_launches"] == 7 and s["launches"] == 7 and s["main_ms"] > 0
    g.profile(True, every=3)  # launches 0, 3, 6 timed, all counted
    g.step(7)
    s = g.profile_read()
    assert s["main_launches"] == 3 and s["timed_launches"] == 3 and s["launches"] == 7 and s["main_ms"] > 0


@pytest.mark.parametrize("form", [FORM_FP64, FORM_FP32])
def test_minmax_async_equals_minmax(form):
    """dl_get_minmax_async copies into pinned memory the same two values that
    dl_get_minmax returns once the stream has passed the copy."""
    import torch

    shape = (24, 20, 16)
    P, f, mode, force = make_case("plain", shape)
    g = Droplet(P, shape, form)
    start(g, f, mode, force)
    buf = torch.zeros(2, dtype=torch.float64).pin_memory()
    for _ in range(3):
        g.step(1)
        g.minmax_async(buf.data_ptr())
        g.sync()
        assert (float(buf[0]), float(buf[1])) == g.minmax()


@pytest.mark.parametrize("form,tol_phi,tol_u", [(FORM_FP32, 1e-5, 1e-7), (FORM_FP16, 5e-4, 5e-6)])
@pytest.mark.parametrize("shape,lz", [((32, 32, 32), 0), ((40, 20, 22), 8)])
def test_projection_in_step_equals_own_launch(form, tol_phi, tol_u, shape, lz):
    """The band projection of the new u done by each block of the fused step
    after its march gives the run of the projection's own launch, up to the FP32
    summation order (odd sizes: partial tiles in x and y, a partial z chunk).
    Tolerances: half of the form's tolerance against the oracle."""
    P, f, mode, force = make_case("spectral_les", shape)
    out = {}
    for proj in (0, 1):
        g = Droplet(P, shape, form)
        g.set_option("push", 0)  # the projection options are the pull form's
        g.set_option("projection", proj)
        if lz:
            g.set_option("lz", lz)
        start(g, f, mode, force)
        g.step(40)
        out[proj] = g.get_fields()
    e = errors(P, out[1], out[0])
    assert e["phi"] <= tol_phi and e["u"] <= tol_u and e["p"] <= tol_u, e


@pytest.mark.parametrize("form,push", [(FORM_FP64, 0), (FORM_FP32, 0), (FORM_FP32, 1), (FORM_FP16, 0)])
def test_minmax_mirror_holds_every_step(form, push):
    """dl_set_minmax_mirror: the step that takes the counter to n writes the
    phi range of step n into slot n % nslots of the pinned mirror (the push
    form: the range of step n-1, the state it loaded, into slot n-1), the
    values that dl_get_minmax returns for that state; off again, the steps
    write nothing; memory that is not page-locked is refused on the host."""
    import torch

    from droplet_gb300 import DropletError

    shape = (24, 20, 16)
    P, f, mode, force = make_case("plain", shape)
    g = Droplet(P, shape, form)
    if form == FORM_FP32:
        g.set_option("push", push)
    start(g, f, mode, force)
    buf = torch.full((4, 2), -1.0, dtype=torch.float64).pin_memory()
    g.set_minmax_mirror(buf.data_ptr(), 4)
    for n in range(1, 10):
        before = g.minmax()  # the range of step n-1 (settles a push step's state)
        g.step(1)
        g.sync()
        if push:
            # (before the first step the range is init's (phi1, phi2), not a computed one)
            if n > 1:
                assert (float(buf[(n - 1) % 4, 0]), float(buf[(n - 1) % 4, 1])) == before, n
        else:
            assert (float(buf[n % 4, 0]), float(buf[n % 4, 1])) == g.minmax(), n
    with pytest.raises(DropletError):
        g.set_minmax_mirror(buf.data_ptr(), 3)  # not a power of two
    g.set_minmax_mirror(0)
    before = buf.clone()
    g.step(2)
    g.sync()
    assert torch.equal(buf, before)
    pageable = np.zeros(4)
    with pytest.raises(DropletError):
        g.set_minmax_mirror(pageable.ctypes.data, 2)
