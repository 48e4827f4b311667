"""The push form of the FP32 step (step_push.cu: each site collided by its own
thread, streamed by the store) against the oracle and against the pull form,
through the C-ABI, and the handle's settle of a push step's state.

A push launch takes the moments of the state it loads, so after it phi, u, p
are those of the step before, and the band force and wall reflection of its
streaming are completed by the next load; everything that reads the state
(fields, populations, diagnostics, the phi range) settles it first. The
tolerances are those of the FP32 form against the oracle: 2e-5 in
phi~ = 2 (phi - phi1)/(phi2 - phi1) - 1 and 2e-6 in u and p after 30 steps;
push against pull (both FP32, different order of evaluation): 1e-5 and 1e-6."""
import numpy as np
import pytest

from droplet_gb300 import configs
from droplet_gb300 import _abi
from droplet_gb300._lib import DropletError
from droplet_gb300.solver import Droplet, FORM_FP32
from oracle import pyoracle

from test_gpu_fast import errors, make_case, start

pytestmark = pytest.mark.gpu

CASES = ["plain", "walls", "les_static_force", "spectral_les"]


def run(P, f, mode, force, shape, steps, push, lz=0):
    g = Droplet(P, shape, FORM_FP32)
    g.set_option("push", push)
    if lz:
        g.set_option("lz", lz)
    start(g, f, mode, force)
    g.step(steps)
    return g


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("shape,lz", [((40, 20, 16), 0), ((33, 17, 19), 5), ((64, 24, 12), 12)])
def test_push_tracks_oracle_and_pull(case, shape, lz):
    P, f, mode, force = make_case(case, shape)
    o = pyoracle.OracleDroplet(P, shape)
    start(o, f, mode, force)
    o.step(30)
    ref = o.get_fields()
    g = run(P, f, mode, force, shape, 30, 1, lz)
    assert g.get_option("pushed") == 1
    a = g.get_fields()
    assert g.get_option("pushed") == 0 and g.step_count == 30
    e = errors(P, a, ref)
    assert e["phi"] <= 2e-5 and e["u"] <= 2e-6 and e["p"] <= 2e-6, e
    b = run(P, f, mode, force, shape, 30, 0, lz).get_fields()
    e2 = errors(P, a, b)
    assert e2["phi"] <= 1e-5 and e2["u"] <= 1e-6 and e2["p"] <= 1e-6, e2


@pytest.mark.parametrize("case", ["walls", "spectral_les"])
def test_push_populations_match_oracle(case):
    """get_populations of a push step's state (settled: the band force and the
    wall reflection of the last streaming included)."""
    shape = (32, 16, 12)
    P, f, mode, force = make_case(case, shape)
    o = pyoracle.OracleDroplet(P, shape)
    start(o, f, mode, force)
    o.step(7)
    g = run(P, f, mode, force, shape, 7, 1)
    fg, gg = g.get_populations()
    fo, go = o.get_populations()
    assert np.abs(fg - fo).max() <= 2e-6 and np.abs(gg - go).max() <= 2e-6


@pytest.mark.parametrize("case", ["walls", "spectral_les"])
def test_push_pull_settle_sequence(case):
    """push steps, a read (settle), push steps, pull steps, push steps: the run
    tracks the oracle as one sequence of 24 steps."""
    shape = (36, 18, 14)
    P, f, mode, force = make_case(case, shape)
    o = pyoracle.OracleDroplet(P, shape)
    start(o, f, mode, force)
    o.step(24)
    g = Droplet(P, shape, FORM_FP32)
    start(g, f, mode, force)
    g.step(5)
    g.reduce()
    g.step(6)
    g.set_option("push", 0)
    g.step(6)
    g.set_option("push", 1)
    g.step(7)
    e = errors(P, g.get_fields(), o.get_fields())
    assert e["phi"] <= 2e-5 and e["u"] <= 2e-6 and e["p"] <= 2e-6, e


def test_push_single_phase_spectral_tracks_oracle():
    """The precursor step (g only) with band forcing in the push form."""
    shape = (32, 24, 20)
    w = configs.precursor(n=32)
    P = w.params
    f = w.fields
    o = pyoracle.OracleDroplet(P, (32, 32, 32), single_phase=True)
    g = Droplet(P, (32, 32, 32), FORM_FP32, single_phase=True)
    for s in (o, g):
        s.set_fields(**f)
        s.init_equilibrium()
        s.set_force(_abi.DL_FORCE_SPECTRAL)
        s.step(25)
    a, b = g.get_fields(), o.get_fields()
    for k in ("u1", "u2", "u3", "p"):
        assert np.abs(a[k] - b[k]).max() <= 1e-7, k
    del shape


def test_push_is_the_fp32_default_and_falls_back():
    """FP32 steps in the push form by default; a viscosity ratio other than 1
    (tau_g from the phi range of the collided state) steps in the pull form."""
    shape = (24, 16, 12)
    P, f, mode, force = make_case("plain", shape)
    g = Droplet(P, shape, FORM_FP32)
    assert g.get_option("push") == 1
    start(g, f, mode, force)
    g.step(2)
    assert g.get_option("pushed") == 1
    P2, f2, mode2, force2 = make_case("eta", shape)
    h = Droplet(P2, shape, FORM_FP32)
    start(h, f2, mode2, force2)
    h.step(2)
    assert h.get_option("pushed") == 0


@pytest.mark.parametrize("case", CASES)
def test_staged_planes_equal_loaded_planes(case):
    """The populations of the next plane staged in shared memory by
    asynchronous copies (option "stage" = 1, the default) give the same bits
    as the same values loaded into registers (a partial tile in x and y)."""
    shape = (40, 20, 14)
    P, f, mode, force = make_case(case, shape)
    out = {}
    for stage in (0, 1):
        g = Droplet(P, shape, FORM_FP32)
        g.set_option("stage", stage)
        start(g, f, mode, force)
        g.step(9)
        out[stage] = (g.get_fields(), g.get_populations())
        g.sync()
    for k in out[0][0]:
        assert np.array_equal(out[0][0][k], out[1][0][k]), k
    assert np.array_equal(out[0][1][0], out[1][1][0]) and np.array_equal(out[0][1][1], out[1][1][1])


def test_push_bitwise_independent_of_z_chunks():
    """Without band forcing (no FP64 atomics in the step) the push form gives
    the same bits whatever the z chunk of a block: every site's loads,
    moments and collision are the same arithmetic in every block that takes
    them (the ring sites are computed again by each neighbouring block)."""
    shape = (40, 24, 30)
    P, f, mode, force = make_case("les_static_force", shape)
    out = []
    for lz in (4, 7, 30):
        g = run(P, f, mode, force, shape, 12, 1, lz)
        out.append(g.get_fields())
    for k in out[0]:
        assert np.array_equal(out[0][k], out[1][k]) and np.array_equal(out[0][k], out[2][k]), k


@pytest.mark.parametrize("case", CASES)
def test_tensor_staged_planes_equal_loaded_planes(case):
    """The next plane staged by two tensor (TMA) copies per block and plane,
    completing on an mbarrier (option "stage" = 2; full tiles), gives the same
    bits as the per-thread copies and as loads into registers."""
    shape = (64, 16, 14)
    P, f, mode, force = make_case(case, shape)
    out = {}
    for stage in (0, 1, 2):
        g = Droplet(P, shape, FORM_FP32)
        g.set_option("stage", stage)
        start(g, f, mode, force)
        g.step(9)
        out[stage] = (g.get_fields(), g.get_populations())
        g.sync()
    for stage in (1, 2):
        for k in out[0][0]:
            assert np.array_equal(out[0][0][k], out[stage][0][k]), (stage, k)
        for j in (0, 1):
            assert np.array_equal(out[0][1][j], out[stage][1][j]), (stage, j)


def test_tensor_staged_single_phase():
    """The precursor step (g only, band forcing) with its plane staged by one
    tensor copy per block and plane: the same bits as the per-thread copies."""
    w = configs.precursor(n=32)
    out = {}
    for stage in (1, 2):
        g = Droplet(w.params, (32, 32, 32), FORM_FP32, single_phase=True)
        g.set_option("stage", stage)
        g.set_fields(**w.fields)
        g.init_equilibrium()
        g.set_force(_abi.DL_FORCE_SPECTRAL)
        g.step(12)
        out[stage] = g.get_fields()
        g.sync()
    for k in out[1]:
        assert np.array_equal(out[1][k], out[2][k]), k


def test_tensor_stage_needs_full_tiles():
    P, f, mode, force = make_case("plain", (40, 16, 8))
    g = Droplet(P, (40, 16, 8), FORM_FP32)
    with pytest.raises(DropletError) as e:
        g.set_option("stage", 2)
    assert e.value.status == _abi.DL_ERR_UNSUPPORTED
    assert g.get_option("stage") == 0


def test_tensor_stage_wait_limit_reports_timeout():
    """The blocks' waits for the staged plane are bounded in time: with the
    mbarrier told to expect 16 bytes more than the copies bring, no phase
    completes, every block gives up after "wait_ns", the step finishes and
    dl_sync reports DL_ERR_TIMEOUT; the device stays usable."""
    shape = (64, 16, 12)
    P, f, mode, force = make_case("plain", shape)
    g = Droplet(P, shape, FORM_FP32)
    g.set_option("stage", 2)
    g.set_option("wait_ns", 200000)
    g.set_option("stage_extra_tx", 16)
    start(g, f, mode, force)
    g.step(2)
    with pytest.raises(DropletError) as e:
        g.sync()
    assert e.value.status == _abi.DL_ERR_TIMEOUT
    g.close()
    h = Droplet(P, shape, FORM_FP32)
    h.set_option("stage", 2)
    start(h, f, mode, force)
    h.step(3)
    h.sync()
    assert np.isfinite(h.get_fields()["phi"]).all()


@pytest.mark.parametrize("lz", [1, 5])
def test_tensor_staged_planes_with_uneven_z_chunks(lz):
    """Stage 2 (tensor copies) with z chunks that do not divide nz (5, 5, 4 of
    14) and with chunks of a single plane: the same bits as loads into registers."""
    shape = (64, 16, 14)
    P, f, mode, force = make_case("les_static_force", shape)
    out = {}
    for stage in (0, 2):
        g = Droplet(P, shape, FORM_FP32)
        g.set_option("stage", stage)
        g.set_option("lz", lz)
        start(g, f, mode, force)
        g.step(7)
        out[stage] = g.get_fields()
        g.sync()
    for k in out[0]:
        assert np.array_equal(out[0][k], out[2][k]), k
