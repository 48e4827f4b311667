"""Batched ensembles over members of uneven sizes and parameters, in both
modes: the members' own steps launched concurrently (the default) and one
persistent launch per step (in the push form when every member takes it, FP32;
else the pull form). Each member must get the result it gets when stepped on
its own in the same form (bitwise without spectral forcing, whose FP64
accumulation order is not fixed; within FP32 rounding with it)."""
import numpy as np
import pytest

from droplet_gb300 import Params, init_fields
from droplet_gb300 import _abi
from droplet_gb300.ensemble import Ensemble
from droplet_gb300.solver import Droplet, FORM_FP32, FORM_FP16

pytestmark = pytest.mark.gpu

SHAPES = [(40, 20, 16), (32, 32, 24), (48, 16, 12), (24, 24, 24)]


def member_case(m, shape, spectral, les):
    nx, ny, nz = shape
    P = Params.lbm_drop_xy().replace(tauf=0.8, nu1=0.1, nu2=0.1, kappag=1e-3 * (1 + m))
    if les:
        P = P.replace(les=True, Cs=0.1, delta=1.0)
    if spectral:
        P = P.replace(eps=1e-6, kc=3)
    rng = np.random.default_rng(100 + m)
    phi = init_fields.tanh_droplets(shape, P, [(nx / 2 + m, ny / 2, nz / 2)], [min(shape) / 4], width=1.5)
    u = [0.01 * rng.standard_normal((nz, ny, nx)) for _ in range(3)]
    return P, init_fields.fields(phi, *u)


def start(sim, f, spectral):
    sim.set_fields(**f)
    sim.init_equilibrium()
    sim.set_force(_abi.DL_FORCE_SPECTRAL if spectral else _abi.DL_FORCE_NONE)


@pytest.mark.parametrize("form,push", [(FORM_FP32, 1), (FORM_FP32, 0), (FORM_FP16, 0)])
@pytest.mark.parametrize("persistent,spectral,les,graph,steps", [(1, False, False, 1, 7), (1, False, True, 0, 6),
                                                                 (1, True, True, 1, 9), (0, False, True, 0, 7),
                                                                 (0, True, True, 0, 9)])
def test_ensemble_matches_members_stepped_alone(form, push, persistent, spectral, les, graph, steps):
    cases = [member_case(m, s, spectral, les) for m, s in enumerate(SHAPES)]
    ens = Ensemble([c[0] for c in cases], SHAPES, form)
    ens.set_option("persistent", persistent)
    assert ens.get_option("persistent") == persistent
    ens.set_option("graph", graph)
    ens.set_option("lz", 8)
    for mem, (P, f) in zip(ens.members, cases):
        if form == FORM_FP32:
            mem.set_option("push", push)
        start(mem, f, spectral)
    ens.step(steps)
    for m, (mem, (P, f)) in enumerate(zip(ens.members, cases)):
        solo = Droplet(P, SHAPES[m], form)
        solo.set_option("lz", 8)
        if form == FORM_FP32:
            solo.set_option("push", push)
        start(solo, f, spectral)
        solo.step(steps)
        a, b = mem.get_fields(), solo.get_fields()
        assert mem.step_count == steps
        for k in ("phi", "u1", "u2", "u3", "p"):
            if spectral:
                assert np.abs(a[k] - b[k]).max() <= 1e-5 * max(1.0, np.abs(b[k]).max()), (m, k)
            else:
                assert np.array_equal(a[k], b[k]), (m, k, np.abs(a[k] - b[k]).max())
        assert mem.reduce()["nan_flag"] == 0


def test_ensemble_options_and_state_checks():
    cases = [member_case(m, s, False, False) for m, s in enumerate(SHAPES[:2])]
    ens = Ensemble([c[0] for c in cases], SHAPES[:2], FORM_FP32)
    for opt, val in (("lz", 4), ("blocks_per_sm", 1), ("graph", 0), ("persistent", 1), ("persistent", 0)):
        ens.set_option(opt, val)
        assert ens.get_option(opt) == val
    from droplet_gb300 import DropletError

    with pytest.raises(DropletError):
        ens.step(1)  # members not initialised


def test_concurrent_members_need_not_be_in_step():
    """The default mode steps each member from its own state: member 0 taken one
    step ahead alone, then the whole ensemble stepped, ends where a solo run of
    one more step ends (bitwise, no spectral forcing), the others as solo runs."""
    cases = [member_case(m, s, False, True) for m, s in enumerate(SHAPES)]
    ens = Ensemble([c[0] for c in cases], SHAPES, FORM_FP32)
    assert ens.get_option("persistent") == 0
    ens.set_option("lz", 8)
    for mem, (P, f) in zip(ens.members, cases):
        start(mem, f, False)
    ens.members[0].step(1)
    ens.step(5)
    for m, (mem, (P, f)) in enumerate(zip(ens.members, cases)):
        solo = Droplet(P, SHAPES[m], FORM_FP32)
        solo.set_option("lz", 8)
        start(solo, f, False)
        solo.step(6 if m == 0 else 5)
        a, b = mem.get_fields(), solo.get_fields()
        for k in ("phi", "u1", "u2", "u3", "p"):
            assert np.array_equal(a[k], b[k]), (m, k)
        assert mem.step_count == (6 if m == 0 else 5)


def test_concurrent_members_on_their_own_streams():
    """Members whose handles carry streams of their own (set-up enqueued there):
    the batched steps wait for those streams and the members' streams see the
    results, so every member still equals its solo run."""
    import torch

    cases = [member_case(m, s, True, True) for m, s in enumerate(SHAPES)]
    ens = Ensemble([c[0] for c in cases], SHAPES, FORM_FP32)
    streams = [torch.cuda.Stream() for _ in SHAPES]
    for mem, st, (P, f) in zip(ens.members, streams, cases):
        mem.set_stream(st.cuda_stream)
        start(mem, f, True)
    ens.step(6)
    for m, (mem, (P, f)) in enumerate(zip(ens.members, cases)):
        solo = Droplet(P, SHAPES[m], FORM_FP32)
        start(solo, f, True)
        solo.step(6)
        a, b = mem.get_fields(), solo.get_fields()
        for k in ("phi", "u1", "u2", "u3", "p"):
            assert np.abs(a[k] - b[k]).max() <= 1e-5 * max(1.0, np.abs(b[k]).max()), (m, k)


@pytest.mark.parametrize("persistent", [0, 1])
def test_ensemble_with_moving_walls_matches_members_alone(persistent):
    """Members with moving walls (sheared droplets) in both modes, the persistent
    one in the push form: the wall terms travel in each member's step arguments;
    bitwise equal to each member stepped alone."""
    shapes = [(32, 16, 16), (24, 24, 20), (40, 16, 12)]
    cases = []
    for m, shape in enumerate(shapes):
        nx, ny, nz = shape
        P = Params.lbm_drop_xy().replace(tauf=0.8, nu1=0.1, nu2=0.1, kappag=1e-3 * (1 + m), walls=True,
                                         wall_u=(0.02 * (m + 1), 0.0, 0.0), wall_start=1)
        phi = init_fields.tanh_droplets(shape, P, [(nx / 2, ny / 2, nz / 2)], [min(shape) / 4], width=1.5)
        cases.append((P, init_fields.fields(phi)))
    ens = Ensemble([c[0] for c in cases], shapes, FORM_FP32)
    ens.set_option("persistent", persistent)
    ens.set_option("lz", 8)
    for mem, (P, f) in zip(ens.members, cases):
        start(mem, f, False)
    ens.step(9)
    for m, (mem, (P, f)) in enumerate(zip(ens.members, cases)):
        solo = Droplet(P, shapes[m], FORM_FP32)
        solo.set_option("lz", 8)
        start(solo, f, False)
        solo.step(9)
        a, b = mem.get_fields(), solo.get_fields()
        for k in ("phi", "u1", "u2", "u3", "p"):
            assert np.array_equal(a[k], b[k]), (m, k, np.abs(a[k] - b[k]).max())
