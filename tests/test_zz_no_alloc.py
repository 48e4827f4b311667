"""dl_reduce_static (diagnostics with no device allocation, fixed scratch
inside the library) against dl_reduce on the same fields: two calls in a row
each agree with dl_reduce to rounding and are identical to each other, for
every form and for the smallest, default and largest block counts. Block
counts beyond the scratch are refused with a message."""
import numpy as np
import pytest

from droplet_gb300 import DropletError, Params, init_fields
from droplet_gb300 import _abi
from droplet_gb300.solver import Droplet, FORM_FP16, FORM_FP32, FORM_FP64

pytestmark = pytest.mark.gpu

REL = 1e-12  # relative to the sum of the magnitudes of a quantity's terms


def make(form, shape=(36, 28, 20), steps=3):
    nx, ny, nz = shape
    P = Params.lbm_drop_xy().replace(tauf=0.8, nu1=0.1, nu2=0.05, kappag=2e-3)
    rng = np.random.default_rng(11)
    phi = init_fields.tanh_droplets(shape, P, [(10.0, 14.0, 9.0), (27.0, 6.0, 12.0)], [6.0, 4.5], width=1.5)
    u = [0.02 * rng.standard_normal((nz, ny, nx)) for _ in range(3)]
    sim = Droplet(P, shape, form)
    sim.set_fields(**init_fields.fields(phi, *u))
    sim.init_equilibrium()
    sim.step(steps)
    return sim


def scales(sim):
    """Per quantity, a bound on the sum of the magnitudes of its terms."""
    n = sim.nx * sim.ny * sim.nz
    f = sim.get_fields()
    P = sim.params
    ph = np.abs(f["phi"]).max()
    pm = np.abs(f["p"]).max()
    um = max(np.abs(f[k]).max() for k in ("u1", "u2", "u3"))
    wm = max(np.abs((f["phi"] - P.phi1) / (P.phi2 - P.phi1)).max(), 1.0)
    ext = float(max(sim.nx, sim.ny, sim.nz))
    return {"phi_sum": n * ph, "p_sum": n * pm, "p_in": n * pm, "p_out": n * pm, "mom": n * um,
            "vol_smooth": n * wm, "w_sum": n * wm, "w_x": n * wm * ext, "w_xx": n * wm * ext * ext}


def compare(ref, got, scale):
    for k, v in ref.items():
        if k in ("step", "nan_flag", "phi_min", "phi_max"):
            assert got[k] == v, k
            continue
        # ke, diss and the counts have terms of one sign: their own size bounds them
        s = scale.get(k, float(np.abs(np.asarray(v, dtype=float)).max()))
        assert np.allclose(np.asarray(got[k], dtype=float), np.asarray(v, dtype=float), rtol=0.0,
                           atol=REL * max(s, 1e-30)), (k, got[k], v)


@pytest.mark.parametrize("form", [FORM_FP64, FORM_FP32, FORM_FP16])
@pytest.mark.parametrize("nblocks", [0, 1, 304, _abi.DL_REDUCE_STATIC_MAX_BLOCKS])
def test_static_matches_reduce_twice(form, nblocks):
    sim = make(form)
    scale = scales(sim)
    first = sim.reduce_static(nblocks)
    ref = sim.reduce()
    second = sim.reduce_static(nblocks)
    compare(ref, first, scale)
    compare(ref, second, scale)
    assert first == second
    sim.step(2)
    ref2 = sim.reduce()
    third = sim.reduce_static(nblocks)
    compare(ref2, third, scale)
    sim.close()


def test_two_handles_in_turn():
    a, b = make(FORM_FP32), make(FORM_FP64, shape=(24, 24, 24), steps=2)
    for _ in range(2):
        compare(a.reduce(), a.reduce_static(), scales(a))
        compare(b.reduce(), b.reduce_static(), scales(b))
    a.close()
    b.close()


@pytest.mark.parametrize("nblocks", [-1, _abi.DL_REDUCE_STATIC_MAX_BLOCKS + 1, 1 << 20])
def test_block_count_beyond_scratch_is_refused(nblocks):
    sim = make(FORM_FP32, steps=0)
    with pytest.raises(DropletError) as e:
        sim.reduce_static(nblocks)
    assert str(_abi.DL_REDUCE_STATIC_MAX_BLOCKS) in str(e.value)
    # the handle stays usable
    compare(sim.reduce(), sim.reduce_static(), scales(sim))
    sim.close()
