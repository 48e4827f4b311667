"""Failure detection without a GPU fault: a non-finite value is planted in the
host-side input, the step kernels' watchdog flags it, dl_sync returns
DL_ERR_NAN with the step at which it was first seen, and the CUDA context
stays usable for the next handle."""
import numpy as np
import pytest

from droplet_gb300 import DropletError, Params, init_fields
from droplet_gb300 import _abi
from droplet_gb300.solver import Droplet, FORM_FP64, FORM_FP32, FORM_FP16

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("form", [FORM_FP64, FORM_FP32, FORM_FP16])
def test_nan_watchdog_reports_and_context_survives(form):
    shape = (16, 16, 16)
    P = Params.lbm_drop_xy().replace(tauf=0.8, visc_mode=_abi.DL_VISC_FIXED)
    phi = init_fields.tanh_droplets(shape, P, [(7.5, 7.5, 7.5)], [4.0])
    f = init_fields.fields(phi)
    f["u1"][3, 4, 5] = np.nan
    g = Droplet(P, shape, form)
    g.set_fields(**f)
    g.init_equilibrium()
    g.step(2)
    with pytest.raises(DropletError) as ei:
        g.sync()
    assert ei.value.status == _abi.DL_ERR_NAN
    assert g.reduce()["nan_flag"] == 1
    g.close()
    # a fresh handle on the same context steps normally
    h = Droplet(P, shape, form)
    f2 = init_fields.fields(phi)
    h.set_fields(**f2)
    h.init_equilibrium()
    h.step(3)
    h.sync()
    assert np.isfinite(h.get_fields()["phi"]).all()
