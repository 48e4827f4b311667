"""The plain C host (tests/c/abi_host.c) run on the GPU gives the same
diagnostics as the Python host on the same inputs (the initial phi the C
program wrote), bit for bit in every form: one library, one step sequence."""
import subprocess

import numpy as np
import pytest

from droplet_gb300 import Params
from droplet_gb300 import _abi
from droplet_gb300.solver import Droplet, FORM_FP32, FORM_FP64

from c_host import build

pytestmark = pytest.mark.gpu


def python_host(form, shape, steps, phi):
    P = Params.lbm_drop_xy().replace(tauf=0.8, kappaf=0.01, kappag=2e-3, nu1=0.1, nu2=0.1,
                                     visc_mode=_abi.DL_VISC_MINMAX, kc=3)
    zero = np.zeros_like(phi)
    g = Droplet(P, shape, form)
    g.set_fields(phi, zero, zero, zero, np.full_like(phi, 1.0 / 3.0))
    g.init_equilibrium()
    g.step(steps)
    d = g.reduce()
    g.close()
    return [d["phi_sum"], d["p_sum"], *d["mom"], d["vol_count"], d["phi_min"], d["phi_max"], d["step"]]


@pytest.mark.parametrize("form", [FORM_FP64, FORM_FP32])
def test_c_host_matches_python_host(tmp_path, form):
    shape, steps = (24, 20, 16), 8
    exe = build(tmp_path)
    phi_file = str(tmp_path / "phi0.bin")
    out = subprocess.run([exe, str(form), *map(str, shape), str(steps), phi_file], capture_output=True, text=True,
                         check=True)
    c = [float(v) for v in out.stdout.split()]
    nx, ny, nz = shape
    phi = np.fromfile(phi_file, dtype=np.float64).reshape(nz, ny, nx)
    py = python_host(form, shape, steps, phi)
    assert c[-1] == py[-1] == steps
    assert c[:8] == [float(v) for v in py[:8]]
