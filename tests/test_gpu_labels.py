"""Droplet labelling on the GPU against a NumPy periodic labelling: same
partition into components (up to the order of equal volumes) and the same
volumes, for every connectivity, for droplets that cross the periodic
boundaries."""
import numpy as np
import pytest

from droplet_gb300 import Params, init_fields
from droplet_gb300.solver import Droplet, FORM_FP64, FORM_FP32, FORM_FP16
from oracle import np_labels

pytestmark = pytest.mark.gpu


def field(shape, P, seed):
    nx, ny, nz = shape
    rng = np.random.default_rng(seed)
    centers = [(rng.uniform(0, nx), rng.uniform(0, ny), rng.uniform(0, nz)) for _ in range(9)]
    centers += [(0.2, ny / 2, nz / 2), (nx / 2, ny - 0.4, 0.3)]  # across the boundaries
    radii = list(rng.uniform(1.0, 4.0, size=len(centers)))
    phi = init_fields.tanh_droplets(shape, P, centers, radii, width=1.0)
    phi += 0.6 * (P.phi2 - P.phi1) * (rng.random(phi.shape) < 0.02)  # isolated specks
    return phi


def same_partition(a, b):
    pairs = set(zip(a.reshape(-1).tolist(), b.reshape(-1).tolist()))
    la = {p[0] for p in pairs}
    lb = {p[1] for p in pairs}
    return len(pairs) == len(la) == len(lb)


@pytest.mark.parametrize("form", [FORM_FP64, FORM_FP32, FORM_FP16])
@pytest.mark.parametrize("conn", [6, 14, 18, 26])
def test_labels_match_numpy(form, conn):
    shape = (40, 24, 20)
    P = Params.lbm_drop_xy()
    phi = field(shape, P, seed=conn)
    g = Droplet(P, shape, form)
    g.set_fields(**init_fields.fields(phi))
    vols, lab = g.label_droplets(conn, labels=True)
    if form == FORM_FP64:
        mask = phi >= (P.phi1 + P.phi2) / 2.0
    else:
        d = (phi - P.phi1).astype(np.float32)
        mask = d >= np.float32((P.phi2 - P.phi1) / 2.0)
    rv, rl = np_labels.label(mask, conn)
    assert np.array_equal(vols, rv)
    assert same_partition(lab, rl)
    assert (lab > 0).sum() == mask.sum()
