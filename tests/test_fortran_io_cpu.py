"""Fortran record-format I/O (no GPU): byte layout and round trips."""
import numpy as np

from droplet_gb300 import fortran_io


def test_fields_record_layout_and_roundtrip(tmp_path):
    shape = (3, 2, 2)
    nx, ny, nz = shape
    rng = np.random.default_rng(0)
    f = {k: rng.standard_normal((nz, ny, nx)) for k in ("phi", "u1", "u2", "u3", "p")}
    p = tmp_path / "0_0_100.bin"
    fortran_io.write_fields(p, f)
    raw = p.read_bytes()
    assert len(raw) == nx * ny * nz * (4 + 40 + 4)
    assert np.frombuffer(raw[:4], "<i4")[0] == 40 and np.frombuffer(raw[44:48], "<i4")[0] == 40
    # first record = site (x=0, y=0, z=0): phi, u1, u2, u3, p
    first = np.frombuffer(raw[4:44], "<f8")
    assert np.array_equal(first, [f[k][0, 0, 0] for k in ("phi", "u1", "u2", "u3", "p")])
    # second record = x = 1 (x fastest, the Fortran loop order)
    second = np.frombuffer(raw[52:92], "<f8")
    assert second[0] == f["phi"][0, 0, 1]
    back = fortran_io.read_fields(p, shape)
    for k in f:
        assert np.array_equal(back[k], f[k])


def test_populations_and_precursor_roundtrip(tmp_path):
    shape = (2, 3, 2)
    nx, ny, nz = shape
    rng = np.random.default_rng(1)
    f = rng.standard_normal((nz, ny, nx, 15))
    g = rng.standard_normal((nz, ny, nx, 15))
    fortran_io.write_populations(tmp_path / "fg.bin", f, g)
    raw = (tmp_path / "fg.bin").read_bytes()
    assert len(raw) == 15 * nx * ny * nz * 24
    f2, g2 = fortran_io.read_populations(tmp_path / "fg.bin", shape)
    assert np.array_equal(f2, f) and np.array_equal(g2, g)
    for pairs in (False, True):
        fortran_io.write_precursor_g(tmp_path / "pre.bin", g, pairs=pairs)
        assert np.array_equal(fortran_io.read_precursor_g(tmp_path / "pre.bin", shape, pairs=pairs), g)
    p, u = fortran_io.moments_from_g(g)
    assert np.allclose(p, g.sum(-1) / 3) and np.allclose(u[0], g[..., 1] - g[..., 4] + g[..., 7] - g[..., 8]
                                                          + g[..., 9] + g[..., 10] - g[..., 11] + g[..., 12]
                                                          - g[..., 13] - g[..., 14])
