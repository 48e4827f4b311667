"""Readers and writers for the reference's Fortran unformatted sequential
files, so that its analysis and plotting programs read this library's output
unchanged.

Layouts (one MPI rank holds the whole domain here, so one file per dump):
  * fields (output, program/lbm_drop_xy.f90:695-719): one record per site,
    loops z -> y -> x, each record phi, u1, u2, u3, p as five FP64 values;
  * populations (outputfg, :721-743): one record per site and direction,
    loops z -> y -> x -> i, each record (f_i, g_i) as two FP64 values;
  * precursor g (read at step_input, :789-823; written by
    program/lbm_iht_xy.f90:848-870): one FP64 g_i per record, loops
    z -> y -> x -> i; the LES variant (program/LES_drop_xy.f90) reads
    (dummy, g_i) pairs.
Each record is framed by 4-byte little-endian length markers, the gfortran
sequential-access convention.
"""
from __future__ import annotations

import numpy as np


def _rec_dtype(nvals: int):
    return np.dtype([("h", "<i4"), ("v", "<f8", (nvals,)), ("t", "<i4")])


def _write(path, values: np.ndarray):
    """values: (nrec, nvals) float64 -> framed records."""
    nrec, nvals = values.shape
    rec = np.empty(nrec, dtype=_rec_dtype(nvals))
    rec["h"] = 8 * nvals
    rec["t"] = 8 * nvals
    rec["v"] = values
    rec.tofile(path)


def _read(path, nvals: int) -> np.ndarray:
    rec = np.fromfile(path, dtype=_rec_dtype(nvals))
    if rec.size and not (np.all(rec["h"] == 8 * nvals) and np.all(rec["t"] == 8 * nvals)):
        raise ValueError(f"{path}: record markers do not match {nvals} FP64 values per record")
    return rec["v"]


def write_fields(path, fields: dict):
    """fields phi, u1, u2, u3, p with shape (nz, ny, nx)."""
    vals = np.stack([np.asarray(fields[k], dtype=np.float64).reshape(-1) for k in ("phi", "u1", "u2", "u3", "p")],
                    axis=1)
    _write(path, vals)


def read_fields(path, shape) -> dict:
    nx, ny, nz = shape
    v = _read(path, 5)
    if v.shape[0] != nx * ny * nz:
        raise ValueError(f"{path}: {v.shape[0]} records, expected {nx * ny * nz}")
    return {k: np.ascontiguousarray(v[:, j]).reshape(nz, ny, nx) for j, k in enumerate(("phi", "u1", "u2", "u3", "p"))}


def write_populations(path, f: np.ndarray, g: np.ndarray):
    """f, g with shape (nz, ny, nx, 15) (direction fastest)."""
    vals = np.stack([np.asarray(f, dtype=np.float64).reshape(-1), np.asarray(g, dtype=np.float64).reshape(-1)], axis=1)
    _write(path, vals)


def read_populations(path, shape):
    nx, ny, nz = shape
    v = _read(path, 2)
    if v.shape[0] != 15 * nx * ny * nz:
        raise ValueError(f"{path}: {v.shape[0]} records, expected {15 * nx * ny * nz}")
    return (np.ascontiguousarray(v[:, 0]).reshape(nz, ny, nx, 15), np.ascontiguousarray(v[:, 1]).reshape(nz, ny, nx, 15))


def write_precursor_g(path, g: np.ndarray, pairs: bool = False):
    """g with shape (nz, ny, nx, 15); pairs=True writes (0, g_i) records."""
    gv = np.asarray(g, dtype=np.float64).reshape(-1, 1)
    _write(path, np.concatenate([np.zeros_like(gv), gv], axis=1) if pairs else gv)


def read_precursor_g(path, shape, pairs: bool = False) -> np.ndarray:
    nx, ny, nz = shape
    v = _read(path, 2 if pairs else 1)
    if v.shape[0] != 15 * nx * ny * nz:
        raise ValueError(f"{path}: {v.shape[0]} records, expected {15 * nx * ny * nz}")
    return np.ascontiguousarray(v[:, -1]).reshape(nz, ny, nx, 15)


def moments_from_g(g: np.ndarray):
    """p = sum g / 3 and u = sum c g of a precursor g (the recomputation of
    program/lbm_drop_xy.f90:805-822)."""
    from .params import CX, CY, CZ

    p = g.sum(axis=-1) / 3.0
    u = [np.tensordot(g, np.asarray(c, dtype=np.float64), axes=([-1], [0])) for c in (CX, CY, CZ)]
    return p, u
