"""Periodic connected-component labelling by iterated minimum propagation.
TEST INFRASTRUCTURE ONLY (checker of dl_label_droplets)."""
from __future__ import annotations

import numpy as np


def neighbour_set(conn: int):
    out = []
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                n = (dx != 0) + (dy != 0) + (dz != 0)
                if n == 0:
                    continue
                if conn == 6 and n != 1:
                    continue
                if conn == 18 and n > 2:
                    continue
                if conn == 14 and not (n == 1 or (n == 2 and dz != 0)):
                    continue
                out.append((dx, dy, dz))
    return out


def label(mask: np.ndarray, conn: int):
    """Returns (volumes sorted decreasing, labels with 0 = background and
    k = k-th largest component)."""
    big = np.iinfo(np.int64).max
    lab = np.where(mask, np.arange(mask.size, dtype=np.int64).reshape(mask.shape), big)
    dirs = neighbour_set(conn)
    while True:
        new = lab.copy()
        for dx, dy, dz in dirs:
            nb = np.roll(lab, shift=(-dz, -dy, -dx), axis=(0, 1, 2))
            new = np.minimum(new, nb)
        new = np.where(mask, new, big)
        if np.array_equal(new, lab):
            break
        lab = new
    roots, counts = np.unique(lab[mask], return_counts=True)
    order = np.argsort(-counts, kind="stable")
    out = np.zeros(mask.shape, dtype=np.int32)
    for rank, k in enumerate(order):
        out[lab == roots[k]] = rank + 1
    return counts[order].astype(np.float64), out
