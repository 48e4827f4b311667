"""The NumPy periodic labelling used as the checker of dl_label_droplets,
against a breadth-first search over the same neighbour sets."""
from collections import deque

import numpy as np
import pytest

from oracle import np_labels


def bfs_volumes(mask, conn):
    nz, ny, nx = mask.shape
    seen = np.zeros_like(mask, dtype=bool)
    dirs = np_labels.neighbour_set(conn)
    vols = []
    for s in zip(*np.nonzero(mask)):
        if seen[s]:
            continue
        seen[s] = True
        q = deque([s])
        n = 0
        while q:
            z, y, x = q.popleft()
            n += 1
            for dx, dy, dz in dirs:
                t = ((z + dz) % nz, (y + dy) % ny, (x + dx) % nx)
                if mask[t] and not seen[t]:
                    seen[t] = True
                    q.append(t)
        vols.append(n)
    return sorted(vols, reverse=True)


@pytest.mark.parametrize("conn", [6, 14, 18, 26])
def test_neighbour_counts(conn):
    dirs = np_labels.neighbour_set(conn)
    assert len(dirs) == conn
    assert set(dirs) == {(-a, -b, -c) for a, b, c in dirs}


@pytest.mark.parametrize("conn", [6, 14, 18, 26])
@pytest.mark.parametrize("density", [0.2, 0.35])
def test_label_matches_bfs(conn, density):
    rng = np.random.default_rng(conn * 7 + int(density * 100))
    mask = rng.random((9, 7, 11)) < density
    vols, lab = np_labels.label(mask, conn)
    assert list(vols.astype(int)) == bfs_volumes(mask, conn)
    assert (lab > 0).sum() == mask.sum()
    for k, v in enumerate(vols):
        assert (lab == k + 1).sum() == v


def test_periodic_join():
    mask = np.zeros((4, 4, 8), dtype=bool)
    mask[1, 1, 0] = mask[1, 1, 7] = True      # joined across x
    mask[3, 2, 3] = mask[0, 2, 3] = True      # joined across z
    vols, _ = np_labels.label(mask, 6)
    assert list(vols) == [2.0, 2.0]


def test_edges_of_14():
    mask = np.zeros((6, 6, 6), dtype=bool)
    mask[2, 2, 2] = mask[3, 2, 3] = True      # xz edge: joined under 14
    mask[2, 4, 4] = mask[2, 5, 5] = True      # xy edge: not joined under 14
    assert list(np_labels.label(mask, 14)[0]) == [2.0, 1.0, 1.0]
    assert list(np_labels.label(mask, 18)[0]) == [2.0, 2.0]
