"""Oracle (test infrastructure): numpy restatement of the reference's lat-lon sampling.

* ``ll2cs(N, X, Y, Z)``             -- interpolation.py:38-140 (equiangular grid, no caching)
* ``nearest_neighbour(f, i, j, p)`` -- interpolation.py:145-150

Pinned against the reference run in this container (tests/golden/latlon.npz).
"""
import numpy as np


def inverse_equiangular_gnomonic_map(X, Y, Z, panel):
    """cs_transform.py:101-126"""
    if panel == 0:
        tanx, tany = Y / X, Z / X
    elif panel == 1:
        tanx, tany = -X / Y, Z / Y
    elif panel == 2:
        tanx, tany = Y / X, -Z / X
    elif panel == 3:
        tanx, tany = -X / Y, -Z / Y
    elif panel == 4:
        tanx, tany = Y / Z, -X / Z
    else:
        tanx, tany = -Y / Z, -X / Z
    return np.arctan(tanx), np.arctan(tany)


def ll2cs(N, X, Y, Z):
    """Panel and interior indices (i, j) of the cell holding each point (interpolation.py:38-140)."""
    pio4 = (np.pi * 0.5) * 0.5
    dx = 2 * pio4 / N
    xmin = -pio4
    i = np.zeros(np.shape(X), dtype=np.uint32)
    j = np.zeros(np.shape(X), dtype=np.uint32)
    panel = np.zeros(np.shape(X), dtype=np.uint32)
    P = np.stack([np.abs(X), np.abs(Y), np.abs(Z)], axis=-1)
    PM = P.max(axis=-1)
    # masks in the reference's order: a later one overrides an earlier one
    panel[np.logical_and(PM == np.abs(X), X > 0)] = 0
    panel[np.logical_and(PM == np.abs(Y), Y > 0)] = 1
    panel[np.logical_and(PM == np.abs(X), X < 0)] = 2
    panel[np.logical_and(PM == np.abs(Y), Y < 0)] = 3
    panel[np.logical_and(PM == np.abs(Z), Z > 0)] = 4
    panel[np.logical_and(PM == np.abs(Z), Z <= 0)] = 5
    for p in range(6):
        m = panel == p
        x, y = inverse_equiangular_gnomonic_map(X[m], Y[m], Z[m], p)
        i[m] = np.array(np.floor((x - xmin) / dx), dtype=np.uint32)
        j[m] = np.array(np.floor((y - xmin) / dx), dtype=np.uint32)
    return i, j, panel


def nearest_neighbour(f, i, j, panel):
    """f[i, j, panel] per lat-lon point (interpolation.py:145-150); f is (N, N, 6)."""
    out = np.zeros(np.shape(i))
    for p in range(6):
        m = panel == p
        out[m] = f[i[m], j[m], p]
    return out
