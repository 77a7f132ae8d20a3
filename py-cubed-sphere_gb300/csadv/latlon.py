"""Lat-lon output of cubed-sphere fields: the reference's plotting path without the plots.

Same names and arguments as the reference:

* ``latlon_grid(Nlat, Nlon)``                   -- cs_datastruct.py:569-582
* ``ll2cs(cs_grid, latlon_grid)``               -- interpolation.py:38-140
* ``nearest_neighbour(Q, cs_grid, latlon_grid)`` -- interpolation.py:145-150

``ll2cs`` runs on the GPU (``csadv_ll2cs``).  ``nearest_neighbour`` gathers on the GPU when
``Q`` is a plan tracer (``csadv.Plan`` or ``(plan, tracer)``) or a simulation of
``csadv.advection``; for an array already on the host (``Q.f`` or an ``(N, N, 6)`` array, as the
reference's grid-quality fields are) it indexes that array as the reference does.  The result
is ``(Nlon, Nlat)`` float64, written to ``.npy`` by ``save_latlon`` where the reference plots it.
"""
import ctypes

import numpy as np

from . import _lib as L

NLAT = 720        # lat-lon grid of the reference's plots (constants.py:36-37)
NLON = 2 * NLAT


class latlon_grid:
    """Regular lon-lat grid; X, Y, Z on the unit sphere (cs_datastruct.py:569-582)."""

    def __init__(self, Nlat, Nlon):
        self.Nlat, self.Nlon = int(Nlat), int(Nlon)
        lat = np.linspace(-np.pi * 0.5, np.pi * 0.5, self.Nlat)
        lon = np.linspace(-np.pi, np.pi, self.Nlon)
        self.lat, self.lon = np.meshgrid(lat, lon)
        # sph2cart (sphgeo.py:18-22)
        self.X = np.cos(self.lat) * np.cos(self.lon)
        self.Y = np.cos(self.lat) * np.sin(self.lon)
        self.Z = np.sin(self.lat)
        self.ix, self.jy, self.mask = [], [], []


def ll2cs(cs_grid, latlon_grid):
    """Panel and interior cell indices of every lat-lon point (interpolation.py:38-140), on the GPU.
    Returns (i, j, panel), uint32 arrays shaped like the lat-lon grid.

    As the reference does, the indices are kept in ``griddir + cs_grid.name + "_ll2cs.nc"``: read
    from there when that file exists (and matches the lat-lon grid's shape), else computed and
    written there.  The file is used only when the grid directory exists (the reference's driver
    creates it; ``python -m csadv`` does too), so library calls elsewhere leave no files."""
    import os
    from . import gridfile
    if getattr(cs_grid, "projection", "gnomonic_equiangular") != "gnomonic_equiangular":
        print("ERROR: invalid grid transformation.")
        raise SystemExit(1)
    name = getattr(cs_grid, "name", None)
    path = os.path.join(gridfile.griddir, name + "_ll2cs.nc") if name else None
    use_file = path is not None and os.path.isdir(gridfile.griddir)
    if use_file and os.path.isfile(path):
        i, j, p = gridfile.load_ll2cs(path)
        if i.shape == np.shape(latlon_grid.X):
            return i, j, p
    i, j, p = _ll2cs_gpu(cs_grid, latlon_grid)
    if use_file:
        gridfile.ll2cs_netcdf(i, j, p, cs_grid, path)
    return i, j, p


def _ll2cs_gpu(cs_grid, latlon_grid):
    X = np.ascontiguousarray(latlon_grid.X, dtype=np.float64)
    Y = np.ascontiguousarray(latlon_grid.Y, dtype=np.float64)
    Z = np.ascontiguousarray(latlon_grid.Z, dtype=np.float64)
    shp = X.shape
    i = np.empty(shp, dtype=np.uint32)
    j = np.empty(shp, dtype=np.uint32)
    p = np.empty(shp, dtype=np.uint32)
    L.check(L.lib().csadv_ll2cs(int(cs_grid.N), X.ctypes.data, Y.ctypes.data, Z.ctypes.data, X.size, i.ctypes.data,
                                j.ctypes.data, p.ctypes.data, None), "csadv_ll2cs")
    return i, j, p


def _plan_tracer(Q):
    from .plan import Plan
    if isinstance(Q, Plan):
        return Q, 0
    if isinstance(Q, tuple) and len(Q) == 2 and isinstance(Q[0], Plan):
        return Q
    plan = getattr(Q, "plan", None)
    if isinstance(plan, Plan):  # csadv.advection.adv_simulation_par
        return plan, 0
    return None, 0


def nearest_neighbour(Q, cs_grid, latlon_grid):
    """Q at the cell of every lat-lon point (interpolation.py:145-150), shape (Nlon, Nlat)."""
    ix = np.ascontiguousarray(latlon_grid.ix, dtype=np.uint32)
    jy = np.ascontiguousarray(latlon_grid.jy, dtype=np.uint32)
    mask = np.ascontiguousarray(latlon_grid.mask, dtype=np.uint32)
    plan, tracer = _plan_tracer(Q)
    if plan is not None:
        out = np.empty(ix.shape, dtype=np.float64)
        L.check(L.lib().csadv_nearest_neighbour(plan._h, int(tracer), ix.ctypes.data, jy.ctypes.data,
                                                mask.ctypes.data, ix.size, out.ctypes.data, plan.stream),
                "csadv_nearest_neighbour")
        return out
    f = np.asarray(getattr(Q, "f", Q))
    Q_ll = np.zeros((latlon_grid.Nlon, latlon_grid.Nlat))
    for p in range(6):
        m = mask == p
        Q_ll[m] = f[ix[m], jy[m], p]
    return Q_ll


def save_latlon(path, Q, cs_grid, latlon_grid):
    """nearest_neighbour(Q, ...) written as an .npy array (the headless form of the
    reference's lat-lon plots, plot.py)."""
    Q_ll = nearest_neighbour(Q, cs_grid, latlon_grid)
    np.save(path, Q_ll)
    return Q_ll
