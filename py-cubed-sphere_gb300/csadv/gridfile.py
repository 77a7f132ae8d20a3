"""The reference's grid file and lat-lon index file (netCDF), without the netCDF4 package.

* ``save_grid_netcdf4(grid, path=None)`` -- plot.py:522-660: ``griddir + grid.name + ".nc"``
  with the reference's dimensions (panel, ix, jy, ix2, jy2, coorddim, r3dim, ed), scalar
  variables (dx, dy, a, ng, ngl, ngr, N, i0, iend, j0, jend) and point arrays (po, pc, pu, pv,
  ex_*, ey_*: [i][j][panel][X, Y, Z, lon, lat]); the arrays are computed on the GPU
  (``csadv_grid_points``).
* ``load_grid(path)`` -- what cubed_sphere(gridload=True) reads back (cs_datastruct.py:45-195):
  the scalars and, per point array, an object with X, Y, Z, lon, lat.
* ``ll2cs_netcdf(i, j, panel_list, cs_grid, path=None)`` -- plot.py:665-703:
  ``griddir + grid.name + "_ll2cs.nc"``, variables i, j, panel (lon, lat), int32.
* ``load_ll2cs(path)`` -- interpolation.py:49-58.
* ``latlon_netcdf(name, fields, ts, path=None)`` -- open_netcdf4 (plot.py:477-515) with its
  values filled: lat-lon fields {name: (Nlon, Nlat, nt)} at times ts, lat/lon axes as the
  reference sets them.

Files are netCDF classic (64-bit offsets; ``csadv.netcdf``), which netCDF4 reads; the reference
writes NETCDF4_CLASSIC (HDF5), which ``load_*`` refuses with a clear error.
"""
import os
from types import SimpleNamespace

import numpy as np

from . import _lib as L
from . import netcdf

griddir = "grid/"   # constants.py:30
datadir = "data/"   # constants.py:31

NBFACES = 6
_KINDS = ("po", "pc", "pu", "pv")


def grid_points(N, kind):
    """(P, EX, EY) of one point family of the equiangular grid with N cells per panel edge, each
    shaped [i][j][panel][5] as in the reference's grid file (computed on the GPU)."""
    k = _KINDS.index(kind)
    n = N + 8
    nx = n + 1 if kind in ("po", "pu") else n
    ny = n + 1 if kind in ("po", "pv") else n
    out = [np.empty((nx, ny, NBFACES, 5)) for _ in range(3)]
    L.check(L.lib().csadv_grid_points(int(N), k, out[0].ctypes.data, out[1].ctypes.data, out[2].ctypes.data, None),
            "csadv_grid_points")
    return tuple(out)


def _grid_path(grid, suffix=""):
    return os.path.join(griddir, grid.name + suffix + ".nc")


def save_grid_netcdf4(grid, path=None):
    """Write the grid file of `grid` (an object with N and name, e.g. csadv.advection.cubed_sphere)."""
    N = int(grid.N)
    n = N + 8
    a = np.pi / 4.0
    dx = (a - (-a)) / N
    path = path or _grid_path(grid)
    print("--------------------------------------------------------")
    print("Creating grid netcdf file " + path)
    dims = {"panel": NBFACES, "ix": n + 1, "jy": n + 1, "ix2": n, "jy2": n, "coorddim": 5, "r3dim": 3, "ed": 4}
    variables = [("dx", np.float64(dx), ()), ("dy", np.float64(dx), ()), ("a", np.float64(a), ())]
    for name, v in (("ng", 8), ("ngl", 4), ("ngr", 4), ("N", N), ("i0", 4), ("iend", 4 + N), ("j0", 4),
                    ("jend", 4 + N)):
        variables.append((name, np.int32(v), ()))
    axes = {"po": ("ix", "jy"), "pc": ("ix2", "jy2"), "pu": ("ix", "jy2"), "pv": ("ix2", "jy")}
    pts, tgs = [], []
    for kind in _KINDS:
        P, EX, EY = grid_points(N, kind)
        d = axes[kind] + ("panel", "coorddim")
        pts.append((kind, P, d))
        tgs += [("ex_" + kind, EX, d), ("ey_" + kind, EY, d)]
    netcdf.write(path, dims, variables + pts + tgs, {"title": grid.name})
    print("Done.")
    print("--------------------------------------------------------\n")
    return path


def load_grid(path):
    """The contents of a grid file as the reference's cubed_sphere holds them after loading."""
    ds = netcdf.read(path)
    g = SimpleNamespace()
    for k in ("dx", "dy", "a"):
        setattr(g, k, float(ds[k]))
    for k in ("N", "ng", "ngl", "ngr", "i0", "iend", "j0", "jend"):
        setattr(g, k, int(ds[k]))
    for kind in _KINDS:
        for pre in ("", "ex_", "ey_"):
            a = ds[pre + kind]
            setattr(g, pre + kind, SimpleNamespace(X=a[..., 0], Y=a[..., 1], Z=a[..., 2], lon=a[..., 3], lat=a[..., 4]))
    g.title = ds.attrs.get("title", "")
    return g


def ll2cs_netcdf(i, j, panel_list, cs_grid, path=None):
    """Write the lat-lon -> cubed-sphere index file."""
    path = path or _grid_path(cs_grid, "_ll2cs")
    Nlon, Nlat = np.shape(i)
    netcdf.write(path, {"lon": Nlon, "lat": Nlat},
                 [("i", np.asarray(i, dtype=np.int32), ("lon", "lat")),
                  ("j", np.asarray(j, dtype=np.int32), ("lon", "lat")),
                  ("panel", np.asarray(panel_list, dtype=np.int32), ("lon", "lat"))],
                 {"title": cs_grid.name + "_ll2cs"})
    return path


def load_ll2cs(path):
    """(i, j, panel) of an index file, uint32 as the reference reads them."""
    ds = netcdf.read(path)
    return tuple(np.asarray(ds[k]).astype(np.uint32) for k in ("i", "j", "panel"))


def latlon_netcdf(name, fields, ts, path=None):
    """Write lat-lon fields {name: (Nlon, Nlat, nt)} at times ts (open_netcdf4's file, filled)."""
    ts = np.atleast_1d(np.asarray(ts, dtype=np.float64))
    arrs = {k: np.asarray(v, dtype=np.float64) for k, v in fields.items()}
    if not arrs:
        raise ValueError("no fields")
    shp = next(iter(arrs.values())).shape
    if len(shp) != 3 or shp[2] != ts.size or any(a.shape != shp for a in arrs.values()):
        raise ValueError("fields must all be (Nlon, Nlat, len(ts))")
    m, n = shp[0], shp[1]
    path = path or os.path.join(datadir, name + ".nc")
    variables = [("time", ts, ("time",)), ("lat", np.linspace(-90.0, 90.0, n), ("lat",)),
                 ("lon", np.linspace(-180.0, 180.0, m), ("lon",))]
    variables += [(k, a, ("lon", "lat", "time")) for k, a in arrs.items()]
    netcdf.write(path, {"time": ts.size, "lat": n, "lon": m}, variables, {"title": name})
    return path
