"""Gnomonic equiangular cubed-sphere geometry (oracle restatement).

Follows cs_datastruct.py:197-493 (grid points, metric tensor, lat-lon/contravariant
coefficients), cs_transform.py:41-96 (equiangular map), :245-397 (tangent vectors) and
sphgeo.py:18-33, 72-88 (spherical conversions, geographic unit vectors).  Unit sphere
(R = 1, cs_datastruct.py:37), 4 ghost cells per side (cs_datastruct.py:225-226).

Panel numbering follows the reference (cs_transform.py:21-28): 0-3 around the equator
(0 centred on lon 0), 4 the north cap, 5 the south cap.
"""
import numpy as np

NBFACES = 6
NGL = 4
NGR = 4
NG = NGL + NGR


def _panel_xyz(invD, XoD, YoD):
    """Cartesian coordinates of each panel (cs_transform.py:63-91)."""
    shp = invD.shape + (NBFACES,)
    X = np.zeros(shp)
    Y = np.zeros(shp)
    Z = np.zeros(shp)
    X[..., 0], Y[..., 0], Z[..., 0] = invD, XoD, YoD
    X[..., 1], Y[..., 1], Z[..., 1] = -XoD, invD, YoD
    X[..., 2], Y[..., 2], Z[..., 2] = -invD, -XoD, YoD
    X[..., 3], Y[..., 3], Z[..., 3] = XoD, -invD, YoD
    X[..., 4], Y[..., 4], Z[..., 4] = -YoD, XoD, invD
    X[..., 5], Y[..., 5], Z[..., 5] = YoD, XoD, -invD
    return X, Y, Z


def cart2sph(X, Y, Z):
    """sphgeo.py:29-33."""
    hyp = np.hypot(X, Y)
    return np.arctan2(Y, X), np.arctan2(Z, hyp)


def sph2cart(lon, lat):
    """sphgeo.py:18-22."""
    return np.cos(lat) * np.cos(lon), np.cos(lat) * np.sin(lon), np.sin(lat)


def equiangular_points(x, y):
    """Equiangular gnomonic map of the tensor grid (x, y) on every panel (cs_transform.py:41-96)."""
    xx, yy = np.meshgrid(x, y, indexing="ij")
    tx = np.tan(xx)
    ty = np.tan(yy)
    D = np.sqrt(1.0 + tx**2 + ty**2)
    invD = 1.0 / D
    X, Y, Z = _panel_xyz(invD, invD * tx, invD * ty)
    lon, lat = cart2sph(X, Y, Z)
    return X, Y, Z, lon, lat


def _tangent(x, y, direction):
    """Tangent vector d(point)/dx or d(point)/dy of the equiangular map.

    The reference evaluates the equidistant tangent at (a tan x, a tan y) and scales it by
    a / cos^2 (cs_transform.py:245-397); the same arithmetic is restated here.
    """
    R = 1.0
    a = R / np.sqrt(3.0)
    xe, ye = np.meshgrid(a * np.tan(x), a * np.tan(y), indexing="ij")
    r2 = a**2 + xe**2 + ye**2
    invr = R / np.sqrt(r2) ** 3
    a2 = a * a
    xy = xe * ye
    shp = xe.shape + (NBFACES,)
    X = np.zeros(shp)
    Y = np.zeros(shp)
    Z = np.zeros(shp)
    if direction == "x":
        ax = a * xe
        b = (a2 + ye * ye) * invr
        X[..., 0], Y[..., 0], Z[..., 0] = -ax * invr, b, -xy * invr
        X[..., 1], Y[..., 1], Z[..., 1] = -(a2 + ye * ye) * invr, -ax * invr, -xy * invr
        X[..., 2], Y[..., 2], Z[..., 2] = ax * invr, -(a2 + ye * ye) * invr, -xy * invr
        X[..., 3], Y[..., 3], Z[..., 3] = b, ax * invr, -xy * invr
        X[..., 4], Y[..., 4], Z[..., 4] = xy * invr, b, -ax * invr
        X[..., 5], Y[..., 5], Z[..., 5] = -xy * invr, b, ax * invr
        ang = np.meshgrid(x, y, indexing="ij")[0]
    else:
        ay = a * ye
        b = (a2 + xe * xe) * invr
        X[..., 0], Y[..., 0], Z[..., 0] = -ay * invr, -xy * invr, b
        X[..., 1], Y[..., 1], Z[..., 1] = xy * invr, -ay * invr, b
        X[..., 2], Y[..., 2], Z[..., 2] = ay * invr, xy * invr, b
        X[..., 3], Y[..., 3], Z[..., 3] = -xy * invr, ay * invr, b
        X[..., 4], Y[..., 4], Z[..., 4] = -(a2 + xe * xe) * invr, -xy * invr, -ay * invr
        X[..., 5], Y[..., 5], Z[..., 5] = (a2 + xe * xe) * invr, -xy * invr, ay * invr
        ang = np.meshgrid(x, y, indexing="ij")[1]
    c = np.cos(ang)
    c2 = c * c
    for p in range(NBFACES):
        X[..., p] = a * X[..., p] / c2
        Y[..., p] = a * Y[..., p] / c2
        Z[..., p] = a * Z[..., p] / c2
    return X, Y, Z


def _geo_unit(lon, lat):
    """Geographic unit vectors e_lon, e_lat (sphgeo.py:72-88)."""
    elon = (-np.sin(lon), np.cos(lon), np.zeros_like(lon))
    elat = (-np.sin(lat) * np.cos(lon), -np.sin(lat) * np.sin(lon), np.cos(lat))
    return elon, elat


class PointSet:
    """One family of grid points (centres pc, x-edges pu or y-edges pv) and its vectors."""

    def __init__(self, x, y):
        self.X, self.Y, self.Z, self.lon, self.lat = equiangular_points(x, y)
        ex = _tangent(x, y, "x")
        ey = _tangent(x, y, "y")
        # metric tensor sqrt(|ex|^2 |ey|^2 - (ex.ey)^2) on panel 0, copied to all panels
        # (cs_datastruct.py:407-446)
        dot = ex[0][..., 0] * ey[0][..., 0] + ex[1][..., 0] * ey[1][..., 0] + ex[2][..., 0] * ey[2][..., 0]
        nx = ex[0][..., 0] ** 2 + ex[1][..., 0] ** 2 + ex[2][..., 0] ** 2
        ny = ey[0][..., 0] ** 2 + ey[1][..., 0] ** 2 + ey[2][..., 0] ** 2
        g0 = np.sqrt(-dot**2 + nx * ny)
        self.metric = np.repeat(g0[..., None], NBFACES, axis=2)
        # lat-lon <-> contravariant coefficients (cs_datastruct.py:456-493)
        elon, elat = _geo_unit(self.lon, self.lat)
        self.ex_elon = ex[0] * elon[0] + ex[1] * elon[1] + ex[2] * elon[2]
        self.ex_elat = ex[0] * elat[0] + ex[1] * elat[1] + ex[2] * elat[2]
        self.ey_elon = ey[0] * elon[0] + ey[1] * elon[1] + ey[2] * elon[2]
        self.ey_elat = ey[0] * elat[0] + ey[1] * elat[1] + ey[2] * elat[2]
        self.det = self.ex_elon * self.ey_elat - self.ey_elon * self.ex_elat


class CubedSphere:
    """Equiangular cubed sphere with N cells per panel edge and 4 ghost layers."""

    def __init__(self, N):
        if N < 8:
            raise ValueError("N must be at least 8")
        self.N = N
        self.R = 1.0
        self.projection = "gnomonic_equiangular"
        self.ngl, self.ngr, self.ng = NGL, NGR, NG
        self.i0, self.iend = NGL, NGL + N
        self.j0, self.jend = NGL, NGL + N
        a = np.pi / 4.0
        self.a = a
        dx = (2 * a) / N
        dy = (2 * a) / N
        self.dx, self.dy = dx, dy
        # 1-D angular coordinates (cs_datastruct.py:240-241, 272-273, 299-300, 324-325)
        self.x_edges = np.linspace(-a - NGL * dx, a + NGR * dx, N + 1 + NG)
        self.y_edges = np.linspace(-a - NGL * dx, a + NGR * dy, N + 1 + NG)
        self.x_centers = np.linspace(-a + dx / 2.0 - NGL * dx, a - dx / 2.0 + NGR * dx, N + NG)
        self.y_centers = np.linspace(-a + dy / 2.0 - NGL * dy, a - dy / 2.0 + NGR * dy, N + NG)
        self.pc = PointSet(self.x_centers, self.y_centers)
        self.pu = PointSet(self.x_edges, self.y_centers)
        self.pv = PointSet(self.x_centers, self.y_edges)
        self.metric_tensor_pc = self.pc.metric
        self.metric_tensor_pu = self.pu.metric
        self.metric_tensor_pv = self.pv.metric

    @property
    def interior(self):
        return (slice(self.i0, self.iend), slice(self.j0, self.jend), slice(None))
