"""Initial conditions, exact solutions and winds (oracle restatement).

Reference cases (advection_ic.py): ICs ``ic`` 1-4 (qexact_adv, :215-281) and winds
``vf`` 1-4 (velocity_adv, :287-313), in the reference's non-dimensional units
(unit sphere, one revolution / period T = 5).

Benchmark extensions (not in the reference; parameterised forms of the same families):
* ``WindSpec('solid', alpha=, u0=)``      -- solid-body rotation about an axis tilted by alpha
* ``WindSpec('deform', k=, T=)``          -- Nair & Lauritzen (2010) case 4 with free k
* ``WindSpec('solid_div', alpha=, u0=, eps=)`` -- solid body + eps*u0 divergent perturbation
* ``ICSpec('hill', lon=, lat=, b0=)``       -- Gaussian hill exp(-b0 |x - xc|^2), advected
                                             by the solid-body rotation for its exact solution
* ``ICSpec('bells')`` / ``ICSpec('smooth_bells')`` -- cosine bells of radius 1/2
"""
import math

import numpy as np

from .grid import sph2cart

PI = math.pi
RAD2DEG = 180.0 / PI
DEG2RAD = 1.0 / RAD2DEG


def qexact_ref(lon, lat, t, ic, vf):
    """advection_ic.py:215-281."""
    if ic == 1:
        return np.ones(np.shape(lon))
    if ic == 2:
        if vf == 1:
            alpha = -45.0 * DEG2RAD
            u0 = 2.0 * PI / 5.0
            wt = -u0 * t
            cosa = np.cos(alpha)
            cos2a = cosa * cosa
            sina = np.sin(alpha)
            sin2a = sina * sina
            coswt = np.cos(wt)
            sinwt = np.sin(wt)
            X, Y, Z = sph2cart(lon, lat)
            rX = (coswt * cos2a + sin2a) * X - sinwt * cosa * Y + (coswt * cosa * sina - cosa * sina) * Z
            rY = sinwt * cosa * X + coswt * Y + sina * sinwt * Z
            rZ = (coswt * sina * cosa - sina * cosa) * X - sinwt * sina * Y + (coswt * sin2a + cos2a) * Z
            X0, Y0, Z0 = sph2cart(PI / 4.0, PI / 6.0)
            return np.exp(-10.0 * ((rX - X0) ** 2 + (rY - Y0) ** 2 + (rZ - Z0) ** 2))
        X, Y, Z = sph2cart(lon, lat)
        X0, Y0, Z0 = sph2cart(0.0, 0.0)
        return np.exp(-10.0 * ((X - X0) ** 2 + (Y - Y0) ** 2 + (Z - Z0) ** 2))
    if ic == 3:
        X, Y, Z = sph2cart(lon, lat)
        if vf == 1:
            c1, c2 = (0, PI / 3.0), (0, -PI / 3.0)
        else:
            c1, c2 = (-PI / 6.0, 0), (PI / 6.0, 0)
        X1, Y1, Z1 = sph2cart(*c1)
        X2, Y2, Z2 = sph2cart(*c2)
        return (np.exp(-5.0 * ((X - X1) ** 2 + (Y - Y1) ** 2 + (Z - Z1) ** 2))
                + np.exp(-5.0 * ((X - X2) ** 2 + (Y - Y2) ** 2 + (Z - Z2) ** 2)))
    if ic == 4:
        alpha = -45.0 * DEG2RAD
        f = -np.cos(lon) * np.cos(lat) * np.sin(alpha) + np.sin(lat) * np.cos(alpha)
        return 1.0 - f * f
    raise ValueError("invalid initial condition %r" % ic)


def velocity_ref(lon, lat, t, vf):
    """advection_ic.py:287-313 (lat-lon wind components)."""
    sin, cos = np.sin, np.cos
    if vf == 1:
        alpha = -45.0 * DEG2RAD
        u0 = 2.0 * PI / 5.0
        ulon = u0 * (cos(lat) * cos(alpha) + sin(lat) * cos(lon) * sin(alpha))
        vlat = -u0 * sin(lon) * sin(alpha)
    elif vf == 2:
        Tp, k = 5.0, 2.0
        lonp = lon - 2 * PI * t / Tp
        ulon = k * (sin((lonp + PI)) ** 2) * (sin(2.0 * lat)) * (cos(PI * t / Tp)) + 2.0 * PI * cos(lat) / Tp
        vlat = k * (sin(2 * (lonp + PI))) * (cos(lat)) * (cos(PI * t / Tp))
    elif vf == 3:
        Tp, k = 5.0, 1.0
        ulon = -k * (sin((lon + PI) / 2.0) ** 2) * (sin(2.0 * lat)) * (cos(lat) ** 2) * (cos(PI * t / Tp))
        vlat = (k / 2.0) * (sin((lon + PI))) * (cos(lat) ** 3) * (cos(PI * t / Tp))
    elif vf == 4:
        m = n = 1
        ulon = -m * (sin(lon) * sin(m * lon) * cos(n * lat) ** 3)
        vlat = -4 * n * (cos(n * lat) ** 3) * sin(n * lat) * cos(m * lon) * sin(lon)
    else:
        raise ValueError("invalid vector field %r" % vf)
    return ulon, vlat


class WindSpec:
    """Benchmark wind (see module docstring).  ``time_dependent`` mirrors the reference's vf>=2."""

    def __init__(self, kind, **kw):
        self.kind = kind
        self.alpha = kw.get("alpha", -PI / 4.0)
        self.u0 = kw.get("u0", 2.0 * PI / 5.0)
        self.k = kw.get("k", 2.0)
        self.T = kw.get("T", 5.0)
        self.eps = kw.get("eps", 0.3)
        if kind not in ("solid", "deform", "solid_div"):
            raise ValueError(kind)

    @property
    def time_dependent(self):
        return self.kind == "deform"

    def __call__(self, lon, lat, t):
        sin, cos = np.sin, np.cos
        if self.kind in ("solid", "solid_div"):
            a, u0 = self.alpha, self.u0
            ulon = u0 * (cos(lat) * cos(a) + sin(lat) * cos(lon) * sin(a))
            vlat = -u0 * sin(lon) * sin(a)
            if self.kind == "solid_div":
                e = self.eps * u0
                ulon = ulon + e * sin(lon) ** 2 * cos(lat)
                vlat = vlat + e * sin(2.0 * lon) * cos(lat)
            return ulon, vlat
        Tp, k = self.T, self.k
        lonp = lon - 2 * PI * t / Tp
        ulon = k * sin(lonp + PI) ** 2 * sin(2.0 * lat) * cos(PI * t / Tp) + 2.0 * PI * cos(lat) / Tp
        vlat = k * sin(2 * (lonp + PI)) * cos(lat) * cos(PI * t / Tp)
        return ulon, vlat


def _rotate(X, Y, Z, axis, angle):
    """Rodrigues rotation of points (X, Y, Z) about the unit vector ``axis``."""
    ax, ay, az = axis
    c, s = math.cos(angle), math.sin(angle)
    dot = ax * X + ay * Y + az * Z
    cx = ay * Z - az * Y
    cy = az * X - ax * Z
    cz = ax * Y - ay * X
    return (X * c + cx * s + ax * dot * (1 - c),
            Y * c + cy * s + ay * dot * (1 - c),
            Z * c + cz * s + az * dot * (1 - c))


class ICSpec:
    """Benchmark initial condition (see module docstring)."""

    def __init__(self, kind, **kw):
        self.kind = kind
        self.lon = kw.get("lon", 0.0)
        self.lat = kw.get("lat", 0.0)
        self.b0 = kw.get("b0", 5.0)
        if kind not in ("hill", "bells", "smooth_bells"):
            raise ValueError(kind)

    def __call__(self, lon, lat, t=0.0, wind=None):
        X, Y, Z = sph2cart(lon, lat)
        if t != 0.0 and wind is not None and wind.kind == "solid":
            # solid-body rotation: rotation axis of u = u0 (cos a e_z-ish) ; exact solution
            # is the initial field rotated backwards by angle u0 t about that axis
            a = wind.alpha
            axis = (-math.sin(a), 0.0, math.cos(a))
            X, Y, Z = _rotate(X, Y, Z, axis, -wind.u0 * t)
        if self.kind == "hill":
            X0, Y0, Z0 = sph2cart(self.lon, self.lat)
            return np.exp(-self.b0 * ((X - X0) ** 2 + (Y - Y0) ** 2 + (Z - Z0) ** 2))
        lon2, lat2 = np.arctan2(Y, X), np.arcsin(np.clip(Z, -1.0, 1.0))
        r = 0.5
        h = np.zeros(np.shape(lon))
        for lc in (5.0 * PI / 6.0, 7.0 * PI / 6.0):
            d = np.arccos(np.clip(np.sin(lat2) * 0.0 + np.cos(lat2) * np.cos(lon2 - lc), -1.0, 1.0))
            h = h + np.where(d < r, 0.5 * (1.0 + np.cos(PI * d / r)), 0.0)
        if self.kind == "bells":
            return 0.1 + 0.9 * h
        return 0.95 + 0.05 * h
