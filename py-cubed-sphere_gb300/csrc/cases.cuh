// Analytic winds and initial conditions (device, FP64).
//
// Reference cases: velocity_adv (advection_ic.py:287-313) for vf 1-4 and qexact_adv
// (advection_ic.py:215-281) for ic 1-4; the expressions keep the reference's operation
// order.  Benchmark extensions (codes >= 101, see csadv.h) are parameterised members of
// the same families.
#pragma once
#include <cmath>

#include "../../include/csadv.h"

namespace csadv {

constexpr double PI = 3.141592653589793;

__host__ __device__ inline double deg2rad() { return 1.0 / (180.0 / PI); }

__device__ inline void sph2cart(double lon, double lat, double &X, double &Y, double &Z) {
    X = cos(lat) * cos(lon);
    Y = cos(lat) * sin(lon);
    Z = sin(lat);
}

// lat-lon wind (ulon, vlat) of wind code vf at (lon, lat, t); prm = wind parameters
__device__ inline void wind_latlon(int vf, const double *prm, double lon, double lat, double t, double &ulon,
                                   double &vlat) {
    if (vf == 1) {
        const double alpha = -45.0 * deg2rad();
        const double u0 = 2.0 * PI / 5.0;
        ulon = u0 * (cos(lat) * cos(alpha) + sin(lat) * cos(lon) * sin(alpha));
        vlat = -u0 * sin(lon) * sin(alpha);
    } else if (vf == 2 || vf == CSADV_WIND_DEFORM) {
        const double Tp = (vf == 2) ? 5.0 : prm[1];
        const double k = (vf == 2) ? 2.0 : prm[0];
        double lonp = lon - 2 * PI * t / Tp;
        double s = sin((lonp + PI));
        ulon = k * (s * s) * (sin(2.0 * lat)) * (cos(PI * t / Tp)) + 2.0 * PI * cos(lat) / Tp;
        vlat = k * (sin(2 * (lonp + PI))) * (cos(lat)) * (cos(PI * t / Tp));
    } else if (vf == 3) {
        const double Tp = 5.0, k = 1.0;
        double s = sin((lon + PI) / 2.0);
        double c = cos(lat);
        ulon = -k * (s * s) * (sin(2.0 * lat)) * (c * c) * (cos(PI * t / Tp));
        vlat = (k / 2.0) * (sin((lon + PI))) * pow(c, 3.0) * (cos(PI * t / Tp));
    } else if (vf == 4) {
        double c3 = pow(cos(lat), 3.0);
        ulon = -1.0 * (sin(lon) * sin(lon) * c3);
        vlat = -4.0 * c3 * sin(lat) * cos(lon) * sin(lon);
    } else {  // CSADV_WIND_SOLID / CSADV_WIND_SOLID_DIV
        const double a = prm[0], u0 = prm[1];
        ulon = u0 * (cos(lat) * cos(a) + sin(lat) * cos(lon) * sin(a));
        vlat = -u0 * sin(lon) * sin(a);
        if (vf == CSADV_WIND_SOLID_DIV) {
            double e = prm[2] * u0;
            double sl = sin(lon);
            ulon = ulon + e * (sl * sl) * cos(lat);
            vlat = vlat + e * sin(2.0 * lon) * cos(lat);
        }
    }
}

__host__ __device__ inline bool wind_is_time_dependent(int vf) { return (vf >= 2 && vf <= 4) || vf == CSADV_WIND_DEFORM; }

// Rodrigues rotation of (X, Y, Z) about unit axis (ax, ay, az) by angle
__device__ inline void rotate(double &X, double &Y, double &Z, double ax, double ay, double az, double ang) {
    double c = cos(ang), s = sin(ang);
    double dot = ax * X + ay * Y + az * Z;
    double cx = ay * Z - az * Y, cy = az * X - ax * Z, cz = ax * Y - ay * X;
    double X2 = X * c + cx * s + ax * dot * (1 - c);
    double Y2 = Y * c + cy * s + ay * dot * (1 - c);
    double Z2 = Z * c + cz * s + az * dot * (1 - c);
    X = X2; Y = Y2; Z = Z2;
}

__device__ inline double bells(double X, double Y, double Z) {
    double lon = atan2(Y, X), lat = asin(fmin(1.0, fmax(-1.0, Z)));
    const double r = 0.5;
    double h = 0.0;
    const double lc[2] = {5.0 * PI / 6.0, 7.0 * PI / 6.0};
    for (int b = 0; b < 2; ++b) {
        double dd = acos(fmin(1.0, fmax(-1.0, cos(lat) * cos(lon - lc[b]))));
        if (dd < r) h += 0.5 * (1.0 + cos(PI * dd / r));
    }
    return h;
}

// exact solution q(lon, lat, t) of IC code ic advected by wind code vf
// (wprm = wind parameters, iprm = IC parameters)
__device__ inline double qexact(int ic, const double *iprm, int vf, const double *wprm, double lon, double lat,
                                double t) {
    if (ic == 1) return 1.0;
    if (ic == 2) {
        double X, Y, Z;
        sph2cart(lon, lat, X, Y, Z);
        if (vf == 1) {
            const double alpha = -45.0 * deg2rad();
            const double u0 = 2.0 * PI / 5.0;
            double wt = -u0 * t;
            double cosa = cos(alpha), cos2a = cosa * cosa, sina = sin(alpha), sin2a = sina * sina;
            double coswt = cos(wt), sinwt = sin(wt);
            double rX = (coswt * cos2a + sin2a) * X - sinwt * cosa * Y + (coswt * cosa * sina - cosa * sina) * Z;
            double rY = sinwt * cosa * X + coswt * Y + sina * sinwt * Z;
            double rZ = (coswt * sina * cosa - sina * cosa) * X - sinwt * sina * Y + (coswt * sin2a + cos2a) * Z;
            double X0, Y0, Z0;
            sph2cart(PI / 4.0, PI / 6.0, X0, Y0, Z0);
            double a = rX - X0, b = rY - Y0, c = rZ - Z0;
            return exp(-10.0 * ((a * a + b * b) + c * c));
        }
        double X0, Y0, Z0;
        sph2cart(0.0, 0.0, X0, Y0, Z0);
        double a = X - X0, b = Y - Y0, c = Z - Z0;
        return exp(-10.0 * ((a * a + b * b) + c * c));
    }
    if (ic == 3) {
        double X, Y, Z, X1, Y1, Z1, X2, Y2, Z2;
        sph2cart(lon, lat, X, Y, Z);
        if (vf == 1) {
            sph2cart(0.0, PI / 3.0, X1, Y1, Z1);
            sph2cart(0.0, -PI / 3.0, X2, Y2, Z2);
        } else {
            sph2cart(-PI / 6.0, 0.0, X1, Y1, Z1);
            sph2cart(PI / 6.0, 0.0, X2, Y2, Z2);
        }
        double a = X - X1, b = Y - Y1, c = Z - Z1;
        double e = X - X2, f = Y - Y2, g = Z - Z2;
        return exp(-5.0 * ((a * a + b * b) + c * c)) + exp(-5.0 * ((e * e + f * f) + g * g));
    }
    if (ic == 4) {
        const double alpha = -45.0 * deg2rad();
        double f = -cos(lon) * cos(lat) * sin(alpha) + sin(lat) * cos(alpha);
        return 1.0 - f * f;
    }
    double X, Y, Z;
    sph2cart(lon, lat, X, Y, Z);
    if (t != 0.0 && vf == CSADV_WIND_SOLID) {
        // solid-body rotation about (-sin a, 0, cos a) with angular speed u0
        double a = wprm[0];
        rotate(X, Y, Z, -sin(a), 0.0, cos(a), -wprm[1] * t);
    }
    if (ic == CSADV_IC_HILL) {
        double X0, Y0, Z0;
        sph2cart(iprm[0], iprm[1], X0, Y0, Z0);
        double a = X - X0, b = Y - Y0, c = Z - Z0;
        return exp(-iprm[2] * ((a * a + b * b) + c * c));
    }
    double h = bells(X, Y, Z);
    return ic == CSADV_IC_BELLS ? 0.1 + 0.9 * h : 0.95 + 0.05 * h;
}

}  // namespace csadv
