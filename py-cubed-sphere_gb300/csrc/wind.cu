// Winds (FP64, shared by every tracer of a plan).
//
//  wind_initial / wind_update -- analytic winds on the interior edges -> contravariant
//                   (advection_vars.py:38-53 at t = 0; update_adv, advection_timestep.py:48-75)
//  wind_halo     -- ET-DG: edge->centre cubic band, contravariant->lat-lon, Lagrange ghost
//                   fill of the centre winds, centre->ghost-edge cubic, lat-lon->contravariant
//                   (interpolation.py:347-532).  ET-S72/ET-PL07 with RK2: copy of the edge
//                   winds one inside the neighbour (edges_treatment.py:305-347).
//  wind_average  -- departure-point winds (averaged_velocity.py:14-62)
//  wind_cfl      -- simulation.CFL (advection_vars.py:89-98)
//
// Compiled without FMA contraction so the arithmetic order of the reference is kept.
#include <cmath>

#include "cases.cuh"
#include "common.cuh"
#include "internal.h"

namespace csadv {

struct WindParams {
    int vf;
    double prm[4];
};

// analytic winds at interior edges at time t, converted to contravariant components
__global__ void k_wind_interior(Grid g, double *u, double *v, WindParams wp, double t) {
    const Dims d = g.d;
    const int N = d.N;
    long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    long long per = (long long)(N + 1) * N;
    if (tid >= 2 * NFACE * per) return;
    int which = (int)(tid / (NFACE * per));
    long long r = tid % (NFACE * per);
    int p = (int)(r / per);
    int a = (int)((r % per) / N), b = (int)(r % N);
    if (which == 0) {  // x-edge (pu): i in [i0, iend], j in [j0, jend)
        int i = d.i0 + a, j = d.i0 + b;
        long long o = at(d, p, i, j);
        double ulon, vlat;
        wind_latlon(wp.vf, wp.prm, g.lon_pu[o], g.lat_pu[o], t, ulon, vlat);
        u[o] = (g.cu[3][o] * ulon - g.cu[2][o] * vlat) / g.cu[4][o];
    } else {  // y-edge (pv): i in [i0, iend), j in [j0, jend]
        int i = d.i0 + b, j = d.i0 + a;
        long long o = at(d, p, i, j);
        double ulon, vlat;
        wind_latlon(wp.vf, wp.prm, g.lon_pv[o], g.lat_pv[o], t, ulon, vlat);
        v[o] = (-g.cv[1][o] * ulon + g.cv[0][o] * vlat) / g.cv[4][o];
    }
}

// ---------------------------------------------------------------- time-dependent winds
// The reference re-evaluates the analytic wind on every interior edge each step
// (update_adv, advection_timestep.py:55-58), about ten FP64 transcendental calls per
// edge.  Here the parts that do not depend on t are evaluated once per plan, together
// with the lat-lon -> contravariant factors, so a step costs ~15 FP64 operations per
// edge:
//   vf 2 / deformational:  u_lat-lon = k cos(pi t/T) sin^2(lon - 2 pi t/T) sin(2 lat) + 2 pi cos(lat) / T
//                          v_lat-lon = k cos(pi t/T) sin(2 (lon - 2 pi t/T)) cos(lat)
//                          with sin / cos of (lon - w t) from the angle-difference identities
//   vf 3:                  separable, u = cos(pi t/T) * w0(edge)
//   vf 4:                  constant in time, u = w0(edge)
// Results agree with the reference's direct evaluation to a few ulp.
struct WindTables {
    int kind;             // 1: deformational (6 coefficients per edge), 2: separable / constant (1)
    const double *c[6];   // per-edge coefficient planes (x-edges and y-edges interleaved: [set][coef])
};

// per-edge coefficients (time-independent parts) of the wind at the x-edges (set 0)
// and y-edges (set 1): deformational -> {sin lon, cos lon, sin 2lat, cos lat, a, b} with
// contravariant = a * u_ll + b * v_ll; separable/constant -> {contravariant at t = 0}
__global__ void k_wind_tables(Grid g, WindParams wp, double *tab0, double *tab1, int ncoef) {
    const Dims d = g.d;
    const int N = d.N;
    long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    long long per = (long long)(N + 1) * N;
    if (tid >= 2 * NFACE * per) return;
    int which = (int)(tid / (NFACE * per));
    long long r = tid % (NFACE * per);
    int p = (int)(r / per);
    int a = (int)((r % per) / N), b = (int)(r % N);
    int i = which == 0 ? d.i0 + a : d.i0 + b;
    int j = which == 0 ? d.i0 + b : d.i0 + a;
    long long o = at(d, p, i, j);
    const double *lon = which == 0 ? g.lon_pu : g.lon_pv, *lat = which == 0 ? g.lat_pu : g.lat_pv;
    const double *const *cf = which == 0 ? g.cu : g.cv;
    double *tab = which == 0 ? tab0 : tab1;
    // contravariant = a * ulon + b * vlat  (sphgeo.py:120-125)
    double ca = which == 0 ? cf[3][o] / cf[4][o] : -cf[1][o] / cf[4][o];
    double cb = which == 0 ? -cf[2][o] / cf[4][o] : cf[0][o] / cf[4][o];
    if (ncoef == 6) {
        double L = lon[o], P = lat[o];
        tab[0 * d.field + o] = sin(L);
        tab[1 * d.field + o] = cos(L);
        tab[2 * d.field + o] = sin(2.0 * P);
        tab[3 * d.field + o] = cos(P);
        tab[4 * d.field + o] = ca;
        tab[5 * d.field + o] = cb;
    } else {
        double ulon, vlat;
        wind_latlon(wp.vf, wp.prm, lon[o], lat[o], 0.0, ulon, vlat);  // vf 3 at t = 0 (cos 0 = 1); vf 4
        tab[o] = ca * ulon + cb * vlat;
    }
}

struct Clock {
    long long k;  // completed steps
    double dt;
    double t;     // time of the wind held in the "current" arrays
};

__global__ void k_clock_tick(Clock *c) {
    c->k += 1;
    c->t = (double)c->k * c->dt;
}
__global__ void k_clock_set(Clock *c, long long k, double t) {
    c->k = k;
    c->t = t;
}

// update_adv: old <- current everywhere; current <- wind(t) on interior edges; non-interior
// entries become 0 for ET-S72/ET-PL07 and keep the wind-halo values for ET-DG (the
// reference recomputes them from unchanged lat-lon values)
__global__ void k_wind_update(Dims d, double *u, double *v, double *uo, double *vo, const double *__restrict__ tu,
                              const double *__restrict__ tv, int kind, WindParams wp, const Clock *clk,
                              int zero_ghosts) {
    __shared__ double sc[4];
    if (threadIdx.x == 0) {
        const double t = clk->t;
        if (kind == 1) {
            const double Tp = wp.vf == 2 ? 5.0 : wp.prm[1], k = wp.vf == 2 ? 2.0 : wp.prm[0];
            double w = 2 * PI * t / Tp;
            sc[0] = k * cos(PI * t / Tp);
            sc[1] = sin(w);
            sc[2] = cos(w);
            sc[3] = 2.0 * PI / Tp;
        } else {
            sc[0] = wp.vf == 3 ? cos(PI * t / 5.0) : 1.0;
        }
    }
    __syncthreads();
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y, p = blockIdx.z;
    if (j >= d.pitch) return;
    const long long tid = at(d, p, i, j);
    uo[tid] = u[tid];
    vo[tid] = v[tid];
    const bool iu = (i >= d.i0 && i <= d.iend && j >= d.i0 && j < d.iend);
    const bool iv = (i >= d.i0 && i < d.iend && j >= d.i0 && j <= d.iend);
    for (int which = 0; which < 2; ++which) {
        const bool in = which == 0 ? iu : iv;
        double *out = which == 0 ? u : v;
        const double *tab = which == 0 ? tu : tv;
        if (in) {
            if (kind == 1) {
                double sl = tab[tid], cl = tab[d.field + tid], s2p = tab[2 * d.field + tid], cp = tab[3 * d.field + tid];
                double ca = tab[4 * d.field + tid], cb = tab[5 * d.field + tid];
                double s = sl * sc[2] - cl * sc[1];  // sin(lon - w t)
                double c = cl * sc[2] + sl * sc[1];  // cos(lon - w t)
                double ulon = sc[0] * (s * s) * s2p + sc[3] * cp;
                double vlat = sc[0] * (2.0 * s * c) * cp;
                out[tid] = ca * ulon + cb * vlat;
            } else {
                out[tid] = sc[0] * tab[tid];
            }
        } else if (zero_ghosts) {
            out[tid] = 0.0;
        }
    }
}

static dim3 plane_grid(const Dims &d, int bx) { return dim3(ceil_div(d.pitch, bx), d.n + 1, NFACE); }

// ET-DG wind halo, part 1: cubic edge->centre interpolation of the contravariant wind in
// the band of 4 cells along each panel boundary, then contravariant->lat-lon there
// (interpolation.py:356-425).
__global__ void k_wind_band(Grid g, const double *__restrict__ U, const double *__restrict__ V, double *ulon,
                            double *vlat) {
    const Dims d = g.d;
    const int N = d.N, i0 = d.i0, iend = d.iend;
    long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= (long long)NFACE * N * N) return;
    int p = (int)(tid / ((long long)N * N));
    int i = i0 + (int)((tid / N) % N), j = i0 + (int)(tid % N);
    bool wband = i < i0 + NG, eband = i >= iend - NG, sband = j < i0 + NG, nband = j >= iend - NG;
    if (!(wband || eband || sband || nband)) return;
    const double a1 = 5.0 / 16.0, a2 = 15.0 / 16.0, a3 = -5.0 / 16.0, a4 = 1.0 / 16.0;
    const double b1 = -1.0 / 16.0, b2 = 9.0 / 16.0, b3 = 9.0 / 16.0, b4 = -1.0 / 16.0;
    auto Ux = [&](int ii) { return U[at(d, p, ii, j)]; };
    auto Vy = [&](int jj) { return V[at(d, p, i, jj)]; };
    double uc, vc;
    // x component: west/east bands along whole interior columns, else south/north bands
    if (i == i0) uc = a1 * Ux(i0) + a2 * Ux(i0 + 1) + a3 * Ux(i0 + 2) + a4 * Ux(i0 + 3);
    else if (i == iend - 1) uc = a4 * Ux(iend - 3) + a3 * Ux(iend - 2) + a2 * Ux(iend - 1) + a1 * Ux(iend);
    else if (wband) uc = b1 * Ux(i - 1) + b2 * Ux(i) + b3 * Ux(i + 1) + b4 * Ux(i + 2);
    else if (eband) uc = b4 * Ux(i - 1) + b3 * Ux(i) + b2 * Ux(i + 1) + b1 * Ux(i + 2);
    else uc = b1 * Ux(i - 1) + b2 * Ux(i) + b3 * Ux(i + 1) + b4 * Ux(i + 2);
    if (j == i0) vc = a1 * Vy(i0) + a2 * Vy(i0 + 1) + a3 * Vy(i0 + 2) + a4 * Vy(i0 + 3);
    else if (j == iend - 1) vc = a4 * Vy(iend - 3) + a3 * Vy(iend - 2) + a2 * Vy(iend - 1) + a1 * Vy(iend);
    else if (sband) vc = b1 * Vy(j - 1) + b2 * Vy(j) + b3 * Vy(j + 1) + b4 * Vy(j + 2);
    else if (nband) vc = b4 * Vy(j - 1) + b3 * Vy(j) + b2 * Vy(j + 1) + b1 * Vy(j + 2);
    else vc = b1 * Vy(j - 1) + b2 * Vy(j) + b3 * Vy(j + 1) + b4 * Vy(j + 2);
    long long o = at(d, p, i, j);
    ulon[o] = g.cc[0][o] * uc + g.cc[2][o] * vc;
    vlat[o] = g.cc[1][o] * uc + g.cc[3][o] * vc;
}

// ET-DG wind halo, part 3: centre->edge cubic interpolation of the lat-lon wind at the
// ghost edges, then lat-lon->contravariant (interpolation.py:436-532)
__global__ void k_wind_ghost_edges(Grid g, const double *__restrict__ ul, const double *__restrict__ vl, double *U,
                                   double *V) {
    const Dims d = g.d;
    const int n = d.n, i0 = d.i0, iend = d.iend, N = d.N;
    // x-edges: (a) rows [i0, iend] x ghost columns (8 columns); (b) rows i0-1, iend+1 x all n columns
    // y-edges: (a) ghost rows (8) x columns [j0, jend]; (b) columns j0-1, jend+1 x all n rows
    long long na = (long long)(N + 1) * 2 * NG, nb = 2LL * n;
    long long per = na + nb;
    long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= 2 * NFACE * per) return;
    int which = (int)(tid / (NFACE * per));
    long long r = tid % (NFACE * per);
    int p = (int)(r / per);
    long long q = r % per;
    const double c1 = 9.0 / 16.0, c2 = -1.0 / 16.0;
    auto C = [&](const double *f, int i, int j) { return f[at(d, p, i, j)]; };
    int i, j;
    double u, v;
    if (which == 0) {
        if (q < na) {
            i = i0 + (int)(q / (2 * NG));
            int c = (int)(q % (2 * NG));
            j = c < NG ? c : iend + (c - NG);
            u = c1 * (C(ul, i, j) + C(ul, i - 1, j)) + c2 * (C(ul, i + 1, j) + C(ul, i - 2, j));
            v = c1 * (C(vl, i, j) + C(vl, i - 1, j)) + c2 * (C(vl, i + 1, j) + C(vl, i - 2, j));
        } else {
            q -= na;
            j = (int)(q % n);
            if (q < n) {
                i = i0 - 1;
                u = c1 * (C(ul, i0 - 2, j) + C(ul, i0 - 1, j)) + c2 * (C(ul, i0, j) + C(ul, i0 - 3, j));
                v = c1 * (C(vl, i0 - 2, j) + C(vl, i0 - 1, j)) + c2 * (C(vl, i0, j) + C(vl, i0 - 3, j));
            } else {
                i = iend + 1;
                u = c1 * (C(ul, iend, j) + C(ul, iend + 1, j)) + c2 * (C(ul, iend - 1, j) + C(ul, iend + 2, j));
                v = c1 * (C(vl, iend, j) + C(vl, iend + 1, j)) + c2 * (C(vl, iend - 1, j) + C(vl, iend + 2, j));
            }
        }
        long long o = at(d, p, i, j);
        U[o] = (g.cu[3][o] * u - g.cu[2][o] * v) / g.cu[4][o];
    } else {
        if (q < na) {
            j = i0 + (int)(q / (2 * NG));
            int c = (int)(q % (2 * NG));
            i = c < NG ? c : iend + (c - NG);
            u = c1 * (C(ul, i, j) + C(ul, i, j - 1)) + c2 * (C(ul, i, j + 1) + C(ul, i, j - 2));
            v = c1 * (C(vl, i, j) + C(vl, i, j - 1)) + c2 * (C(vl, i, j + 1) + C(vl, i, j - 2));
        } else {
            q -= na;
            i = (int)(q % n);
            if (q < n) {
                j = i0 - 1;
                u = c1 * (C(ul, i, i0 - 2) + C(ul, i, i0 - 1)) + c2 * (C(ul, i, i0) + C(ul, i, i0 - 3));
                v = c1 * (C(vl, i, i0 - 2) + C(vl, i, i0 - 1)) + c2 * (C(vl, i, i0) + C(vl, i, i0 - 3));
            } else {
                j = iend + 1;
                u = c1 * (C(ul, i, iend) + C(ul, i, iend + 1)) + c2 * (C(ul, i, iend - 1) + C(ul, i, iend + 2));
                v = c1 * (C(vl, i, iend) + C(vl, i, iend + 1)) + c2 * (C(vl, i, iend - 1) + C(vl, i, iend + 2));
            }
        }
        long long o = at(d, p, i, j);
        V[o] = (-g.cv[1][o] * u + g.cv[0][o] * v) / g.cv[4][o];
    }
}

// ET-S72/ET-PL07 + RK2: the edge one beyond each cube edge takes the neighbour's edge one
// inside, with the sign between the panels' coordinate directions
__global__ void k_wind_adjacent(Dims d, double *U, double *V) {
    const int N = d.N;
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= NFACE * 4 * N) return;
    int k = d.i0 + tid % N;
    int s = (tid / N) % 4;
    int p = tid / (4 * N);
    const Conn c = c_conn[p][s];
    int kk = c.rev ? d.n - 1 - k : k;
    double val;
    switch (c.qs) {
        case SIDE_W: val = U[at(d, c.q, d.i0 + 1, kk)]; break;
        case SIDE_E: val = U[at(d, c.q, d.iend - 1, kk)]; break;
        case SIDE_S: val = V[at(d, c.q, kk, d.i0 + 1)]; break;
        default: val = V[at(d, c.q, kk, d.iend - 1)]; break;
    }
    if (vec_sign(s, c.qs) < 0) val = -val;
    switch (s) {
        case SIDE_E: U[at(d, p, d.iend + 1, k)] = val; break;
        case SIDE_W: U[at(d, p, d.i0 - 1, k)] = val; break;
        case SIDE_N: V[at(d, p, k, d.iend + 1)] = val; break;
        default: V[at(d, p, k, d.i0 - 1)] = val; break;
    }
}

// departure-point winds (averaged_velocity.py:14-62)
// RK2 average at edge (i, j) along direction dir (0: x, 1: y): the wind extrapolated to
// n+1/2, interpolated linearly at the departure point on the upwind side
__device__ __forceinline__ double rk2_average(const double *__restrict__ U, const double *__restrict__ Uo,
                                              const Dims &d, int p, int i, int j, int dir, double dto2, double dx) {
    auto ui = [&](int k) {
        long long o = dir == 0 ? at(d, p, k, j) : at(d, p, i, k);
        return 1.5 * U[o] - 0.5 * Uo[o];
    };
    const int e = dir == 0 ? i : j;
    const double u = U[at(d, p, i, j)];
    const double a = u * dto2 / dx;
    return (u >= 0) ? (1.0 - a) * ui(e) + a * ui(e - 1) : -a * ui(e + 1) + (1.0 + a) * ui(e);
}

__global__ void k_wind_average(Dims d, const double *__restrict__ U, const double *__restrict__ Uo, double *Ua,
                               const double *__restrict__ V, const double *__restrict__ Vo, double *Va, int rk2,
                               double dto2, double dx) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y, p = blockIdx.z;
    if (j >= d.pitch) return;
    const long long tid = at(d, p, i, j);
    if (!rk2) {
        Ua[tid] = U[tid];
        Va[tid] = V[tid];
        return;
    }
    if (j < d.n && i >= d.i0 && i <= d.iend) Ua[tid] = rk2_average(U, Uo, d, p, i, j, 0, dto2, dx);
    if (i < d.n && j >= d.i0 && j <= d.iend) Va[tid] = rk2_average(V, Vo, d, p, i, j, 1, dto2, dx);
}

// departure-point wind and upwind flag of the fused engine in one pass: the wind in the
// state's precision, and one bit per edge (warp ballot over 32 consecutive columns)
template <class real>
__global__ void k_wind_avgprep(Dims d, const double *__restrict__ U, const double *__restrict__ Uo,
                               const double *__restrict__ V, const double *__restrict__ Vo, real *ua, real *va,
                               uint32_t *ubits, uint32_t *vbits, int wpitch, int rk2, double dto2, double dx) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y, p = blockIdx.z;
    const bool ok = j < d.pitch;
    double u = 0.0, v = 0.0, au = 0.0, av = 0.0;
    long long tid = 0;
    if (ok) {
        tid = at(d, p, i, j);
        u = U[tid];
        v = V[tid];
        au = u;
        av = v;
        if (rk2) {
            au = (j < d.n && i >= d.i0 && i <= d.iend) ? rk2_average(U, Uo, d, p, i, j, 0, dto2, dx) : 0.0;
            av = (i < d.n && j >= d.i0 && j <= d.iend) ? rk2_average(V, Vo, d, p, i, j, 1, dto2, dx) : 0.0;
        }
        ua[tid] = (real)au;
        va[tid] = (real)av;
    }
    unsigned bu = __ballot_sync(0xffffffffu, ok && u >= 0.0);
    unsigned bv = __ballot_sync(0xffffffffu, ok && v >= 0.0);
    if (ok && (threadIdx.x & 31) == 0) {
        long long w = ((long long)p * (d.n + 1) + i) * wpitch + (j >> 5);
        ubits[w] = bu;
        vbits[w] = bv;
    }
}

// max over x-edges [i0, iend] x all columns of u*dt/dx (signed), same for y; one block
__global__ void k_wind_cfl(Dims d, const double *__restrict__ U, const double *__restrict__ V, double dt, double dx,
                           double *out) {
    __shared__ double rx[512], ry[512];
    double mx = -INFINITY, my = -INFINITY;
    long long cnt = (long long)NFACE * (d.N + 1) * d.n;
    for (long long t = threadIdx.x; t < cnt; t += blockDim.x) {
        int p = (int)(t / ((long long)(d.N + 1) * d.n));
        int a = (int)((t / d.n) % (d.N + 1)), b = (int)(t % d.n);
        mx = fmax(mx, U[at(d, p, d.i0 + a, b)] * dt / dx);
        my = fmax(my, V[at(d, p, b, d.i0 + a)] * dt / dx);
    }
    rx[threadIdx.x] = mx;
    ry[threadIdx.x] = my;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            rx[threadIdx.x] = fmax(rx[threadIdx.x], rx[threadIdx.x + s]);
            ry[threadIdx.x] = fmax(ry[threadIdx.x], ry[threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = rx[0];
        out[1] = ry[0];
    }
}

static WindParams wparams(const Options &o) {
    WindParams wp;
    wp.vf = o.vf;
    for (int c = 0; c < 4; ++c) wp.prm[c] = o.wp[c];
    return wp;
}

// Allocate and fill the time-independent wind coefficients and the device clock.
int wind_setup(const Options &o, const Grid &g, Winds &w, DeviceArena &mem, double dt, cudaStream_t st) {
    const Dims d = g.d;
    Clock *clk = mem.alloc<Clock>(1);
    if (!mem.ok()) return CSADV_ERR_OOM;
    w.clock = clk;
    k_clock_set<<<1, 1, 0, st>>>(clk, 0, 0.0);
    Clock h{0, dt, 0.0};
    CSADV_CUDA(cudaMemcpyAsync(clk, &h, sizeof(Clock), cudaMemcpyHostToDevice, st));
    if (!wind_time_dependent(o)) {
        w.tkind = 0;
        return CSADV_OK;
    }
    const bool deform = (o.vf == 2 || o.vf == CSADV_WIND_DEFORM);
    const int nc = deform ? 6 : 1;
    w.tkind = deform ? 1 : 2;
    for (int s2 = 0; s2 < 2; ++s2) {
        w.tab[s2] = mem.alloc<double>(nc * d.field);
        if (!mem.ok()) return CSADV_ERR_OOM;
        CSADV_CUDA(cudaMemsetAsync(w.tab[s2], 0, nc * d.field * sizeof(double), st));
    }
    long long tot = 2LL * NFACE * (d.N + 1) * d.N;
    k_wind_tables<<<ceil_div(tot, 128), 128, 0, st>>>(g, wparams(o), w.tab[0], w.tab[1], nc);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

// Winds of the interior edges at the initial time (advection_vars.py:38-53).
int wind_initial(const Options &o, const Grid &g, Winds &w, cudaStream_t st) {
    const Dims d = g.d;
    if (w.tkind == 0) {
        long long tot = 2LL * NFACE * (d.N + 1) * d.N;
        k_wind_interior<<<ceil_div(tot, 128), 128, 0, st>>>(g, w.u_pu, w.v_pv, wparams(o), 0.0);
    } else {
        k_wind_update<<<plane_grid(d, 128), 128, 0, st>>>(d, w.u_pu, w.v_pv, w.u_old, w.v_old, w.tab[0], w.tab[1],
                                                         w.tkind, wparams(o), (const Clock *)w.clock, 0);
    }
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

// update_adv (advection_timestep.py:48-75).  tick: the clock advances by one step (time
// k*dt computed on the device, so the sequence can be replayed from a CUDA graph);
// otherwise the clock is set to (k, t).
int wind_update(const Options &o, const Grid &g, Winds &w, bool tick, long long k, double t, cudaStream_t st) {
    const Dims d = g.d;
    Clock *clk = (Clock *)w.clock;
    if (tick) k_clock_tick<<<1, 1, 0, st>>>(clk);
    else k_clock_set<<<1, 1, 0, st>>>(clk, k, t);
    if (w.tkind != 0)
        k_wind_update<<<plane_grid(d, 128), 128, 0, st>>>(d, w.u_pu, w.v_pv, w.u_old, w.v_old, w.tab[0], w.tab[1],
                                                         w.tkind, wparams(o), clk, o.et != ET_DG);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

int wind_halo(const Options &o, const Grid &g, Winds &w, cudaStream_t st) {
    const Dims d = g.d;
    if (o.et == ET_DG) {
        long long tot = (long long)NFACE * d.N * d.N;
        k_wind_band<<<ceil_div(tot, 128), 128, 0, st>>>(g, w.u_pu, w.v_pv, w.ulon_pc, w.vlat_pc);
        int rc = launch_halo_dg_tracers<double>(w.ulon_pc, 2, g, nullptr, nullptr, st);  // ulon_pc, vlat_pc
        if (rc) return rc;
        long long per = (long long)(d.N + 1) * 2 * NG + 2LL * d.n;
        tot = 2 * NFACE * per;
        k_wind_ghost_edges<<<ceil_div(tot, 128), 128, 0, st>>>(g, w.ulon_pc, w.vlat_pc, w.u_pu, w.v_pv);
    } else if (o.dp == 2) {
        int tot = NFACE * 4 * d.N;
        k_wind_adjacent<<<ceil_div(tot, 128), 128, 0, st>>>(d, w.u_pu, w.v_pv);
    }
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

int wind_average(const Options &o, const Grid &g, Winds &w, double dt, cudaStream_t st) {
    const Dims d = g.d;
    k_wind_average<<<plane_grid(d, 128), 128, 0, st>>>(d, w.u_pu, w.u_old, w.u_avg, w.v_pv, w.v_old, w.v_avg,
                                                       o.dp == 2, dt * 0.5, g.dx);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

template <class real>
int wind_avgprep(const Options &o, const Grid &g, const Winds &w, double dt, real *ua, real *va, uint32_t *ub,
                 uint32_t *vb, int wpitch, cudaStream_t st) {
    const Dims d = g.d;
    k_wind_avgprep<real><<<plane_grid(d, 128), 128, 0, st>>>(d, w.u_pu, w.u_old, w.v_pv, w.v_old, ua, va, ub, vb,
                                                              wpitch, o.dp == 2, dt * 0.5, g.dx);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}
template int wind_avgprep<double>(const Options &, const Grid &, const Winds &, double, double *, double *, uint32_t *,
                                  uint32_t *, int, cudaStream_t);
template int wind_avgprep<float>(const Options &, const Grid &, const Winds &, double, float *, float *, uint32_t *,
                                 uint32_t *, int, cudaStream_t);

int wind_cfl(const Grid &g, const Winds &w, double dt, double *dev_tmp, double &cfl, cudaStream_t st) {
    k_wind_cfl<<<1, 512, 0, st>>>(g.d, w.u_pu, w.v_pv, dt, g.dx, dev_tmp);
    CSADV_CUDA(cudaGetLastError());
    double h[2];
    CSADV_CUDA(cudaMemcpyAsync(h, dev_tmp, sizeof(h), cudaMemcpyDeviceToHost, st));
    CSADV_CUDA(cudaStreamSynchronize(st));
    cfl = fmax(fabs(h[0]), fabs(h[1]));
    return CSADV_OK;
}

}  // namespace csadv
