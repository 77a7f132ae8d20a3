// Winds, shared by every tracer of a plan, stored and advanced in the state's precision W
// (float64 for the plain form, float32 for the FP32 form; GB300's FP64 rate makes FP64
// per-edge work as expensive as the whole FP32 tracer step).  Geometry stays FP64.
//
//  wind_initial / wind_update -- analytic winds on the interior edges -> contravariant
//                   (advection_vars.py:38-53 at t = 0; update_adv, advection_timestep.py:48-75)
//  wind_halo     -- ET-DG: edge->centre cubic band, contravariant->lat-lon, Lagrange ghost
//                   fill of the centre winds, centre->ghost-edge cubic, lat-lon->contravariant
//                   (interpolation.py:347-532).  ET-S72/ET-PL07 with RK2: copy of the edge
//                   winds one inside the neighbour (edges_treatment.py:305-347).
//  wind_average  -- departure-point winds (averaged_velocity.py:14-62)
//  wind_avgprep  -- the same, plus upwind bits, for the fused engine
//  wind_cfl      -- simulation.CFL (advection_vars.py:89-98)
//
// Compiled without FMA contraction so the arithmetic order of the reference is kept.
#include <cmath>
#include <cstddef>

#include "cases.cuh"

#include "common.cuh"
#include "internal.h"
#include "tiles.h"

namespace csadv {

struct WindParams {
    int vf;
    double prm[4];
};

// -x for a double by its sign bit (an integer instruction, not one of the FP64 pipe)
__device__ __forceinline__ double neg_bits(double x) {
    return __hiloint2double(__double2hiint(x) ^ (int)0x80000000, __double2loint(x));
}
__device__ __forceinline__ float neg_bits(float x) { return -x; }

// edge record {wind, +-g}: the sign carries the upwind flag (+: wind >= 0), g = |value|
template <class V, class W>
__device__ __forceinline__ V edge_record(W wind, W g, bool up) {
    V r;
    r.x = wind;
    r.y = up ? g : neg_bits(g);
    return r;
}

// Flux coefficients of an edge for the FP64 line-marching kernel.  The upwind PPM flux through an
// edge (flux.py:20-128, with the metric weights of flux.py:28-31),
//   u >= 0:  F = u (q_R + c/2 (q6 - dq) - q6 c^2/3),   u < 0:  F = u (q_L - c/2 (q6 + dq) - q6 c^2/3)
// with dq = q_R - q_L, q6 = 6 mean - 3 (q_R + q_L) (each weighted by the metric at its point for
// MT-0), c = u dt/dx and u the departure-point wind, is linear in the upwind cell's parabola:
//   F = alpha q_R + beta q_L + gamma mean,
//   u >= 0:  alpha = gR u (1-c)^2,  beta = -gL u c (1-c),  gamma = gC u c (3 - 2c)
//   u <  0:  alpha = gR u c (1+c),  beta = gL u (1+c)^2,   gamma = -gC u c (3 + 2c)
// (the weights gL, gR, gC of the upwind cell's left edge, right edge and centre for MT-0; the edge's
// own metric for all three with MT-PL07, whose flux is F g).  Which cell is upwind follows the sign
// of the current wind (flux.py:48-61); u above is the departure-point wind.  The coefficients
// depend on the wind and the metric alone, so they are formed once per edge and step, here,
// instead of once per tracer and pass in the step kernel, where every FP64 operation costs as much
// as 64 FP32 ones on GB300.
template <class W>
struct UpwindMetric {
    const W *ge;                          // edge metric along the line (x: g_pu natural; y: g_pv transposed)
    const typename Vec2<W>::type *gc;     // cell records {g, 1/g} in the same orientation
    int n;                                // rows of the orientation: edges 0..n, cells 0..n-1
    int pl07;                             // MT-PL07: every weight is the edge's metric
};

// the upwind choice of an edge: wind >= 0 (flux.py:48-61), for FP64 on the integer pipe with 32-bit
// operations on the pattern's words (-0 counts as >= 0, as the comparison does)
__device__ __forceinline__ bool wind_up(float u) { return u >= 0.f; }
__device__ __forceinline__ bool wind_up(double u) {
    const int h = __double2hiint(u);
    return h >= 0 || ((h & 0x7fffffff) | __double2loint(u)) == 0;
}

template <class W>
__device__ __forceinline__ void flux_coefs(W u, W g, bool up, W dtdx, const UpwindMetric<W> &um, const Dims &d, int m,
                                           int col, W &al, W &be, W &ga) {
    W gL = g, gR = g, gC = g;
    if (!um.pl07) {  // the upwind cell: m - 1 (wind >= 0) or m, clamped to the plane
        const int cm = up ? (m > 0 ? m - 1 : 0) : (m < um.n ? m : um.n - 1);
        const int el = up ? (m > 0 ? m - 1 : 0) : m, er = up ? m : (m < um.n ? m + 1 : um.n);
        gL = um.ge[at2(d, el, col)];
        gR = um.ge[at2(d, er, col)];
        gC = um.gc[at2(d, cm, col)].x;
    }
    // one branch-free form of both cases: s = 1 -+ c, P = u s^2, R = u c s;
    // wind >= 0: (alpha, beta) = (gR P, -gL R), else (gR R, gL P); gamma = +-gC u c (3 -+ 2c),
    // and u c (3 -+ 2c) = u c + 2 u c (1 -+ c) = u c + 2 R
    const W c = u * dtdx;
    const W uc = u * c;
    const W s = fma(up ? W(-1) : W(1), c, W(1));
    const W us = u * s;
    const W P = us * s, R = uc * s;
    al = gR * (up ? P : R);
    be = gL * (up ? neg_bits(R) : P);
    const W G = gC * fma(W(2), R, uc);
    ga = up ? G : neg_bits(G);
}

// FP64 records: {u, +-g} (the sign carries the upwind choice) at rec[idx], the coefficients
// {alpha, beta} at rec[idx + cofs] and {gamma, alpha + beta + gamma} at rec[idx + 2 cofs]; `coefs` false: zero
// coefficients (an edge no flux goes through)
__device__ __forceinline__ void put_record(double2 *rec, long long idx, long long cofs, double wind, double g, bool up,
                                           double dtdx, const UpwindMetric<double> &um, const Dims &d, int m, int col,
                                           bool coefs = true) {
    rec[idx] = edge_record<double2>(wind, g, up);
    double al = 0.0, be = 0.0, ga = 0.0;
    if (coefs) flux_coefs(wind, g, up, dtdx, um, d, m, col, al, be, ga);
    rec[idx + cofs] = make_double2(al, be);
    rec[idx + 2 * cofs] = make_double2(ga, (al + be) + ga);  // sigma: the FP64 CW84 march's mean coefficient
}
// FP32 records {u, +-g}: the paired kernel forms the flux terms of both tracers of a pair itself
// (once per pair, in FP32), which measured faster than loading coefficient records
__device__ __forceinline__ void put_record(float2 *rec, long long idx, long long, float wind, float g, bool up, float,
                                           const UpwindMetric<float> &, const Dims &, int, int, bool = true) {
    rec[idx] = edge_record<float2>(wind, g, up);
}

static dim3 plane_grid(const Dims &d, int bx) { return dim3(ceil_div(d.pitch, bx), d.n + 1, NFACE); }

// analytic winds at interior edges at time t, converted to contravariant components
template <class W>
__global__ void k_wind_interior(Grid g, W *u, W *v, WindParams wp, double t) {
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
        u[o] = (W)((g.cu[3][o] * ulon - g.cu[2][o] * vlat) / g.cu[4][o]);
    } else {  // y-edge (pv): i in [i0, iend), j in [j0, jend]
        int i = d.i0 + b, j = d.i0 + a;
        long long o = at(d, p, i, j);
        double ulon, vlat;
        wind_latlon(wp.vf, wp.prm, g.lon_pv[o], g.lat_pv[o], t, ulon, vlat);
        v[o] = (W)((-g.cv[1][o] * ulon + g.cv[0][o] * vlat) / g.cv[4][o]);
    }
}

// ---------------------------------------------------------------- time-dependent winds
// The reference re-evaluates the analytic wind on every interior edge each step
// (update_adv, advection_timestep.py:55-58), about ten transcendental calls per edge.
// Here the parts that do not depend on t are evaluated once per plan (in FP64, stored in
// W), together with the lat-lon -> contravariant factors, so a step costs ~15 operations
// per edge:
//   vf 2 / deformational:  u_lat-lon = k cos(pi t/T) sin^2(lon - 2 pi t/T) sin(2 lat) + 2 pi cos(lat) / T
//                          v_lat-lon = k cos(pi t/T) sin(2 (lon - 2 pi t/T)) cos(lat)
//                          with sin / cos of (lon - w t) from the angle-difference identities
//   vf 3:                  separable, u = cos(pi t/T) * w0(edge)
//   vf 4:                  constant in time, u = w0(edge)
// In FP64 the results agree with the reference's direct evaluation to a few ulp.

// per-edge coefficients of the x-edges (tab0) and y-edges (tab1): deformational ->
// {sin lon, cos lon, sin 2lat, cos lat, a, b} with contravariant = a u_ll + b v_ll;
// separable / constant -> {contravariant wind at t = 0}
template <class W>
__global__ void k_wind_tables(Grid g, WindParams wp, W *tab0, W *tab1, int ncoef) {
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
    W *tab = which == 0 ? tab0 : tab1;
    // contravariant = a * ulon + b * vlat  (sphgeo.py:120-125)
    double ca = which == 0 ? cf[3][o] / cf[4][o] : -cf[1][o] / cf[4][o];
    double cb = which == 0 ? -cf[2][o] / cf[4][o] : cf[0][o] / cf[4][o];
    if (ncoef == 6) {
        double L = lon[o], P = lat[o];
        tab[0 * d.field + o] = (W)sin(L);
        tab[1 * d.field + o] = (W)cos(L);
        tab[2 * d.field + o] = (W)sin(2.0 * P);
        tab[3 * d.field + o] = (W)cos(P);
        tab[4 * d.field + o] = (W)ca;
        tab[5 * d.field + o] = (W)cb;
    } else {
        double ulon, vlat;
        wind_latlon(wp.vf, wp.prm, lon[o], lat[o], 0.0, ulon, vlat);  // vf 3 at t = 0 (cos 0 = 1); vf 4
        tab[o] = (W)(ca * ulon + cb * vlat);
    }
}

// Device clock: step count and time of the wind in the "current" arrays, plus the
// step's time factors of the analytic wind (computed once here in FP64, not per block).
struct Clock {
    long long k;  // completed steps
    double dt;
    double t;     // time of the current wind
    double f[4];  // deformational: k cos(pi t/T), sin(2 pi t/T), cos(2 pi t/T), 2 pi/T; vf 3: cos(pi t/5)
    double t_old; // time of the previous wind (RK2 extrapolation)
    double hn[4], ho[4];  // time-basis values at t and t_old (basis winds, see wind_basis_h)
    double hx[4];         // 1.5 hn - 0.5 ho: the basis values of the RK2 extrapolation
    float hnf[4], hof[4]; // the same rounded to FP32 (GB300 converts FP64 at the FP64 rate: once here,
                          // not in every thread of the FP32 record kernel)
};

// the values derived from hn and ho once per step instead of in every thread of the record kernels
__device__ __forceinline__ void clock_round(Clock *c) {
    for (int m = 0; m < 4; ++m) {
        c->hnf[m] = (float)c->hn[m];
        c->hof[m] = (float)c->ho[m];
        c->hx[m] = 1.5 * c->hn[m] - 0.5 * c->ho[m];
    }
}

__device__ void clock_factors(Clock *c, WindParams wp, int kind) {
    const double t = c->t;
    if (kind == 1) {
        const double Tp = wp.vf == 2 ? 5.0 : wp.prm[1], k = wp.vf == 2 ? 2.0 : wp.prm[0];
        double w = 2 * PI * t / Tp;
        c->f[0] = k * cos(PI * t / Tp);
        c->f[1] = sin(w);
        c->f[2] = cos(w);
        c->f[3] = 2.0 * PI / Tp;
    } else {
        c->f[0] = wp.vf == 3 ? cos(PI * t / 5.0) : 1.0;
    }
}

__device__ void wind_basis_h(const WindParams &wp, int tkind, double t, double h[4]);

// factors: 1 -> the time factors of the per-edge formula; 0 -> the time-basis values (the
// wind at t_old is the one at the previous t, so each tick evaluates one new set)
__global__ void k_clock_tick(Clock *c, WindParams wp, int kind, int factors) {
    c->t_old = c->t;
    c->k += 1;
    c->t = (double)c->k * c->dt;
    if (factors) {
        clock_factors(c, wp, kind);
    } else {
        for (int m = 0; m < 4; ++m) c->ho[m] = c->hn[m];
        wind_basis_h(wp, kind, c->t, c->hn);
        clock_round(c);
    }
}
__global__ void k_clock_set(Clock *c, long long k, double t, WindParams wp, int kind, int factors) {
    c->t_old = c->t;
    c->k = k;
    c->t = t;
    if (factors) {
        clock_factors(c, wp, kind);
    } else {
        wind_basis_h(wp, kind, c->t_old, c->ho);
        wind_basis_h(wp, kind, c->t, c->hn);
        clock_round(c);
    }
}

// ---------------------------------------------------------------- time-dependent winds as a basis
// For the fused engine a time-dependent wind is stored as u(edge, t) = sum_m C_m(edge) h_m(t)
// on EVERY edge the step reads, ghost edges included: the reference's wind halo
// (interpolation.py:347-532) is linear in the interior wind, so the ghost-edge coefficients
// are the halo of each interior coefficient field, computed once.  A step then evaluates the
// wind at the current and previous times directly (k_wind_rec) instead of running the
// wind update, the wind halo and the departure-point average as separate passes.
//   deformational:  h = {1, K, K cos 2w, K sin 2w}, K = k cos(pi t/T), w = 2 pi t/T, from
//                   sin^2(lon - w) = (1 - cos 2lon cos 2w - sin 2lon sin 2w) / 2 and
//                   sin 2(lon - w) = sin 2lon cos 2w - cos 2lon sin 2w
//   vf 3 / vf 4:    h = {cos(pi t/5)} / {1}
__host__ __device__ inline int wind_nbasis(int tkind) { return tkind == 1 ? 4 : (tkind == 2 ? 1 : 0); }

__device__ void wind_basis_h(const WindParams &wp, int tkind, double t, double h[4]) {
    if (tkind == 1) {
        const double Tp = wp.vf == 2 ? 5.0 : wp.prm[1], k = wp.vf == 2 ? 2.0 : wp.prm[0];
        const double K = k * cos(PI * t / Tp), w2 = 4.0 * PI * t / Tp;
        h[0] = 1.0;
        h[1] = K;
        h[2] = K * cos(w2);
        h[3] = K * sin(w2);
    } else {
        h[0] = wp.vf == 3 ? cos(PI * t / 5.0) : 1.0;
        h[1] = h[2] = h[3] = 0.0;
    }
}

// the M coefficient fields of the interior edges (the other entries are left as they are):
// field m of the x-edges at u + m * field, of the y-edges at v + m * field; each edge's
// trigonometry is evaluated once for all of them
template <class W>
__global__ void k_wind_basis(Grid g, WindParams wp, int M, int tkind, W *u, W *v) {
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
    W *out = (which == 0 ? u : v) + o;
    // contravariant = a * ulon + b * vlat  (sphgeo.py:120-125)
    const double ca = which == 0 ? cf[3][o] / cf[4][o] : -cf[1][o] / cf[4][o];
    const double cb = which == 0 ? -cf[2][o] / cf[4][o] : cf[0][o] / cf[4][o];
    if (tkind == 1) {
        const double L = lon[o], P = lat[o];
        const double Tp = wp.vf == 2 ? 5.0 : wp.prm[1];
        const double s2p = sin(2.0 * P), cp = cos(P), s2l = sin(2.0 * L), c2l = cos(2.0 * L);
        out[0] = (W)(ca * (2.0 * PI / Tp) * cp);
        out[d.field] = (W)(ca * 0.5 * s2p);
        out[2 * d.field] = (W)(-ca * 0.5 * s2p * c2l + cb * cp * s2l);
        out[3 * d.field] = (W)(-ca * 0.5 * s2p * s2l - cb * cp * c2l);
    } else {
        double ulon, vlat;
        wind_latlon(wp.vf, wp.prm, lon[o], lat[o], 0.0, ulon, vlat);  // vf 3 at t = 0 (h = 1); vf 4
        out[0] = (W)(ca * ulon + cb * vlat);
    }
}

// the basis coefficients of edge o (M = 4: one vector load)
template <class W, int M>
struct Coefs {
    W c[M];
    Coefs() = default;
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int m = 0; m < M; ++m) c[m] = W(0);
    }
    __device__ __forceinline__ Coefs(const W *__restrict__ B, long long o) { load(B, o); }
    __device__ __forceinline__ void load(const W *__restrict__ B, long long o) {
        if constexpr (M == 4) {
            if constexpr (sizeof(W) == 4) {
                const float4 v = *reinterpret_cast<const float4 *>(B + o * 4);
                c[0] = v.x; c[1] = v.y; c[2] = v.z; c[3] = v.w;
            } else {
                const double2 a = *reinterpret_cast<const double2 *>(B + o * 4);
                const double2 b = *reinterpret_cast<const double2 *>(B + o * 4 + 2);
                c[0] = a.x; c[1] = a.y; c[2] = b.x; c[3] = b.y;
            }
        } else {
#pragma unroll
            for (int m = 0; m < M; ++m) c[m] = B[o * M + m];
        }
    }
    __device__ __forceinline__ W at(const W *h) const {
        W s = W(0);
#pragma unroll
        for (int m = 0; m < M; ++m) s += c[m] * h[m];
        return s;
    }
    // the same sum with fused multiply-adds (the FP64 records: every FP64 operation counts); the
    // 4-function basis's first function is the constant 1 (wind_basis_h), and so is its RK2
    // extrapolation 1.5 - 0.5, so its term is c[0] itself (the product by 1 is exact)
    __device__ __forceinline__ W at_fma(const W *h) const {
        W s = M == 4 ? c[0] : c[0] * h[0];
#pragma unroll
        for (int m = 1; m < M; ++m) s = fma(c[m], h[m], s);
        return s;
    }
};

// u, v <- the wind at the clock's current time, u_old, v_old <- at its previous time, on every
// edge of the basis (for the staged operators used on a fused plan, e.g. csadv_divergence)
template <class W>
__global__ void k_wind_sync(Dims d, const W *__restrict__ bu, const W *__restrict__ bv, int M, WindParams wp,
                            int tkind, const Clock *__restrict__ clk, W *u, W *v, W *uo, W *vo) {
    __shared__ W hn[4], ho[4];
    if (threadIdx.x < 8) (threadIdx.x < 4 ? hn : ho)[threadIdx.x & 3] =
        (W)(threadIdx.x < 4 ? clk->hn[threadIdx.x] : clk->ho[threadIdx.x - 4]);
    __syncthreads();
    const long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (o >= d.field) return;
    W a = W(0), b = W(0), ao = W(0), bo = W(0);
    for (int m = 0; m < M; ++m) {
        const W cu = bu[o * M + m], cv = bv[o * M + m];
        a += cu * hn[m];
        b += cv * hn[m];
        ao += cu * ho[m];
        bo += cv * ho[m];
    }
    u[o] = a;
    v[o] = b;
    uo[o] = ao;
    vo[o] = bo;
}

// update_adv: old <- current everywhere; current <- wind(t) on interior edges; non-interior
// entries become 0 for ET-S72/ET-PL07 and keep the wind-halo values for ET-DG (the
// reference recomputes them from unchanged lat-lon values)
template <class W>
__global__ void k_wind_update(Dims d, W *u, W *v, W *uo, W *vo, const W *__restrict__ tu, const W *__restrict__ tv,
                              int kind, const Clock *clk, int zero_ghosts) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y, p = blockIdx.z;
    if (j >= d.pitch) return;
    const W f0 = (W)clk->f[0], f1 = (W)clk->f[1], f2 = (W)clk->f[2], f3 = (W)clk->f[3];
    const long long tid = at(d, p, i, j);
    uo[tid] = u[tid];
    vo[tid] = v[tid];
    const bool iu = (i >= d.i0 && i <= d.iend && j >= d.i0 && j < d.iend);
    const bool iv = (i >= d.i0 && i < d.iend && j >= d.i0 && j <= d.iend);
    for (int which = 0; which < 2; ++which) {
        const bool in = which == 0 ? iu : iv;
        W *out = which == 0 ? u : v;
        const W *tab = which == 0 ? tu : tv;
        if (in) {
            if (kind == 1) {
                W sl = tab[tid], cl = tab[d.field + tid], s2p = tab[2 * d.field + tid], cp = tab[3 * d.field + tid];
                W ca = tab[4 * d.field + tid], cb = tab[5 * d.field + tid];
                W s = sl * f2 - cl * f1;  // sin(lon - w t)
                W c = cl * f2 + sl * f1;  // cos(lon - w t)
                W ulon = f0 * (s * s) * s2p + f3 * cp;
                W vlat = f0 * (W(2.0) * s * c) * cp;
                out[tid] = ca * ulon + cb * vlat;
            } else {
                out[tid] = f0 * tab[tid];
            }
        } else if (zero_ghosts) {
            out[tid] = W(0);
        }
    }
}

// ET-DG wind halo, part 1: cubic edge->centre interpolation of the contravariant wind in
// the band of 4 cells along each panel boundary, then contravariant->lat-lon there
// (interpolation.py:356-425).
template <class W>
__global__ void k_wind_band(Grid g, const W *__restrict__ U, const W *__restrict__ V, W *ulon, W *vlat) {
    const Dims d = g.d;
    const int N = d.N, i0 = d.i0, iend = d.iend;
    long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= (long long)NFACE * N * N) return;
    int p = (int)(tid / ((long long)N * N));
    int i = i0 + (int)((tid / N) % N), j = i0 + (int)(tid % N);
    bool wband = i < i0 + NG, eband = i >= iend - NG, sband = j < i0 + NG, nband = j >= iend - NG;
    if (!(wband || eband || sband || nband)) return;
    const W a1 = W(5.0 / 16.0), a2 = W(15.0 / 16.0), a3 = W(-5.0 / 16.0), a4 = W(1.0 / 16.0);
    const W b1 = W(-1.0 / 16.0), b2 = W(9.0 / 16.0), b3 = W(9.0 / 16.0), b4 = W(-1.0 / 16.0);
    auto Ux = [&](int ii) { return U[at(d, p, ii, j)]; };
    auto Vy = [&](int jj) { return V[at(d, p, i, jj)]; };
    W uc, vc;
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
    ulon[o] = (W)g.cc[0][o] * uc + (W)g.cc[2][o] * vc;
    vlat[o] = (W)g.cc[1][o] * uc + (W)g.cc[3][o] * vc;
}

// ET-DG wind halo, part 3: centre->edge cubic interpolation of the lat-lon wind at the
// ghost edges, then lat-lon->contravariant (interpolation.py:436-532)
template <class W>
__global__ void k_wind_ghost_edges(Grid g, const W *__restrict__ ul, const W *__restrict__ vl, W *U, W *V) {
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
    const W c1 = W(9.0 / 16.0), c2 = W(-1.0 / 16.0);
    auto C = [&](const W *f, int i, int j) { return f[at(d, p, i, j)]; };
    int i, j;
    W u, v;
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
        U[o] = (W)((g.cu[3][o] * (double)u - g.cu[2][o] * (double)v) / g.cu[4][o]);
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
        V[o] = (W)((-g.cv[1][o] * (double)u + g.cv[0][o] * (double)v) / g.cv[4][o]);
    }
}

// ET-S72/ET-PL07 + RK2: the edge one beyond each cube edge takes the neighbour's edge one
// inside, with the sign between the panels' coordinate directions
template <class W>
__global__ void k_wind_adjacent(Dims d, W *U, W *V) {
    const int N = d.N;
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= NFACE * 4 * N) return;
    int k = d.i0 + tid % N;
    int s = (tid / N) % 4;
    int p = tid / (4 * N);
    const Conn c = c_conn[p][s];
    int kk = c.rev ? d.n - 1 - k : k;
    W val;
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
template <class W>
__device__ __forceinline__ W rk2_average(const W *__restrict__ U, const W *__restrict__ Uo, const Dims &d, int p,
                                         int i, int j, int dir, W dto2, W dx) {
    auto ui = [&](int k) {
        long long o = dir == 0 ? at(d, p, k, j) : at(d, p, i, k);
        return W(1.5) * U[o] - W(0.5) * Uo[o];
    };
    const int e = dir == 0 ? i : j;
    const W u = U[at(d, p, i, j)];
    const W a = u * dto2 / dx;
    return (u >= W(0)) ? (W(1.0) - a) * ui(e) + a * ui(e - 1) : -a * ui(e + 1) + (W(1.0) + a) * ui(e);
}

template <class W>
__global__ void k_wind_average(Dims d, const W *__restrict__ U, const W *__restrict__ Uo, W *Ua,
                               const W *__restrict__ V, const W *__restrict__ Vo, W *Va, int rk2, W dto2, W dx) {
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

// departure-point wind and upwind flag of the fused engine in one pass: the wind, and one
// bit per edge (warp ballot over 32 consecutive columns; flux.py:48-61 selects the upwind
// cell with u >= 0 of the current wind)
template <class W>
__global__ void k_wind_avgprep(Dims d, const W *__restrict__ U, const W *__restrict__ Uo, const W *__restrict__ V,
                               const W *__restrict__ Vo, W *ua, W *va, uint32_t *ubits, uint32_t *vbits, int wpitch,
                               int rk2, W dto2, W dx) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y, p = blockIdx.z;
    const bool ok = j < d.pitch;
    W u = W(0), v = W(0);
    if (ok) {
        const long long tid = at(d, p, i, j);
        u = U[tid];
        v = V[tid];
        W au = u, av = v;
        if (rk2) {
            au = (j < d.n && i >= d.i0 && i <= d.iend) ? rk2_average(U, Uo, d, p, i, j, 0, dto2, dx) : W(0);
            av = (i < d.n && j >= d.i0 && j <= d.iend) ? rk2_average(V, Vo, d, p, i, j, 1, dto2, dx) : W(0);
        }
        ua[tid] = au;
        va[tid] = av;
    }
    unsigned bu = __ballot_sync(0xffffffffu, ok && u >= W(0));
    unsigned bv = __ballot_sync(0xffffffffu, ok && v >= W(0));
    if (ok && (threadIdx.x & 31) == 0) {
        long long w = ((long long)p * (d.n + 1) + i) * wpitch + (j >> 5);
        ubits[w] = bu;
        vbits[w] = bv;
    }
}

// As k_wind_avgprep, for the line-marching kernel: edge records {departure-point wind, +-g},
// x-edges in the natural layout, y-edges transposed (row j, column i) through a shared 32 x 32
// tile, so that both stores stay coalesced.  Block (32, 8) covers rows i in [32 by, 32 by + 32)
// and columns j in [32 bx, 32 bx + 32) of one panel plane.
template <class W, class V>
__global__ void k_wind_avgprep_t(Dims d, const W *__restrict__ U, const W *__restrict__ Uo, const W *__restrict__ V_,
                                 const W *__restrict__ Vo, const W *__restrict__ gpu, const W *__restrict__ gpvT, V *erx,
                                 V *ery, int rk2, W dto2, W dx, long long cofs, W dtdx, UpwindMetric<W> mx,
                                 UpwindMetric<W> my) {
    __shared__ W tv[32][33];
    __shared__ unsigned char tf[32][33];
    const int p = blockIdx.z, jb = blockIdx.x * 32, ib = blockIdx.y * 32;
    const int lane = threadIdx.x, wy = threadIdx.y;
    for (int k = 0; k < 4; ++k) {
        const int r = wy + 8 * k, i = ib + r, j = jb + lane;
        const bool ok = i <= d.n && j < d.pitch;
        W v = W(0), av = W(0);
        if (ok) {
            const long long t = at(d, p, i, j);
            const W u = U[t];
            v = V_[t];
            W au = u;
            av = v;
            if (rk2) {
                au = (j < d.n && i >= d.i0 && i <= d.iend) ? rk2_average(U, Uo, d, p, i, j, 0, dto2, dx) : W(0);
                av = (i < d.n && j >= d.i0 && j <= d.iend) ? rk2_average(V_, Vo, d, p, i, j, 1, dto2, dx) : W(0);
            }
            put_record(erx, t, cofs, au, gpu[at2(d, i, j)], u >= W(0), dtdx, mx, d, i, j);
        }
        tv[r][lane] = av;
        tf[r][lane] = (ok && v >= W(0)) ? 1 : 0;
    }
    __syncthreads();
    for (int k = 0; k < 4; ++k) {
        const int c = wy + 8 * k, j = jb + c, i = ib + lane;
        if (j <= d.n && i < d.pitch)
            put_record(ery, at(d, p, j, i), cofs, tv[lane][c], gpvT[at2(d, j, i)], tf[lane][c] != 0, dtdx, my, d, j, i);
    }
}

// max over x-edges [i0, iend] x all columns of u*dt/dx (signed), same for y
// (advection_vars.py:89-98): per-block maxima, then one block combines them (max is exact,
// so the result does not depend on the split)
template <class W>
__global__ void k_wind_cfl(Dims d, const W *__restrict__ U, const W *__restrict__ V, double dt, double dx,
                           double *out) {
    __shared__ double rx[256], ry[256];
    double mx = -INFINITY, my = -INFINITY;
    const long long cnt = (long long)NFACE * (d.N + 1) * d.n;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < cnt; t += (long long)gridDim.x * blockDim.x) {
        int p = (int)(t / ((long long)(d.N + 1) * d.n));
        int a = (int)((t / d.n) % (d.N + 1)), b = (int)(t % d.n);
        mx = fmax(mx, (double)U[at(d, p, d.i0 + a, b)] * dt / dx);
        my = fmax(my, (double)V[at(d, p, b, d.i0 + a)] * dt / dx);
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
        out[2 * blockIdx.x] = rx[0];
        out[2 * blockIdx.x + 1] = ry[0];
    }
}

// (max of in[2b], max of in[2b+1]) over b < nb -> out[0], out[1]; one block of 256
__global__ void k_max_pairs(const double *__restrict__ in, int nb, double *out) {
    __shared__ double rx[256], ry[256];
    double mx = -INFINITY, my = -INFINITY;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        mx = fmax(mx, in[2 * b]);
        my = fmax(my, in[2 * b + 1]);
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

// ---------------------------------------------------------------- host side
static WindParams wparams(const Options &o) {
    WindParams wp;
    wp.vf = o.vf;
    for (int c = 0; c < 4; ++c) wp.prm[c] = o.wp[c];
    return wp;
}

template <class W>
static int setup_t(const Options &o, const Grid &g, Winds &w, DeviceArena &mem, double dt, cudaStream_t st) {
    const Dims d = g.d;
    const long long F = d.field;
    w.esize = (int)sizeof(W);
    void **wa[] = {&w.u_pu, &w.v_pv, &w.u_old, &w.v_old, &w.u_avg, &w.v_avg};
    for (void **p : wa) *p = mem.alloc<W>(F);
    W *cen = mem.alloc<W>(2 * F);  // lat-lon centre winds, two contiguous fields
    w.ulon_pc = cen;
    w.vlat_pc = cen ? cen + F : nullptr;
    Clock *clk = mem.alloc<Clock>(1);
    if (!mem.ok()) return CSADV_ERR_OOM;
    for (void **p : wa) CSADV_CUDA(cudaMemsetAsync(*p, 0, F * sizeof(W), st));
    CSADV_CUDA(cudaMemsetAsync(cen, 0, 2 * F * sizeof(W), st));
    w.clock = clk;
    Clock h{0, dt, 0.0, {0.0, 0.0, 0.0, 0.0}, 0.0};
    CSADV_CUDA(cudaMemcpyAsync(clk, &h, sizeof(Clock), cudaMemcpyHostToDevice, st));
    CSADV_CUDA(cudaStreamSynchronize(st));
    if (!wind_time_dependent(o)) {
        w.tkind = 0;
        return CSADV_OK;
    }
    const bool deform = (o.vf == 2 || o.vf == CSADV_WIND_DEFORM);
    const int nc = deform ? 6 : 1;
    w.tkind = deform ? 1 : 2;
    for (int s2 = 0; s2 < 2; ++s2) {
        w.tab[s2] = mem.alloc<W>(nc * F);
        if (!mem.ok()) return CSADV_ERR_OOM;
        CSADV_CUDA(cudaMemsetAsync(w.tab[s2], 0, nc * F * sizeof(W), st));
    }
    long long tot = 2LL * NFACE * (d.N + 1) * d.N;
    k_wind_tables<W><<<ceil_div(tot, 128), 128, 0, st>>>(g, wparams(o), (W *)w.tab[0], (W *)w.tab[1], nc);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

template <class W>
static int initial_t(const Options &o, const Grid &g, Winds &w, cudaStream_t st) {
    const Dims d = g.d;
    if (w.tkind == 0) {
        long long tot = 2LL * NFACE * (d.N + 1) * d.N;
        k_wind_interior<W><<<ceil_div(tot, 128), 128, 0, st>>>(g, (W *)w.u_pu, (W *)w.v_pv, wparams(o), 0.0);
    } else {
        k_clock_set<<<1, 1, 0, st>>>((Clock *)w.clock, 0, 0.0, wparams(o), w.tkind, 1);
        if (w.nbasis) k_clock_set<<<1, 1, 0, st>>>((Clock *)w.clock, 0, 0.0, wparams(o), w.tkind, 0);
        k_wind_update<W><<<plane_grid(d, 128), 128, 0, st>>>(d, (W *)w.u_pu, (W *)w.v_pv, (W *)w.u_old, (W *)w.v_old,
                                                            (const W *)w.tab[0], (const W *)w.tab[1], w.tkind,
                                                            (const Clock *)w.clock, 0);
    }
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

template <class W>
static int update_t(const Options &o, const Grid &g, Winds &w, bool tick, long long k, double t, cudaStream_t st) {
    const Dims d = g.d;
    if (w.tkind == 0) return CSADV_OK;  // static wind: nothing changes with time
    Clock *clk = (Clock *)w.clock;
    const int factors = w.nbasis == 0;
    if (tick) k_clock_tick<<<1, 1, 0, st>>>(clk, wparams(o), w.tkind, factors);
    else k_clock_set<<<1, 1, 0, st>>>(clk, k, t, wparams(o), w.tkind, factors);
    if (w.nbasis == 0)  // with the basis, the step evaluates the wind itself
        k_wind_update<W><<<plane_grid(d, 128), 128, 0, st>>>(d, (W *)w.u_pu, (W *)w.v_pv, (W *)w.u_old, (W *)w.v_old,
                                                            (const W *)w.tab[0], (const W *)w.tab[1], w.tkind, clk,
                                                            o.et != ET_DG);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

template <class W>
static int halo_t(const Options &o, const Grid &g, Winds &w, cudaStream_t st) {
    const Dims d = g.d;
    if (o.et == ET_DG) {
        long long tot = (long long)NFACE * d.N * d.N;
        k_wind_band<W><<<ceil_div(tot, 128), 128, 0, st>>>(g, (const W *)w.u_pu, (const W *)w.v_pv, (W *)w.ulon_pc,
                                                           (W *)w.vlat_pc);
        int rc = launch_halo_dg_tracers<W>((W *)w.ulon_pc, 2, g, nullptr, nullptr, st);  // ulon_pc, vlat_pc
        if (rc) return rc;
        long long per = (long long)(d.N + 1) * 2 * NG + 2LL * d.n;
        tot = 2 * NFACE * per;
        k_wind_ghost_edges<W><<<ceil_div(tot, 128), 128, 0, st>>>(g, (const W *)w.ulon_pc, (const W *)w.vlat_pc,
                                                                  (W *)w.u_pu, (W *)w.v_pv);
    } else if (o.dp == 2) {
        int tot = NFACE * 4 * d.N;
        k_wind_adjacent<W><<<ceil_div(tot, 128), 128, 0, st>>>(d, (W *)w.u_pu, (W *)w.v_pv);
    }
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

template <class W>
static int average_t(const Options &o, const Grid &g, Winds &w, double dt, cudaStream_t st) {
    const Dims d = g.d;
    k_wind_average<W><<<plane_grid(d, 128), 128, 0, st>>>(d, (const W *)w.u_pu, (const W *)w.u_old, (W *)w.u_avg,
                                                          (const W *)w.v_pv, (const W *)w.v_old, (W *)w.v_avg,
                                                          o.dp == 2, (W)(dt * 0.5), (W)g.dx);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

template <class W>
static int cfl_t(const Grid &g, const Winds &w, double dt, double *tmp, double &cfl, cudaStream_t st) {
    // tmp holds at least 3 diag_partials(g) + 8 doubles: room for 2 nb + 2
    int nb = diag_partials(g);
    nb = nb < 1024 ? nb : 1024;
    k_wind_cfl<W><<<nb, 256, 0, st>>>(g.d, (const W *)w.u_pu, (const W *)w.v_pv, dt, g.dx, tmp + 2);
    k_max_pairs<<<1, 256, 0, st>>>(tmp + 2, nb, tmp);
    CSADV_CUDA(cudaGetLastError());
    double h[2];
    CSADV_CUDA(cudaMemcpyAsync(h, tmp, sizeof(h), cudaMemcpyDeviceToHost, st));
    CSADV_CUDA(cudaStreamSynchronize(st));
    cfl = fmax(fabs(h[0]), fabs(h[1]));
    return CSADV_OK;
}

int wind_set_dt(Winds &w, double dt, cudaStream_t st) {
    CSADV_CUDA(cudaMemcpyAsync((char *)w.clock + offsetof(Clock, dt), &dt, sizeof(double), cudaMemcpyHostToDevice, st));
    CSADV_CUDA(cudaStreamSynchronize(st));
    return CSADV_OK;
}

int wind_setup(const Options &o, const Grid &g, Winds &w, DeviceArena &mem, double dt, cudaStream_t st) {
    return o.precision == 64 ? setup_t<double>(o, g, w, mem, dt, st) : setup_t<float>(o, g, w, mem, dt, st);
}
int wind_initial(const Options &o, const Grid &g, Winds &w, cudaStream_t st) {
    return o.precision == 64 ? initial_t<double>(o, g, w, st) : initial_t<float>(o, g, w, st);
}
// update_adv (advection_timestep.py:48-75).  tick: the clock advances by one step (time
// k*dt computed on the device, so the sequence can be replayed from a CUDA graph);
// otherwise the clock is set to (k, t).
int wind_update(const Options &o, const Grid &g, Winds &w, bool tick, long long k, double t, cudaStream_t st) {
    return o.precision == 64 ? update_t<double>(o, g, w, tick, k, t, st) : update_t<float>(o, g, w, tick, k, t, st);
}
int wind_halo(const Options &o, const Grid &g, Winds &w, cudaStream_t st) {
    return o.precision == 64 ? halo_t<double>(o, g, w, st) : halo_t<float>(o, g, w, st);
}
int wind_average(const Options &o, const Grid &g, Winds &w, double dt, cudaStream_t st) {
    return o.precision == 64 ? average_t<double>(o, g, w, dt, st) : average_t<float>(o, g, w, dt, st);
}
int wind_cfl(const Options &o, const Grid &g, const Winds &w, double dt, double *tmp, double &cfl, cudaStream_t st) {
    return o.precision == 64 ? cfl_t<double>(g, w, dt, tmp, cfl, st) : cfl_t<float>(g, w, dt, tmp, cfl, st);
}

template <class real>
int wind_avgprep(const Options &o, const Grid &g, const Winds &w, double dt, real *ua, real *va, uint32_t *ub,
                 uint32_t *vb, int wpitch, cudaStream_t st) {
    const Dims d = g.d;
    k_wind_avgprep<real><<<plane_grid(d, 128), 128, 0, st>>>(d, (const real *)w.u_pu, (const real *)w.u_old,
                                                              (const real *)w.v_pv, (const real *)w.v_old, ua, va, ub,
                                                              vb, wpitch, o.dp == 2, (real)(dt * 0.5), (real)g.dx);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}
// dst[o * M + m] = src[o]: the basis coefficients of an edge side by side (one vector load)
template <class W>
__global__ void k_interleave(const W *__restrict__ src, W *dst, long long n, int M, int m) {
    const long long o = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (o < n) dst[o * M + m] = src[o];
}

// dst(a, b) = src(b, a) for the M interleaved coefficients of every edge of each plane, a <= n,
// b < n (the y-edge index range); zero elsewhere
template <class W>
__global__ void k_transpose_coefs(const W *__restrict__ src, W *dst, Dims d, int M) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= d.field) return;
    const int p = (int)(t / d.plane);
    const long long r = t % d.plane;
    const int a = (int)(r / d.pitch), b = (int)(r % d.pitch);
    const bool in = a <= d.n && b < d.n;
    for (int m = 0; m < M; ++m) dst[t * M + m] = in ? src[(p * d.plane + (long long)b * d.pitch + a) * M + m] : W(0);
}

// Edge records of one step from the basis: the x problem (coefficients bu, metric gpu, records
// erx) and the y problem in transposed coordinates (bvT, gpvT, ery) are the same computation,
// blockIdx.z = problem * 6 + panel.  A block covers 32 x 32 edges (rows ib.., columns jb..): the
// wind at the clock's current time and its RK2 extrapolation 1.5 u - 0.5 u_old on rows
// ib-1 .. ib+32 into shared memory, then the departure-point average along the row index
// (averaged_velocity.py:14-62) and the record (put_record).
//   FP32 (W = float): every coefficient load of a thread is issued before the first is used; the
//   wind and the extrapolation are sums over the basis at the two times (the records {u, +-g}).
//   FP64 (W = double): the FP64 pipe bounds it, so the extrapolation is one fused sum over the basis
//   with the time factors combined first, the average is written with fused multiply-adds, the
//   rows are loaded one at a time (few registers: several blocks share an SM), no wind is formed in
//   the padding columns, and the records carry the edges' flux coefficients (cofs) where fluxes go.
template <class W, int M>
__global__ void __launch_bounds__(256) k_wind_rec(Dims d, const W *__restrict__ bu, const W *__restrict__ bvT,
                                                  const Clock *__restrict__ clk, const W *__restrict__ gpu,
                                                  const W *__restrict__ gpvT, typename Vec2<W>::type *erx,
                                                  typename Vec2<W>::type *ery, int rk2, W c_half, long long cofs, W dtdx,
                                                  UpwindMetric<W> mx, UpwindMetric<W> my, int zbase,
                                                  WindParams wp, int tkind, int peek) {
    using V = typename Vec2<W>::type;
    constexpr bool F64 = sizeof(W) == 8;
    __shared__ W sx[34][33];  // extrapolated winds, rows ib-1 .. ib+32
    __shared__ W sn[32][33];  // winds now, rows ib .. ib+31
    const int z = blockIdx.z + zbase;
    const bool ydir = z >= NFACE;
    const int p = z - (ydir ? NFACE : 0);
    const W *B = ydir ? bvT : bu;
    const W *G = ydir ? gpvT : gpu;
    V *E = (ydir ? ery : erx) + p * d.plane;
    const UpwindMetric<W> &um = ydir ? my : mx;
    const int jb = blockIdx.x * 32, ib = blockIdx.y * 32, lane = threadIdx.x & 31, wy = threadIdx.x >> 5;
    const int j = jb + lane;
    W hn[M], ho[M];
    if (peek) {
        // the records of the clock's next step before the clock has ticked: the time factors that
        // k_clock_tick and clock_round will set (the same operations, so the same bits), while
        // the clock still holds the current ones
        __shared__ W ph[2][4];
        if (threadIdx.x == 0) {
            double h[4];
            wind_basis_h(wp, tkind, (double)(clk->k + 1) * clk->dt, h);
            for (int m = 0; m < M; ++m) {
                if constexpr (F64) {
                    ph[0][m] = h[m];
                    ph[1][m] = 1.5 * h[m] - 0.5 * clk->hn[m];
                } else {
                    ph[0][m] = (float)h[m];
                    ph[1][m] = (float)clk->hn[m];
                }
            }
        }
        __syncthreads();
#pragma unroll
        for (int m = 0; m < M; ++m) {
            hn[m] = ph[0][m];
            ho[m] = ph[1][m];
        }
    } else {
#pragma unroll
        for (int m = 0; m < M; ++m) {
            if constexpr (F64) {
                hn[m] = clk->hn[m];
                ho[m] = clk->hx[m];  // the extrapolation's time factors
            } else {
                hn[m] = clk->hnf[m];
                ho[m] = clk->hof[m];
            }
        }
    }
    constexpr int NQ = 5;  // rows wy + 8 q, q < 5, cover the 34 rows
    if constexpr (F64) {  // columns j >= n are padding: no wind there
#pragma unroll 1
        for (int q = 0; q < NQ; ++q) {
            const int r = wy + 8 * q, i = ib - 1 + r;
            if (r >= 34) break;
            W xs = W(0), xn = W(0);
            if (i >= 0 && i <= d.n && j < d.n) {
                Coefs<W, M> c;
                c.load(B, p * d.plane + (long long)i * d.pitch + j);
                xs = c.at_fma(ho);
                if (r >= 1 && r <= 32) xn = c.at_fma(hn);  // the wind now only on the block's own rows
            }
            sx[r][lane] = xs;
            if (r >= 1 && r <= 32) sn[r - 1][lane] = xn;
        }
    } else {
        Coefs<W, M> c[NQ];
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            const int r = wy + 8 * q, i = ib - 1 + r;
            if (r < 34 && i >= 0 && i <= d.n && j < d.pitch) c[q].load(B, p * d.plane + (long long)i * d.pitch + j);
            else c[q].zero();
        }
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            const int r = wy + 8 * q;
            if (r < 34) {
                const W un = c[q].at(hn), uo = c[q].at(ho);
                sx[r][lane] = W(1.5) * un - W(0.5) * uo;
                if (r >= 1 && r <= 32) sn[r - 1][lane] = un;
            }
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int r = wy + 8 * k, i = ib + r;
        if (i > d.n || j >= d.pitch) continue;
        const W u = sn[r][lane];
        W au = u;
        if (rk2) {
            const W a = u * c_half;
            const bool in = j < d.n && i >= d.i0 && i <= d.iend;
            if constexpr (F64) {  // (1 - a) s0 + a sm = s0 + a (sm - s0); -a sp + (1 + a) s0 = s0 - a (sp - s0)
                const W s0 = sx[r + 1][lane];
                au = in ? (wind_up(u) ? fma(a, sx[r][lane] - s0, s0) : fma(-a, sx[r + 2][lane] - s0, s0)) : W(0);
            } else {
                au = in ? (u >= W(0) ? (W(1) - a) * sx[r + 1][lane] + a * sx[r][lane]
                                     : -a * sx[r + 2][lane] + (W(1) + a) * sx[r + 1][lane])
                        : W(0);
            }
        }
        // fluxes go through x-edges of rows [i0, iend] at columns below n (y: the same transposed)
        put_record(E, (long long)i * d.pitch + j, cofs, au, G[(long long)i * d.pitch + j], wind_up(u), dtdx, um, d, i,
                   j, i >= d.i0 && i <= d.iend && j < d.n);
    }
}

template <class W>
static int basis_setup_t(const Options &o, const Grid &g, Winds &w, DeviceArena &mem, cudaStream_t st) {
    const Dims d = g.d;
    const int M = wind_nbasis(w.tkind);
    if (M == 0 || o.et != ET_DG) return CSADV_OK;
    for (int c = 0; c < 2; ++c) w.btab[c] = mem.alloc<W>((long long)M * d.field);
    if (!mem.ok()) return CSADV_ERR_OOM;
    const size_t F = (size_t)d.field * sizeof(W);
    const long long tot = 2LL * NFACE * (d.N + 1) * d.N;
    // the interior coefficients of all M fields in one pass, into a scratch of 2 M fields (freed
    // in stream order at the end)
    W *scr = nullptr;
    cudaMemPool_t pool = device_pool();
    if (!pool || cudaMallocFromPoolAsync((void **)&scr, 2 * M * F, pool, st) != cudaSuccess) {
        (void)cudaGetLastError();
        return CSADV_ERR_OOM;
    }
    int rc = CSADV_OK;
    if (cudaMemsetAsync(scr, 0, 2 * M * F, st) != cudaSuccess) rc = CSADV_ERR_CUDA;
    if (!rc) {
        k_wind_basis<W><<<ceil_div(tot, 128), 128, 0, st>>>(g, wparams(o), M, w.tkind, scr, scr + (size_t)M * d.field);
        if (cudaGetLastError() != cudaSuccess) rc = CSADV_ERR_CUDA;
    }
    for (int m = 0; m < M && !rc; ++m) {
        // the halo of coefficient field m, computed with the reference's wind-halo operators
        if (cudaMemcpyAsync(w.u_pu, scr + (size_t)m * d.field, F, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
            cudaMemcpyAsync(w.v_pv, scr + (size_t)(M + m) * d.field, F, cudaMemcpyDeviceToDevice, st) != cudaSuccess) {
            rc = CSADV_ERR_CUDA;
            break;
        }
        rc = wind_halo(o, g, w, st);
        if (rc) break;
        const int nb = ceil_div(d.field, 256);
        k_interleave<W><<<nb, 256, 0, st>>>((const W *)w.u_pu, (W *)w.btab[0], d.field, M, m);
        k_interleave<W><<<nb, 256, 0, st>>>((const W *)w.v_pv, (W *)w.btab[1], d.field, M, m);
        if (cudaGetLastError() != cudaSuccess) rc = CSADV_ERR_CUDA;
    }
    cudaFreeAsync(scr, st);
    if (rc) return rc;
    CSADV_CUDA(cudaMemsetAsync(w.u_pu, 0, F, st));
    CSADV_CUDA(cudaMemsetAsync(w.v_pv, 0, F, st));
    {  // the record kernel reads the y coefficients transposed
        w.btabT = mem.alloc<W>((long long)M * d.field);
        if (!mem.ok()) return CSADV_ERR_OOM;
        k_transpose_coefs<W><<<ceil_div(d.field, 256), 256, 0, st>>>((const W *)w.btab[1], (W *)w.btabT, d, M);
        CSADV_CUDA(cudaGetLastError());
    }
    w.nbasis = M;
    return CSADV_OK;  // the clock's basis values are set by wind_initial (k_clock_set)
}

int wind_basis_setup(const Options &o, const Grid &g, Winds &w, DeviceArena &mem, cudaStream_t st) {
    return o.precision == 64 ? basis_setup_t<double>(o, g, w, mem, st) : basis_setup_t<float>(o, g, w, mem, st);
}

// the metric the flux coefficients need (flux_coefs): x-lines natural, y-lines transposed
template <class W>
static void upwind_metrics(const Options &o, const Dims &d, const void *gpu, const void *gpvT, const void *crx,
                           const void *cry, UpwindMetric<W> &mx, UpwindMetric<W> &my) {
    using V = typename Vec2<W>::type;
    mx = UpwindMetric<W>{(const W *)gpu, (const V *)crx, d.n, o.mt == MT_PL07 ? 1 : 0};
    my = UpwindMetric<W>{(const W *)gpvT, (const V *)cry, d.n, o.mt == MT_PL07 ? 1 : 0};
}

template <class real, class V>
int wind_step(const Options &o, const Grid &g, const Winds &w, double dt, const real *gpu, const real *gpvT, V *erx,
              V *ery, const void *crx, const void *cry, cudaStream_t st, int part, int peek) {
    const Dims d = g.d;
    if (!w.btabT) return CSADV_ERR_UNSUPPORTED;
    const real *bu = (const real *)w.btab[0], *bvT = (const real *)w.btabT;
    const Clock *clk = (const Clock *)w.clock;
    // part -1: every edge; 0: the x-edges; 1: the y-edges (blockIdx.z + zbase = problem * 6 + panel)
    dim3 g2(d.pitch / 32, ceil_div(d.n + 1, 32), part < 0 ? 2 * NFACE : NFACE);
    const int zbase = part == 1 ? NFACE : 0;
    const real ch = (real)(dt * 0.5 / g.dx), dtdx = (real)(dt / g.dx);
    const long long cofs = record_coef_offset<real>(d);
    UpwindMetric<real> mx{}, my{};
    if (cofs) upwind_metrics<real>(o, d, gpu, gpvT, crx, cry, mx, my);
    if (w.nbasis == 4)
        k_wind_rec<real, 4><<<g2, 256, 0, st>>>(d, bu, bvT, clk, gpu, gpvT, erx, ery, o.dp == 2, ch, cofs, dtdx, mx, my,
                                                 zbase, wparams(o), w.tkind, peek);
    else
        k_wind_rec<real, 1><<<g2, 256, 0, st>>>(d, bu, bvT, clk, gpu, gpvT, erx, ery, o.dp == 2, ch, cofs, dtdx, mx, my,
                                                 zbase, wparams(o), w.tkind, peek);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}
template int wind_step<double, double2>(const Options &, const Grid &, const Winds &, double, const double *,
                                        const double *, double2 *, double2 *, const void *, const void *, cudaStream_t,
                                        int, int);
template int wind_step<float, float2>(const Options &, const Grid &, const Winds &, double, const float *,
                                      const float *, float2 *, float2 *, const void *, const void *, cudaStream_t, int,
                                      int);

template <class W>
static int sync_t(const Options &o, const Grid &g, const Winds &w, cudaStream_t st) {
    const Dims d = g.d;
    k_wind_sync<W><<<ceil_div(d.field, 256), 256, 0, st>>>(d, (const W *)w.btab[0], (const W *)w.btab[1], w.nbasis,
                                                            wparams(o), w.tkind, (const Clock *)w.clock, (W *)w.u_pu,
                                                            (W *)w.v_pv, (W *)w.u_old, (W *)w.v_old);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

int wind_sync(const Options &o, const Grid &g, const Winds &w, cudaStream_t st) {
    if (w.nbasis == 0) return CSADV_OK;
    return o.precision == 64 ? sync_t<double>(o, g, w, st) : sync_t<float>(o, g, w, st);
}

template <class real, class V>
int wind_avgprep_t(const Options &o, const Grid &g, const Winds &w, double dt, const real *gpu, const real *gpvT,
                   V *erx, V *ery, const void *crx, const void *cry, cudaStream_t st) {
    const Dims d = g.d;
    dim3 grid(d.pitch / 32, ceil_div(d.n + 1, 32), NFACE);
    const long long cofs = record_coef_offset<real>(d);
    UpwindMetric<real> mx{}, my{};
    if (cofs) upwind_metrics<real>(o, d, gpu, gpvT, crx, cry, mx, my);
    k_wind_avgprep_t<real, V><<<grid, dim3(32, 8), 0, st>>>(d, (const real *)w.u_pu, (const real *)w.u_old,
                                                             (const real *)w.v_pv, (const real *)w.v_old, gpu, gpvT,
                                                             erx, ery, o.dp == 2, (real)(dt * 0.5), (real)g.dx, cofs,
                                                             (real)(dt / g.dx), mx, my);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}
template int wind_avgprep_t<double, double2>(const Options &, const Grid &, const Winds &, double, const double *,
                                             const double *, double2 *, double2 *, const void *, const void *,
                                             cudaStream_t);
template int wind_avgprep_t<float, float2>(const Options &, const Grid &, const Winds &, double, const float *,
                                           const float *, float2 *, float2 *, const void *, const void *, cudaStream_t);
template int wind_avgprep<double>(const Options &, const Grid &, const Winds &, double, double *, double *, uint32_t *,
                                  uint32_t *, int, cudaStream_t);
template int wind_avgprep<float>(const Options &, const Grid &, const Winds &, double, float *, float *, uint32_t *,
                                 uint32_t *, int, cudaStream_t);

}  // namespace csadv
