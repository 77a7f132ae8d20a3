// Winds (FP64, shared by every tracer of a plan).
//
//  wind_interior -- analytic winds on the interior edges -> contravariant
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

// old <- current over the whole arrays; for ET-S72/ET-PL07 the non-interior entries of the
// current wind then become 0 (update_adv converts lat-lon winds that are 0 there).  For
// ET-DG those entries keep their value: update_adv recomputes them from the lat-lon winds
// the wind halo stored with them, which gives the same numbers.
__global__ void k_wind_shift(Dims d, double *u, double *v, double *uo, double *vo, int zero_ghosts) {
    long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= d.field) return;
    int p = (int)(tid / d.plane);
    long long r = tid - p * d.plane;
    int i = (int)(r / d.pitch), j = (int)(r % d.pitch);
    (void)p;
    uo[tid] = u[tid];
    vo[tid] = v[tid];
    if (zero_ghosts) {
        bool iu = (i >= d.i0 && i <= d.iend && j >= d.i0 && j < d.iend);
        bool iv = (i >= d.i0 && i < d.iend && j >= d.i0 && j <= d.iend);
        if (!iu) u[tid] = 0.0;
        if (!iv) v[tid] = 0.0;
    }
}

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
__global__ void k_wind_average(Dims d, const double *__restrict__ U, const double *__restrict__ Uo, double *Ua,
                               const double *__restrict__ V, const double *__restrict__ Vo, double *Va, int rk2,
                               double dto2, double dx) {
    long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= d.field) return;
    if (!rk2) {
        Ua[tid] = U[tid];
        Va[tid] = V[tid];
        return;
    }
    int p = (int)(tid / d.plane);
    long long r = tid - p * d.plane;
    int i = (int)(r / d.pitch), j = (int)(r % d.pitch);
    if (j < d.n && i >= d.i0 && i <= d.iend) {  // x-edges [i0, iend] x all columns
        double u = U[tid];
        double a = u * dto2 / dx;
        auto ui = [&](int ii) {
            long long o = at(d, p, ii, j);
            return 1.5 * U[o] - 0.5 * Uo[o];
        };
        Ua[tid] = (u >= 0) ? (1.0 - a) * ui(i) + a * ui(i - 1) : -a * ui(i + 1) + (1.0 + a) * ui(i);
    }
    if (i < d.n && j >= d.i0 && j <= d.iend) {  // y-edges all rows x [j0, jend]
        double v = V[tid];
        double a = v * dto2 / dx;
        auto vi = [&](int jj) {
            long long o = at(d, p, i, jj);
            return 1.5 * V[o] - 0.5 * Vo[o];
        };
        Va[tid] = (v >= 0) ? (1.0 - a) * vi(j) + a * vi(j - 1) : -a * vi(j + 1) + (1.0 + a) * vi(j);
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

int wind_interior(const Options &o, const Grid &g, Winds &w, double t, bool shift, cudaStream_t st) {
    const Dims d = g.d;
    if (shift) {
        k_wind_shift<<<ceil_div(d.field, 256), 256, 0, st>>>(d, w.u_pu, w.v_pv, w.u_old, w.v_old, o.et != ET_DG);
    }
    long long tot = 2LL * NFACE * (d.N + 1) * d.N;
    k_wind_interior<<<ceil_div(tot, 128), 128, 0, st>>>(g, w.u_pu, w.v_pv, wparams(o), t);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

int wind_halo(const Options &o, const Grid &g, Winds &w, cudaStream_t st) {
    const Dims d = g.d;
    if (o.et == ET_DG) {
        long long tot = (long long)NFACE * d.N * d.N;
        k_wind_band<<<ceil_div(tot, 128), 128, 0, st>>>(g, w.u_pu, w.v_pv, w.ulon_pc, w.vlat_pc);
        int rc = launch_halo_dg<double>(w.ulon_pc, g, st);
        if (rc) return rc;
        rc = launch_halo_dg<double>(w.vlat_pc, g, st);
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
    k_wind_average<<<ceil_div(d.field, 256), 256, 0, st>>>(d, w.u_pu, w.u_old, w.u_avg, w.v_pv, w.v_old, w.v_avg,
                                                          o.dp == 2, dt * 0.5, g.dx);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

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
