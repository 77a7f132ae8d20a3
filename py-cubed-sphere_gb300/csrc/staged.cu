// Staged engine: the dimension-split divergence as a sequence of full-array kernels, one
// per stage of discrete_operators.py:18-101.  It supports every option combination of
// the reference and is the engine the bit-level parity of the FP64 form is established
// on (this translation unit is compiled without FMA contraction; expressions keep the
// reference's operation order).
//
// Per tracer and step:  recon x / recon y -> [ET-PL07 edge treatment] -> flux x / flux y
// -> split (Qx, Qy) -> [ET-S72/ET-PL07 halo of Qx, Qy] -> recon / [edge treatment] /
// flux of the crossed fields -> [MF-AF] -> div (+ MF-PR partial sums) -> [MF-PR sum]
// -> Q update.
//
// Directions: "x" runs along rows i (stride = pitch), "y" along columns j (stride 1).
// Thread indices put the contiguous column index innermost in both cases.
#include "common.cuh"
#include "internal.h"

namespace csadv {

// numpy.sign: -1, 0 or +1 (NaN passes through)
template <class real>
__device__ __forceinline__ real rsign(real x) {
    return x > real(0) ? real(1) : (x < real(0) ? real(-1) : (x == real(0) ? real(0) : x));
}

// element of line `l`, position `k` along direction DIR (0: x, 1: y)
template <int DIR>
__device__ __forceinline__ long long lat(const Dims &d, int p, int l, int k) {
    return DIR == 0 ? at(d, p, k, l) : at(d, p, l, k);
}

// ---------------------------------------------------------------- reconstruction
// reconstruction_1d.py:26-192 (x) / :204-380 (y): q_L, q_R of cells [i0-1, iend]
template <class real, int REC, int DIR>
__global__ void k_recon(const real *__restrict__ A, real *qL, real *qR, Dims d) {
    const int n = d.n, ncell = d.N + 2;
    long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= (long long)NFACE * ncell * n) return;
    int p, l, c;
    if (DIR == 0) {  // (p, c, l) with l (= column j) innermost
        l = (int)(tid % n);
        c = d.i0 - 1 + (int)((tid / n) % ncell);
        p = (int)(tid / ((long long)n * ncell));
    } else {  // (p, l, c) with c (= column j) innermost
        c = d.i0 - 1 + (int)(tid % ncell);
        l = (int)((tid / ncell) % n);
        p = (int)(tid / ((long long)n * ncell));
    }
    auto Q = [&](int k) { return A[lat<DIR>(d, p, l, k)]; };
    real L, R;
    if (REC == REC_PPM0) {
        const real a = real(7.0 / 12.0);
        auto Qe = [&](int e) { return a * (Q(e) + Q(e - 1)) - (Q(e + 1) + Q(e - 2)) / real(12.0); };
        R = Qe(c + 1);
        L = Qe(c);
    } else if (REC == REC_PL07) {
        const real a1 = real(2.0 / 60.0), a2 = real(-13.0 / 60.0), a3 = real(47.0 / 60.0), a4 = real(27.0 / 60.0),
                   a5 = real(-3.0 / 60.0);
        real q1 = Q(c - 2), q2 = Q(c - 1), q3 = Q(c), q4 = Q(c + 1), q5 = Q(c + 2);
        R = a1 * q1 + a2 * q2 + a3 * q3 + a4 * q4 + a5 * q5;
        L = a5 * q1 + a4 * q2 + a3 * q3 + a2 * q4 + a1 * q5;
    } else if (REC == REC_CW84) {
        real q[7];
#pragma unroll
        for (int m = 0; m < 7; ++m) q[m] = Q(c - 3 + m);  // q[3] = Q(c)
        real dQ[3];                                        // dQ(c-1), dQ(c), dQ(c+1)
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            real qm = q[m + 1], q0 = q[m + 2], qp = q[m + 3];
            real d0 = real(0.5) * (qp - qm);
            real d1 = real(2.0) * (qp - q0);
            real d2 = real(2.0) * (q0 - qm);
            real s = fmin(fabs(d0), fabs(d1));
            s = fmin(s, fabs(d2)) * rsign(d0);
            if (!((qp - q0) * (q0 - qm) > real(0))) s = real(0);
            dQ[m] = s;
        }
        R = real(0.5) * (q[4] + q[3]) - (dQ[2] - dQ[1]) / real(6.0);
        L = real(0.5) * (q[3] + q[2]) - (dQ[1] - dQ[0]) / real(6.0);
        real qc = q[3];
        real dq = R - L;
        real q6 = real(6) * qc - real(3) * (R + L);
        if ((R - qc) * (qc - L) <= real(0)) {
            R = qc;
            L = qc;
        }
        bool over = fabs(dq) < fabs(q6);
        real DL = R - L;
        real mid = qc - real(0.5) * (R + L);
        bool mleft = DL * mid > (DL * DL) / real(6.0);
        bool mright = (-(DL * DL)) / real(6.0) > DL * mid;
        if (over && mleft) L = real(3.0) * qc - real(2.0) * R;
        else if (over && mright) R = real(3.0) * qc - real(2.0) * L;
    } else {  // REC_L04
        real q[7];
#pragma unroll
        for (int m = 0; m < 7; ++m) q[m] = Q(c - 3 + m);
        real mono[3];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            real qm = q[m + 1], q0 = q[m + 2], qp = q[m + 3];
            real dq = real(0.25) * (qp - qm);
            real qmax = fmax(fmax(qm, q0), qp);
            real qmin = fmin(fmin(qm, q0), qp);
            real dmin = qmax - q0;
            real dmax = q0 - qmin;
            mono[m] = fmin(fmin(fabs(dq), dmin), dmax) * rsign(dq);
        }
        R = real(0.5) * (q[4] + q[3]) - (mono[2] - mono[1]) / real(3.0);
        L = real(0.5) * (q[3] + q[2]) - (mono[1] - mono[0]) / real(3.0);
        real q0 = q[3], m2 = real(2.0) * mono[1];
        real lim = fmin(real(2.0) * fabs(mono[1]), fabs(L - q0)) * rsign(m2);
        L = q0 - lim;
        lim = fmin(real(2.0) * fabs(mono[1]), fabs(R - q0)) * rsign(m2);
        R = q0 + lim;
    }
    long long o = lat<DIR>(d, p, l, c);
    qL[o] = L;
    qR[o] = R;
}

// ---------------------------------------------------------------- ET-PL07 edge treatment
// edges_extrapolation + average_parabola_cube_edges (edges_treatment.py:82-178, 31-76).
// One thread per (cube edge, along-edge position) handles both panels of the edge.
struct EdgePairs {
    int8_t p[12], s[12];
};

template <class real>
struct ParabolaRefs {
    const real *Qa, *Qb;  // x-reconstruction input, y-reconstruction input
    real *qLx, *qRx, *qLy, *qRy;
};

// one-sided extrapolations next to side s of panel p on the line through along index k
template <class real>
__device__ void extrapolate_side(const ParabolaRefs<real> &r, const Dims &d, int p, int s, int k, int recon) {
    const bool xdir = (s == SIDE_E || s == SIDE_W);
    const real *Qa = xdir ? r.Qa : r.Qb;
    real *L = xdir ? r.qLx : r.qLy;
    real *R = xdir ? r.qRx : r.qRy;
    auto id = [&](int c) { return xdir ? at(d, p, c, k) : at(d, p, k, c); };
    auto Q = [&](int c) { return Qa[id(c)]; };
    const int i0 = d.i0, iend = d.iend;
    if (s == SIDE_W || s == SIDE_S) {
        L[id(i0)] = real(1.5) * Q(i0) - real(0.5) * Q(i0 + 1);
        real v = (real(3.0) * Q(i0) + real(11.0) * Q(i0 + 1) - real(2.0) * (Q(i0 + 2) - Q(i0))) / real(14.0);
        R[id(i0)] = v;
        L[id(i0 + 1)] = v;
        if (recon == REC_PL07) R[id(i0 + 1)] = L[id(i0 + 2)];
    } else {
        R[id(iend - 1)] = real(1.5) * Q(iend - 1) - real(0.5) * Q(iend - 2);
        real v = (real(3.0) * Q(iend - 1) + real(11.0) * Q(iend - 2) - real(2.0) * (Q(iend - 3) - Q(iend - 1))) /
                 real(14.0);
        L[id(iend - 1)] = v;
        R[id(iend - 2)] = v;
        if (recon == REC_PL07) L[id(iend - 2)] = R[id(iend - 3)];
    }
}

// pointers to the value at the cube edge and at the far face of the boundary (or ghost) cell
template <class real>
__device__ void boundary_cell(const ParabolaRefs<real> &r, const Dims &d, int p, int s, int k, bool ghost,
                              real *&edge, real *&far) {
    switch (s) {
        case SIDE_E: {
            long long o = at(d, p, ghost ? d.iend : d.iend - 1, k);
            edge = ghost ? r.qLx + o : r.qRx + o;
            far = ghost ? r.qRx + o : r.qLx + o;
        } break;
        case SIDE_W: {
            long long o = at(d, p, ghost ? d.i0 - 1 : d.i0, k);
            edge = ghost ? r.qRx + o : r.qLx + o;
            far = ghost ? r.qLx + o : r.qRx + o;
        } break;
        case SIDE_N: {
            long long o = at(d, p, k, ghost ? d.iend : d.iend - 1);
            edge = ghost ? r.qLy + o : r.qRy + o;
            far = ghost ? r.qRy + o : r.qLy + o;
        } break;
        default: {
            long long o = at(d, p, k, ghost ? d.i0 - 1 : d.i0);
            edge = ghost ? r.qRy + o : r.qLy + o;
            far = ghost ? r.qLy + o : r.qRy + o;
        } break;
    }
}

template <class real>
__global__ void k_edges_extrap(ParabolaRefs<real> r, Dims d, EdgePairs pairs, int recon) {
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= 12 * d.N) return;
    int e = tid / d.N;
    int k = d.i0 + tid % d.N;
    int p = pairs.p[e], s = pairs.s[e];
    const Conn c = c_conn[p][s];
    int kk = c.rev ? d.n - 1 - k : k;
    extrapolate_side(r, d, p, s, k, recon);
    extrapolate_side(r, d, c.q, c.qs, kk, recon);
    real *ep, *fp, *eq, *fq;
    boundary_cell(r, d, p, s, k, false, ep, fp);
    boundary_cell(r, d, c.q, c.qs, kk, false, eq, fq);
    real v = (*ep + *eq) * real(0.5);
    *ep = v;
    *eq = v;
    real *gep, *gfp, *geq, *gfq;
    boundary_cell(r, d, p, s, k, true, gep, gfp);
    boundary_cell(r, d, c.q, c.qs, kk, true, geq, gfq);
    *gep = v;
    *gfp = *fq;
    *geq = v;
    *gfq = *fp;
}

// ---------------------------------------------------------------- upwind flux
// numerical_flux_ppm_x / _y (flux.py:20-128): edges [i0, iend] along the direction
template <class real, int DIR>
__global__ void k_flux(const real *__restrict__ A, const real *__restrict__ qL, const real *__restrict__ qR, real *f,
                       const real *__restrict__ uavg, const real *__restrict__ ucur,
                       const double *__restrict__ gE, const double *__restrict__ gC, Dims d, double dt, double dx,
                       int mt) {
    const int n = d.n, nedge = d.N + 1;
    long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= (long long)NFACE * nedge * n) return;
    int p, l, e;
    if (DIR == 0) {
        l = (int)(tid % n);
        e = d.i0 + (int)((tid / n) % nedge);
        p = (int)(tid / ((long long)n * nedge));
    } else {
        e = d.i0 + (int)(tid % nedge);
        l = (int)((tid / nedge) % n);
        p = (int)(tid / ((long long)n * nedge));
    }
    long long oe = lat<DIR>(d, p, l, e);
    auto g2 = [&](const double *g, int k) { return DIR == 0 ? g[at2(d, k, l)] : g[at2(d, l, k)]; };
    const bool upos = ucur[oe] >= real(0);
    const int c = upos ? e - 1 : e;
    long long oc = lat<DIR>(d, p, l, c);
    real L = qL[oc], R = qR[oc], q = A[oc];
    if (mt == MT_0) {
        L = L * (real)g2(gE, c);
        R = R * (real)g2(gE, c + 1);
        q = q * (real)g2(gC, c);
    }
    real dq = R - L;
    real q6 = real(6) * q - real(3) * (R + L);
    const real ua = uavg[oe];
    const real cc = ua * (real)dt / (real)dx;
    real fl;
    if (upos) fl = R + cc * real(0.5) * (q6 - dq) - q6 * cc * cc / real(3.0);
    else fl = L - cc * real(0.5) * (q6 + dq) - q6 * cc * cc / real(3.0);
    fl = fl * ua;
    if (mt == MT_PL07) fl = fl * (real)g2(gE, e);
    f[oe] = fl;
}

// ---------------------------------------------------------------- MF-AF
// average_flux_cube_edges (edges_treatment.py:231-278)
template <class real>
__global__ void k_mfaf(real *fx, real *fy, Dims d, EdgePairs pairs) {
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= 12 * d.N) return;
    int e = tid / d.N;
    int k = d.i0 + tid % d.N;
    int p = pairs.p[e], s = pairs.s[e];
    const Conn c = c_conn[p][s];
    int kk = c.rev ? d.n - 1 - k : k;
    auto ref = [&](int pp, int ss, int kx) -> real * {
        switch (ss) {
            case SIDE_E: return fx + at(d, pp, d.iend, kx);
            case SIDE_W: return fx + at(d, pp, d.i0, kx);
            case SIDE_N: return fy + at(d, pp, kx, d.iend);
            default: return fy + at(d, pp, kx, d.i0);
        }
    };
    real *a = ref(p, s, k), *b = ref(c.q, c.qs, kk);
    if (vec_sign(s, c.qs) > 0) {
        real v = real(0.5) * *a + real(0.5) * *b;
        *a = v;
        *b = v;
    } else {
        real v = real(0.5) * *a - real(0.5) * *b;
        *a = v;
        *b = -v;
    }
}

// ---------------------------------------------------------------- splitting
// F/G operators (discrete_operators.py:109-138) and the splitting step (:49-73) on every cell
template <class real>
__global__ void k_split(const real *__restrict__ Q, const real *__restrict__ fx, const real *__restrict__ fy, real *Qx,
                        real *Qy, const double *__restrict__ g_pc, const double *__restrict__ g_pu,
                        const double *__restrict__ g_pv, const real *__restrict__ uavg,
                        const real *__restrict__ vavg, Dims d, double dt, double dx, int split) {
    const int n = d.n;
    long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= (long long)NFACE * n * n) return;
    int j = (int)(tid % n), i = (int)((tid / n) % n), p = (int)(tid / ((long long)n * n));
    long long o = at(d, p, i, j);
    const real rdt = (real)dt, rdx = (real)dx;
    real dFx = real(0), dFy = real(0);
    if (i >= d.i0 && i < d.iend) {
        dFx = -(fx[at(d, p, i + 1, j)] - fx[o]);
        dFx = dFx * rdt / rdx;
    }
    if (j >= d.i0 && j < d.iend) {
        dFy = -(fy[at(d, p, i, j + 1)] - fy[o]);
        dFy = dFy * rdt / rdx;
    }
    const real q = Q[o];
    const real g = (real)g_pc[at2(d, i, j)];
    if (split == SP_AVLT) {
        real gQ = q * g;
        Qx[o] = (gQ + real(0.5) * dFx) / g;
        Qy[o] = (gQ + real(0.5) * dFy) / g;
        return;
    }
    real c1x = (real)g_pu[at2(d, i + 1, j)] * (uavg[at(d, p, i + 1, j)] * rdt / rdx);
    real c2x = (real)g_pu[at2(d, i, j)] * (uavg[o] * rdt / rdx);
    real c1y = (real)g_pv[at2(d, i, j + 1)] * (vavg[at(d, p, i, j + 1)] * rdt / rdx);
    real c2y = (real)g_pv[at2(d, i, j)] * (vavg[o] * rdt / rdx);
    if (split == SP_L04) {
        real gQ = q * g;
        Qx[o] = (gQ + real(0.5) * dFx + real(0.5) * (c1x - c2x) * q) / g;
        Qy[o] = (gQ + real(0.5) * dFy + real(0.5) * (c1y - c2y) * q) / g;
    } else {
        Qx[o] = real(0.5) * (q + (q + dFx) / (real(1.0) - (c1x - c2x)));
        Qy[o] = real(0.5) * (q + (q + dFy) / (real(1.0) - (c1y - c2y)));
    }
}

// ---------------------------------------------------------------- divergence and update
// div = -(dFx + dFy) / (dt g) on interior cells (discrete_operators.py:95) and, for MF-PR,
// per-block FP64 partial sums of div*g (:98)
constexpr int DIV_BLOCK = 256;

template <class real>
__global__ void k_div(const real *__restrict__ fx, const real *__restrict__ fy, real *div,
                      const double *__restrict__ g_pc, Dims d, double dt, double dx, double *partials) {
    __shared__ double red[DIV_BLOCK];
    const int N = d.N;
    long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    double acc = 0.0;
    if (tid < (long long)NFACE * N * N) {
        int j = d.i0 + (int)(tid % N), i = d.i0 + (int)((tid / N) % N), p = (int)(tid / ((long long)N * N));
        long long o = at(d, p, i, j);
        const real rdt = (real)dt, rdx = (real)dx;
        real dFx = -(fx[at(d, p, i + 1, j)] - fx[o]);
        dFx = dFx * rdt / rdx;
        real dFy = -(fy[at(d, p, i, j + 1)] - fy[o]);
        dFy = dFy * rdt / rdx;
        const double gd = g_pc[at2(d, i, j)];
        const real g = (real)gd;
        real dv = -(dFx + dFy) / (rdt * g);
        div[o] = dv;
        acc = (double)dv * gd;
    }
    if (partials) {
        red[threadIdx.x] = acc;
        __syncthreads();
        for (int s = DIV_BLOCK / 2; s > 0; s >>= 1) {
            if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
            __syncthreads();
        }
        if (threadIdx.x == 0) partials[blockIdx.x] = red[0];
    }
}

// fixed-order sum of the partials -> scal[0] = m0 (one block)
__global__ void k_sum_partials(const double *__restrict__ partials, int npart, double *scal) {
    __shared__ double red[1024];
    double acc = 0.0;
    for (int t = threadIdx.x; t < npart; t += blockDim.x) acc += partials[t];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) scal[0] = red[0];
}

// Q <- Q - dt * (div - g m0 / a2)  (MF-PR, discrete_operators.py:98-101 and
// advection_timestep.py:43), or Q <- Q - dt * div
// (Q == nullptr: write the corrected divergence back into div instead)
template <class real>
__global__ void k_update(real *Q, real *div, const double *__restrict__ g_pc, Dims d, double dt,
                         const double *__restrict__ scal, double a2) {
    const int N = d.N;
    long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= (long long)NFACE * N * N) return;
    int j = d.i0 + (int)(tid % N), i = d.i0 + (int)((tid / N) % N), p = (int)(tid / ((long long)N * N));
    long long o = at(d, p, i, j);
    real dv = div[o];
    if (scal) {
        const double g = g_pc[at2(d, i, j)];
        dv = (real)((double)dv - g * scal[0] / a2);
    }
    if (Q) Q[o] = Q[o] - (real)dt * dv;
    else div[o] = dv;
}

// ---------------------------------------------------------------- host orchestration
static EdgePairs edge_pairs() {
    EdgePairs ep;
    int cnt = 0;
    bool seen[NFACE][4] = {};
    for (int p = 0; p < NFACE; ++p)
        for (int s = 0; s < 4; ++s) {
            if (seen[p][s]) continue;
            const Conn c = h_conn[p][s];
            seen[p][s] = seen[c.q][c.qs] = true;
            ep.p[cnt] = (int8_t)p;
            ep.s[cnt] = (int8_t)s;
            ++cnt;
        }
    return ep;
}

template <class real, int DIR>
static void launch_recon(int recon, const real *A, real *L, real *R, const Dims &d, cudaStream_t st) {
    long long tot = (long long)NFACE * (d.N + 2) * d.n;
    int b = 128, gsz = ceil_div(tot, b);
    switch (recon) {
        case REC_PPM0: k_recon<real, REC_PPM0, DIR><<<gsz, b, 0, st>>>(A, L, R, d); break;
        case REC_CW84: k_recon<real, REC_CW84, DIR><<<gsz, b, 0, st>>>(A, L, R, d); break;
        case REC_PL07: k_recon<real, REC_PL07, DIR><<<gsz, b, 0, st>>>(A, L, R, d); break;
        default: k_recon<real, REC_L04, DIR><<<gsz, b, 0, st>>>(A, L, R, d); break;
    }
}

// compute_fluxes(Qa, Qb) (flux.py:9-15): x-reconstruction and flux of Qa, y of Qb
template <class real>
static int compute_fluxes(const Options &o, const Grid &g, const Winds &w, double dt, const real *Qa,
                          const real *Qb, const Scratch &s, cudaStream_t st) {
    const Dims d = g.d;
    real *qLx = (real *)s.qLx, *qRx = (real *)s.qRx, *qLy = (real *)s.qLy, *qRy = (real *)s.qRy;
    launch_recon<real, 0>(o.recon, Qa, qLx, qRx, d, st);
    launch_recon<real, 1>(o.recon, Qb, qLy, qRy, d, st);
    if (o.et == ET_PL07) {
        ParabolaRefs<real> r{Qa, Qb, qLx, qRx, qLy, qRy};
        k_edges_extrap<real><<<ceil_div(12LL * d.N, 128), 128, 0, st>>>(r, d, edge_pairs(), o.recon);
    }
    long long tot = (long long)NFACE * (d.N + 1) * d.n;
    k_flux<real, 0><<<ceil_div(tot, 128), 128, 0, st>>>(Qa, qLx, qRx, (real *)s.fx, (const real *)w.u_avg,
                                                        (const real *)w.u_pu, g.g_pu, g.g_pc, d, dt, g.dx, o.mt);
    k_flux<real, 1><<<ceil_div(tot, 128), 128, 0, st>>>(Qb, qLy, qRy, (real *)s.fy, (const real *)w.v_avg,
                                                        (const real *)w.v_pv, g.g_pv, g.g_pc, d, dt, g.dx, o.mt);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

int staged_partial_count(const Grid &g) { return ceil_div((long long)NFACE * g.d.N * g.d.N, DIV_BLOCK); }

template <class real>
int staged_divergence(const Options &o, const Grid &g, const Winds &w, double dt, real *Q, const Scratch &s,
                      double *partials, int npart, cudaStream_t st) {
    const Dims d = g.d;
    (void)npart;
    int rc = compute_fluxes<real>(o, g, w, dt, Q, Q, s, st);
    if (rc) return rc;
    real *Qx = (real *)s.Qx, *Qy = (real *)s.Qy;
    long long tot = (long long)NFACE * d.n * d.n;
    k_split<real><<<ceil_div(tot, 128), 128, 0, st>>>(Q, (real *)s.fx, (real *)s.fy, Qx, Qy, g.g_pc, g.g_pu, g.g_pv,
                                                      (const real *)w.u_avg, (const real *)w.v_avg, d, dt, g.dx,
                                                      o.opsplit);
    if (o.et != ET_DG) {
        rc = launch_halo_adjacent<real>(Qx, Qy, g, st);
        if (rc) return rc;
    }
    rc = compute_fluxes<real>(o, g, w, dt, Qy, Qx, s, st);
    if (rc) return rc;
    if (o.mf == MF_AF) k_mfaf<real><<<ceil_div(12LL * d.N, 128), 128, 0, st>>>((real *)s.fx, (real *)s.fy, d, edge_pairs());
    tot = (long long)NFACE * d.N * d.N;
    k_div<real><<<ceil_div(tot, DIV_BLOCK), DIV_BLOCK, 0, st>>>((real *)s.fx, (real *)s.fy, (real *)s.div, g.g_pc, d,
                                                                 dt, g.dx, o.mf == MF_PR ? partials : nullptr);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

template <class real>
int staged_update(const Options &o, const Grid &g, double dt, real *Q, const Scratch &s, double *partials, int npart,
                  double *scal, cudaStream_t st) {
    const Dims d = g.d;
    if (o.mf == MF_PR) k_sum_partials<<<1, 1024, 0, st>>>(partials, npart, scal);
    long long tot = (long long)NFACE * d.N * d.N;
    k_update<real><<<ceil_div(tot, 256), 256, 0, st>>>(Q, (real *)s.div, g.g_pc, d, dt,
                                                        o.mf == MF_PR ? scal : nullptr, g.a2);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

template int staged_divergence<double>(const Options &, const Grid &, const Winds &, double, double *, const Scratch &,
                                       double *, int, cudaStream_t);
template int staged_divergence<float>(const Options &, const Grid &, const Winds &, double, float *, const Scratch &,
                                      double *, int, cudaStream_t);
template int staged_update<double>(const Options &, const Grid &, double, double *, const Scratch &, double *, int,
                                   double *, cudaStream_t);
template int staged_update<float>(const Options &, const Grid &, double, float *, const Scratch &, double *, int,
                                  double *, cudaStream_t);

}  // namespace csadv
