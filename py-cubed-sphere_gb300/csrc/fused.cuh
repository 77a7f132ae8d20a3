// Fused engine: the whole dimension-split divergence and the Q update of one time step
// in one kernel (ET-DG family: every reconstruction, the three splitting / metric pairs,
// MF-0 and MF-PR, RK1/RK2 winds; MF-AF and the ET-S72/ET-PL07 edge treatments use the
// staged engine because they couple neighbouring panels inside the step).
//
// Each CTA owns a TI x TJ tile of one panel's interior and loops over the tracers.  Per
// tracer, everything stays in shared memory:
//   A  load Q on the tile plus 3 halo cells (ghost cells were filled by the ghost-cell
//      kernel; a pending MF-PR correction g*corr is added to interior cells on load)
//   B  first-pass upwind PPM fluxes: x-edges of the tile rows over the tile columns +-3,
//      y-edges of the tile columns over the tile rows +-3 (one thread per edge computes
//      the reconstruction of the upwind cell only: flux.py:46-66 needs just that one)
//   C  splitting: Qx on the tile rows (columns +-3), Qy on the tile columns (rows +-3)
//      (discrete_operators.py:49-73)
//   D  second-pass fluxes: x of Qy, y of Qx on the tile edges
//   E  div = -(dFx + dFy) / (dt g) and Q* = Q - dt div; with MF-PR, an FP64 block
//      partial of sum(div g); the last CTA to finish sums the partials in a fixed order
//      and stores corr = dt * m0 / a2, so that Q = Q* + g corr (discrete_operators.py:98-101)
//      is applied when Q* is next read -- no second launch and no extra pass over Q.
// The winds (u_avg, v_avg, upwind flags) and the metric are staged once per tile and
// shared by all tracers.
#pragma once
#include "common.cuh"
#include "halo.cuh"
#include "internal.h"
#include "tiles.h"

namespace csadv {


template <class real>
struct RealOps {
    __device__ static __forceinline__ real fmn(real a, real b) { return fmin(a, b); }
    __device__ static __forceinline__ real fmx(real a, real b) { return fmax(a, b); }
    __device__ static __forceinline__ real ab(real a) { return fabs(a); }
};
template <>
struct RealOps<float> {
    __device__ static __forceinline__ float fmn(float a, float b) { return fminf(a, b); }
    __device__ static __forceinline__ float fmx(float a, float b) { return fmaxf(a, b); }
    __device__ static __forceinline__ float ab(float a) { return fabsf(a); }
};

template <class real>
__device__ __forceinline__ real fsign(real x) {
    return x > real(0) ? real(1) : (x < real(0) ? real(-1) : (x == real(0) ? real(0) : x));
}

// Division by a constant.  The fused engine multiplies by the rounded reciprocal (one
// rounding more than the reference's division, far inside both forms' error budgets; an
// IEEE division costs ~10 FP32 or ~15 FP64 instructions, and GB300's FP64 rate is 1/64 of
// FP32).  The staged engine keeps the reference's divisions.
template <class real>
struct Div {
    static constexpr bool exact = false;
    __device__ static __forceinline__ real by(real x, real d, real inv_d) { return exact ? x / d : x * inv_d; }
};

// q_L, q_R of the cell at position 2 of the 5-point window q[0..4] (reconstruction_1d.py:26-192)
template <class real, int REC>
__device__ __forceinline__ void recon5f(const real q[5], real &L, real &R) {
    using O = RealOps<real>;
    using D = Div<real>;
    if (REC == REC_PPM0) {
        const real a = real(7.0 / 12.0);
        R = a * (q[3] + q[2]) - D::by(q[4] + q[1], real(12.0), real(1.0 / 12.0));
        L = a * (q[2] + q[1]) - D::by(q[3] + q[0], real(12.0), real(1.0 / 12.0));
    } else if (REC == REC_PL07) {
        const real a1 = real(2.0 / 60.0), a2 = real(-13.0 / 60.0), a3 = real(47.0 / 60.0), a4 = real(27.0 / 60.0),
                   a5 = real(-3.0 / 60.0);
        R = a1 * q[0] + a2 * q[1] + a3 * q[2] + a4 * q[3] + a5 * q[4];
        L = a5 * q[0] + a4 * q[1] + a3 * q[2] + a2 * q[3] + a1 * q[4];
    } else if (REC == REC_CW84) {
        real dQ[3];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            const real qm = q[m], q0 = q[m + 1], qp = q[m + 2];
            const real d0 = real(0.5) * (qp - qm);
            const real d1 = real(2.0) * (qp - q0);
            const real d2 = real(2.0) * (q0 - qm);
            real s = O::fmn(O::fmn(O::ab(d0), O::ab(d1)), O::ab(d2)) * fsign(d0);
            dQ[m] = ((qp - q0) * (q0 - qm) > real(0)) ? s : real(0);
        }
        R = real(0.5) * (q[3] + q[2]) - D::by(dQ[2] - dQ[1], real(6.0), real(1.0 / 6.0));
        L = real(0.5) * (q[2] + q[1]) - D::by(dQ[1] - dQ[0], real(6.0), real(1.0 / 6.0));
        const real qc = q[2];
        const real dq = R - L;
        const real q6 = real(6) * qc - real(3) * (R + L);
        const bool flat = (R - qc) * (qc - L) <= real(0);
        R = flat ? qc : R;
        L = flat ? qc : L;
        const bool over = O::ab(dq) < O::ab(q6);
        const real DL = R - L;
        const real mid = qc - real(0.5) * (R + L);
        const real d2 = D::by(DL * DL, real(6.0), real(1.0 / 6.0));
        const real prod = DL * mid;
        const bool ml = over && prod > d2;
        const bool mr = over && !ml && -d2 > prod;
        const real Ln = real(3.0) * qc - real(2.0) * R;
        const real Rn = real(3.0) * qc - real(2.0) * L;
        L = ml ? Ln : L;
        R = mr ? Rn : R;
    } else {  // REC_L04
        real mono[3];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            const real qm = q[m], q0 = q[m + 1], qp = q[m + 2];
            const real dq = real(0.25) * (qp - qm);
            const real dmin = O::fmx(O::fmx(qm, q0), qp) - q0;
            const real dmax = q0 - O::fmn(O::fmn(qm, q0), qp);
            mono[m] = O::fmn(O::fmn(O::ab(dq), dmin), dmax) * fsign(dq);
        }
        R = real(0.5) * (q[3] + q[2]) - D::by(mono[2] - mono[1], real(3.0), real(1.0 / 3.0));
        L = real(0.5) * (q[2] + q[1]) - D::by(mono[1] - mono[0], real(3.0), real(1.0 / 3.0));
        const real q0 = q[2], m2 = real(2.0) * mono[1];
        L = q0 - O::fmn(real(2.0) * O::ab(mono[1]), O::ab(L - q0)) * fsign(m2);
        R = q0 + O::fmn(real(2.0) * O::ab(mono[1]), O::ab(R - q0)) * fsign(m2);
    }
}

// upwind PPM flux through an edge (flux.py:20-128).  w = the 5-point window around the
// upwind cell; gl, gr = metric at the cell's left/right edges, gc at its centre; c = Courant
template <class real, int REC>
__device__ __forceinline__ real ppm_flux(const real w[5], bool upos, real ua, real c, real gl, real gr, real gc,
                                         real gedge, int mt) {
    using D = Div<real>;
    real L, R;
    recon5f<real, REC>(w, L, R);
    real q = w[2];
    if (mt == MT_0) {
        L = L * gl;
        R = R * gr;
        q = q * gc;
    }
    const real dq = R - L;
    const real q6 = real(6) * q - real(3) * (R + L);
    const real e = upos ? R : L;
    const real hc = c * real(0.5);
    const real t1 = upos ? hc * (q6 - dq) : -(hc * (q6 + dq));
    real f = e + t1 - D::by(q6 * c * c, real(3.0), real(1.0 / 3.0));
    f = f * ua;
    if (mt == MT_PL07) f = f * gedge;
    return f;
}

// Tile kernel.  blockDim = (32, NW): lanes run along contiguous columns, warps along rows,
// so shared-memory accesses are conflict-free and no index needs a division.  TJ + 6 is
// best a multiple of 32 (the tile columns plus the 3-cell halo on each side).
template <class real, int REC, int TI, int TJ>
__global__ void __launch_bounds__(256) k_fused(FusedArgs a) {
    constexpr int QI = TI + 6, QJ = TJ + 6;
    using D = Div<real>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // per tile (shared by all tracers)
    real *sUa = (real *)smem_raw;       // [TI+1][QJ]  x-edge wind, rows I0.., cols J0-3..
    real *sVa = sUa + (TI + 1) * QJ;    // [QI][TJ+1]  y-edge wind, rows I0-3.., cols J0..
    real *sG = sVa + QI * (TJ + 1);     // [QI][QJ]    g at centres
    real *sIG = sG + QI * QJ;           // [QI][QJ]    1/g (FP32 form)
    real *sGu = sIG + QI * QJ;          // [TI+3][QJ]  g at x-edges, rows I0-1..
    real *sGv = sGu + (TI + 3) * QJ;    // [QI][TJ+3]  g at y-edges, cols J0-1..
    // per tracer
    real *sQ = sGv + QI * (TJ + 3);     // [QI][QJ]
    real *sFx = sQ + QI * QJ;           // [TI+1][QJ]
    real *sFy = sFx + (TI + 1) * QJ;    // [QI][TJ+1]
    real *sQx = sFy + QI * (TJ + 1);    // [TI][QJ]
    real *sQy = sQx + TI * QJ;          // [QI][TJ]
    unsigned char *sUp = (unsigned char *)(sQy + QI * TJ);  // [TI+1][QJ]
    unsigned char *sVp = sUp + (TI + 1) * QJ;                // [QI][TJ+1]
    __shared__ double red[256];

    const Dims d = a.d;
    const int tile = blockIdx.x % a.ntiles;
    const int p = blockIdx.x / a.ntiles;
    const int I0 = d.i0 + (tile / a.ntj) * TI, J0 = d.i0 + (tile % a.ntj) * TJ;
    const int ni = min(TI, d.iend - I0), nj = min(TJ, d.iend - J0);
    const int tx = threadIdx.x, ty = threadIdx.y, NW = blockDim.y;
    const int tid = ty * 32 + tx, nth = 32 * NW;
    const size_t pofs = (size_t)p * d.plane;
    const int P = d.pitch;
    const real *ua = (const real *)a.ua + pofs, *va = (const real *)a.va + pofs;
    const real *gpc = (const real *)a.g_pc, *gpu = (const real *)a.g_pu, *gpv = (const real *)a.g_pv;
    const uint32_t *ub = a.upos + (size_t)p * (d.n + 1) * a.wpitch, *vb = a.vpos + (size_t)p * (d.n + 1) * a.wpitch;
    const real dtdx = (real)(a.dt / a.dx);  // FP32: one rounding; FP64 path keeps u*dt/dx below
    const real rdt = (real)a.dt, rdx = (real)a.dx;

    // ---- per-tile data
    for (int r = ty; r <= ni; r += NW)
        for (int c = tx; c < nj + 6; c += 32) {
            const int i = I0 + r, j = J0 - 3 + c;
            sUa[r * QJ + c] = ua[i * P + j];
            sUp[r * QJ + c] = (ub[i * a.wpitch + (j >> 5)] >> (j & 31)) & 1u;
        }
    for (int r = ty; r < ni + 6; r += NW)
        for (int c = tx; c <= nj; c += 32) {
            const int i = I0 - 3 + r, j = J0 + c;
            sVa[r * (TJ + 1) + c] = va[i * P + j];
            sVp[r * (TJ + 1) + c] = (vb[i * a.wpitch + (j >> 5)] >> (j & 31)) & 1u;
        }
    for (int r = ty; r < ni + 6; r += NW)
        for (int c = tx; c < nj + 6; c += 32) {
            const real g = gpc[(I0 - 3 + r) * P + J0 - 3 + c];
            sG[r * QJ + c] = g;
            if (!D::exact) sIG[r * QJ + c] = real(1) / g;
        }
    for (int r = ty; r < ni + 3; r += NW)
        for (int c = tx; c < nj + 6; c += 32) sGu[r * QJ + c] = gpu[(I0 - 1 + r) * P + J0 - 3 + c];
    for (int r = ty; r < ni + 6; r += NW)
        for (int c = tx; c < nj + 3; c += 32) sGv[r * (TJ + 3) + c] = gpv[(I0 - 3 + r) * P + J0 - 1 + c];
    __syncthreads();

    for (int tr = 0; tr < a.T; ++tr) {
        const real *Qin = (const real *)a.Qin + (size_t)tr * d.field + pofs;
        real *Qout = (real *)a.Qout + (size_t)tr * d.field + pofs;
        const bool hc = a.corr_in != nullptr;
        const real corr = hc ? (real)a.corr_in[tr] : real(0);
        // A: Q on the tile + halo (+ pending mass-fixer correction on interior cells)
        for (int r = ty; r < ni + 6; r += NW) {
            const int i = I0 - 3 + r;
            const bool irow = i >= d.i0 && i < d.iend;
            for (int c = tx; c < nj + 6; c += 32) {
                const int j = J0 - 3 + c;
                real v = Qin[i * P + j];
                if (hc && irow && j >= d.i0 && j < d.iend) v = corrected(v, sG[r * QJ + c], corr);
                sQ[r * QJ + c] = v;
            }
        }
        __syncthreads();
        // B: first-pass fluxes.  x-edges: rows I0+e (e <= ni), cols J0-3+c
        for (int e = ty; e <= ni; e += NW)
            for (int c = tx; c < nj + 6; c += 32) {
                const int wi = e * QJ + c;
                const bool up = sUp[wi];
                const int cr = e + (up ? 2 : 3);  // upwind cell's row in sQ
                real w[5];
#pragma unroll
                for (int m = 0; m < 5; ++m) w[m] = sQ[(cr - 2 + m) * QJ + c];
                const real u = sUa[wi];
                const real cc = D::exact ? u * rdt / rdx : u * dtdx;
                sFx[wi] = ppm_flux<real, REC>(w, up, u, cc, sGu[(cr - 2) * QJ + c], sGu[(cr - 1) * QJ + c],
                                              sG[cr * QJ + c], sGu[(e + 1) * QJ + c], a.mt);
            }
        // y-edges: rows I0-3+r, cols J0+e (e <= nj)
        for (int r = ty; r < ni + 6; r += NW)
            for (int e = tx; e <= nj; e += 32) {
                const int wi = r * (TJ + 1) + e;
                const bool up = sVp[wi];
                const int cc0 = e + (up ? 2 : 3);  // upwind cell's column in sQ
                real w[5];
#pragma unroll
                for (int m = 0; m < 5; ++m) w[m] = sQ[r * QJ + cc0 - 2 + m];
                const real v = sVa[wi];
                const real cc = D::exact ? v * rdt / rdx : v * dtdx;
                sFy[wi] = ppm_flux<real, REC>(w, up, v, cc, sGv[r * (TJ + 3) + cc0 - 2],
                                              sGv[r * (TJ + 3) + cc0 - 1], sG[r * QJ + cc0],
                                              sGv[r * (TJ + 3) + e + 1], a.mt);
            }
        __syncthreads();
        // C: splitting (discrete_operators.py:49-73)
        for (int r = ty; r < ni; r += NW)  // Qx: rows I0+r, cols J0-3+c
            for (int c = tx; c < nj + 6; c += 32) {
                const int sq = (r + 3) * QJ + c;
                const real q = sQ[sq], g = sG[sq];
                real dF = -(sFx[(r + 1) * QJ + c] - sFx[r * QJ + c]);
                dF = D::exact ? dF * rdt / rdx : dF * dtdx;
                real out;
                if (a.split == SP_AVLT) {
                    out = D::exact ? (q * g + real(0.5) * dF) / g : q + real(0.5) * dF * sIG[sq];
                } else {
                    const real c1 = sGu[(r + 2) * QJ + c] * (D::exact ? sUa[(r + 1) * QJ + c] * rdt / rdx
                                                                      : sUa[(r + 1) * QJ + c] * dtdx);
                    const real c2 = sGu[(r + 1) * QJ + c] * (D::exact ? sUa[r * QJ + c] * rdt / rdx
                                                                      : sUa[r * QJ + c] * dtdx);
                    if (a.split == SP_L04)
                        out = D::exact ? (q * g + real(0.5) * dF + real(0.5) * (c1 - c2) * q) / g
                                       : (q * g + real(0.5) * dF + real(0.5) * (c1 - c2) * q) * sIG[sq];
                    else
                        out = real(0.5) * (q + (q + dF) / (real(1.0) - (c1 - c2)));
                }
                sQx[r * QJ + c] = out;
            }
        for (int r = ty; r < ni + 6; r += NW)  // Qy: rows I0-3+r, cols J0+c
            for (int c = tx; c < nj; c += 32) {
                const int sq = r * QJ + c + 3;
                const real q = sQ[sq], g = sG[sq];
                real dF = -(sFy[r * (TJ + 1) + c + 1] - sFy[r * (TJ + 1) + c]);
                dF = D::exact ? dF * rdt / rdx : dF * dtdx;
                real out;
                if (a.split == SP_AVLT) {
                    out = D::exact ? (q * g + real(0.5) * dF) / g : q + real(0.5) * dF * sIG[sq];
                } else {
                    const real c1 = sGv[r * (TJ + 3) + c + 2] * (D::exact ? sVa[r * (TJ + 1) + c + 1] * rdt / rdx
                                                                         : sVa[r * (TJ + 1) + c + 1] * dtdx);
                    const real c2 = sGv[r * (TJ + 3) + c + 1] * (D::exact ? sVa[r * (TJ + 1) + c] * rdt / rdx
                                                                         : sVa[r * (TJ + 1) + c] * dtdx);
                    if (a.split == SP_L04)
                        out = D::exact ? (q * g + real(0.5) * dF + real(0.5) * (c1 - c2) * q) / g
                                       : (q * g + real(0.5) * dF + real(0.5) * (c1 - c2) * q) * sIG[sq];
                    else
                        out = real(0.5) * (q + (q + dF) / (real(1.0) - (c1 - c2)));
                }
                sQy[r * TJ + c] = out;
            }
        __syncthreads();
        // D: second-pass fluxes (x of Qy, y of Qx) on the tile's edges
        for (int e = ty; e <= ni; e += NW)
            for (int c = tx; c < nj; c += 32) {
                const int wi = e * QJ + c + 3;
                const bool up = sUp[wi];
                const int cr = e + (up ? 2 : 3);  // upwind cell's row in sQy
                real w[5];
#pragma unroll
                for (int m = 0; m < 5; ++m) w[m] = sQy[(cr - 2 + m) * TJ + c];
                const real u = sUa[wi];
                const real cc = D::exact ? u * rdt / rdx : u * dtdx;
                sFx[wi] = ppm_flux<real, REC>(w, up, u, cc, sGu[(cr - 2) * QJ + c + 3], sGu[(cr - 1) * QJ + c + 3],
                                              sG[cr * QJ + c + 3], sGu[(e + 1) * QJ + c + 3], a.mt);
            }
        for (int r = ty; r < ni; r += NW)
            for (int e = tx; e <= nj; e += 32) {
                const int wi = (r + 3) * (TJ + 1) + e;
                const bool up = sVp[wi];
                const int cc0 = e + (up ? 2 : 3);  // upwind cell's column in sQx
                real w[5];
#pragma unroll
                for (int m = 0; m < 5; ++m) w[m] = sQx[r * QJ + cc0 - 2 + m];
                const real v = sVa[wi];
                const real cc = D::exact ? v * rdt / rdx : v * dtdx;
                sFy[wi] = ppm_flux<real, REC>(w, up, v, cc, sGv[(r + 3) * (TJ + 3) + cc0 - 2],
                                              sGv[(r + 3) * (TJ + 3) + cc0 - 1], sG[(r + 3) * QJ + cc0],
                                              sGv[(r + 3) * (TJ + 3) + e + 1], a.mt);
            }
        __syncthreads();
        // E: divergence and update; the MF-PR partial sum is kept in the state's precision
        // per thread (at most a few cells) and in FP64 across threads and CTAs
        real acc = real(0);
        for (int r = ty; r < ni; r += NW)
            for (int c = tx; c < nj; c += 32) {
                const real s = (sFx[(r + 1) * QJ + c + 3] - sFx[r * QJ + c + 3]) +
                               (sFy[(r + 3) * (TJ + 1) + c + 1] - sFy[(r + 3) * (TJ + 1) + c]);
                const int sq = (r + 3) * QJ + c + 3;
                real dv, qn;
                if (D::exact) {
                    real dFx = -(sFx[(r + 1) * QJ + c + 3] - sFx[r * QJ + c + 3]);
                    dFx = dFx * rdt / rdx;
                    real dFy = -(sFy[(r + 3) * (TJ + 1) + c + 1] - sFy[(r + 3) * (TJ + 1) + c]);
                    dFy = dFy * rdt / rdx;
                    dv = -(dFx + dFy) / (rdt * sG[sq]);
                    qn = sQ[sq] - rdt * dv;
                } else {
                    // div = (fluxes out - in) / (dx g); Q - dt div
                    dv = s * sIG[sq] * (real(1) / rdx);
                    qn = sQ[sq] - s * dtdx * sIG[sq];
                }
                Qout[(I0 + r) * P + J0 + c] = qn;
                if (a.mfpr) acc += dv * sG[sq];
            }
        if (a.mfpr) {
            double dacc = (double)acc;
            for (int o = 16; o > 0; o >>= 1) dacc += __shfl_xor_sync(0xffffffffu, dacc, o);
            if (tx == 0) red[ty] = dacc;
            __syncthreads();
            if (tid == 0) {
                double s = 0.0;
                for (int w = 0; w < NW; ++w) s += red[w];
                a.partials[(size_t)tr * gridDim.x + blockIdx.x] = s;
            }
        }
        __syncthreads();
    }
    if (!a.mfpr) return;
    // last CTA: fixed-order sum of the partials -> corr = dt * m0 / a2 per tracer
    __shared__ bool last;
    if (tid == 0) {
        __threadfence();
        unsigned int prev = atomicAdd(a.counter, 1u);
        last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    for (int tr = 0; tr < a.T; ++tr) {
        double acc = 0.0;
        const volatile double *pp = a.partials + (size_t)tr * gridDim.x;
        for (int b = tid; b < (int)gridDim.x; b += nth) acc += pp[b];
        red[tid] = acc;
        __syncthreads();
        for (int s = nth / 2; s > 0; s >>= 1) {
            if (tid < s) red[tid] += red[tid + s];
            __syncthreads();
        }
        if (tid == 0) a.corr_out[tr] = a.dt * red[0] / a.a2;
        __syncthreads();
    }
    if (tid == 0) *a.counter = 0u;
}

template <class real, int TI, int TJ>
constexpr size_t fused_smem_bytes() {
    constexpr int QI = TI + 6, QJ = TJ + 6;
    size_t reals = (size_t)(TI + 1) * QJ + QI * (TJ + 1) + 2 * QI * QJ + (TI + 3) * QJ + QI * (TJ + 3) + QI * QJ +
                   (TI + 1) * QJ + QI * (TJ + 1) + TI * QJ + QI * TJ;
    size_t bytes = reals * sizeof(real) + (size_t)(TI + 1) * QJ + QI * (TJ + 1);
    return (bytes + 15) / 16 * 16;
}


template <class real, int REC, int TI, int TJ>
static int fused_go(FusedArgs a, cudaStream_t st) {
    constexpr size_t smem = fused_smem_bytes<real, TI, TJ>();
    if (st == (cudaStream_t)-1) {  // prepare only
        CSADV_CUDA(cudaFuncSetAttribute(k_fused<real, REC, TI, TJ>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem));
        return CSADV_OK;
    }
    a.ntj = (a.d.N + TJ - 1) / TJ;
    a.ntiles = ((a.d.N + TI - 1) / TI) * a.ntj;
    k_fused<real, REC, TI, TJ><<<NFACE * a.ntiles, dim3(32, 8), smem, st>>>(a);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

template <class real, int REC>
static int fused_tile(FusedArgs a, int tile, cudaStream_t st) {
    switch (tile) {
        case 0: return fused_go<real, REC, 16, 58>(a, st);
        case 1: return fused_go<real, REC, 32, 58>(a, st);
        case 2: return fused_go<real, REC, 16, 26>(a, st);
        default: return fused_go<real, REC, 32, 26>(a, st);
    }
}

template <class real>
int fused_launch(const FusedArgs &a, int recon, int tile, cudaStream_t st) {
    switch (recon) {
        case REC_PPM0: return fused_tile<real, REC_PPM0>(a, tile, st);
        case REC_CW84: return fused_tile<real, REC_CW84>(a, tile, st);
        case REC_PL07: return fused_tile<real, REC_PL07>(a, tile, st);
        default: return fused_tile<real, REC_L04>(a, tile, st);
    }
}


}  // namespace csadv
