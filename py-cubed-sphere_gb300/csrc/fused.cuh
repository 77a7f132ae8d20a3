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
#include "internal.h"

namespace csadv {

struct FusedArgs {
    Dims d;
    int T;                 // tracers
    int ntj, ntiles;       // tiles along j, tiles per panel
    double dt, dx, a2;
    const void *Qin;       // T fields (real), ghost cells filled
    void *Qout;            // T fields (real), interior written
    const double *corr_in; // [T] pending MF-PR correction of Qin (nullptr: none)
    double *corr_out;      // [T] correction of Qout (MF-PR only)
    double *partials;      // [T][gridDim.x]
    unsigned int *counter; // arrival counter (MF-PR)
    const void *ua, *va;   // departure-point winds (real) at x-/y-edges, 6 planes
    const uint32_t *upos, *vpos;  // upwind flags: bit j&31 of word [p][i][j>>5] (1: wind >= 0)
    const void *g_pc, *g_pu, *g_pv;  // metric (real), one plane each
    int split, mt, mfpr;
    int wpitch;            // words per row of the flag arrays
};

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

// q_L, q_R of the cell at position 2 of the 5-point window q[0..4] (reconstruction_1d.py:26-192)
template <class real, int REC>
__device__ __forceinline__ void recon5(const real q[5], real &L, real &R) {
    using O = RealOps<real>;
    if (REC == REC_PPM0) {
        const real a = real(7.0 / 12.0);
        R = a * (q[3] + q[2]) - (q[4] + q[1]) / real(12.0);
        L = a * (q[2] + q[1]) - (q[3] + q[0]) / real(12.0);
    } else if (REC == REC_PL07) {
        const real a1 = real(2.0 / 60.0), a2 = real(-13.0 / 60.0), a3 = real(47.0 / 60.0), a4 = real(27.0 / 60.0),
                   a5 = real(-3.0 / 60.0);
        R = a1 * q[0] + a2 * q[1] + a3 * q[2] + a4 * q[3] + a5 * q[4];
        L = a5 * q[0] + a4 * q[1] + a3 * q[2] + a2 * q[3] + a1 * q[4];
    } else if (REC == REC_CW84) {
        real dQ[3];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            real qm = q[m], q0 = q[m + 1], qp = q[m + 2];
            real d0 = real(0.5) * (qp - qm);
            real d1 = real(2.0) * (qp - q0);
            real d2 = real(2.0) * (q0 - qm);
            real s = O::fmn(O::ab(d0), O::ab(d1));
            s = O::fmn(s, O::ab(d2)) * fsign(d0);
            if (!((qp - q0) * (q0 - qm) > real(0))) s = real(0);
            dQ[m] = s;
        }
        R = real(0.5) * (q[3] + q[2]) - (dQ[2] - dQ[1]) / real(6.0);
        L = real(0.5) * (q[2] + q[1]) - (dQ[1] - dQ[0]) / real(6.0);
        const real qc = q[2];
        const real dq = R - L;
        const real q6 = real(6) * qc - real(3) * (R + L);
        if ((R - qc) * (qc - L) <= real(0)) {
            R = qc;
            L = qc;
        }
        const bool over = O::ab(dq) < O::ab(q6);
        const real DL = R - L;
        const real mid = qc - real(0.5) * (R + L);
        if (over && DL * mid > (DL * DL) / real(6.0)) L = real(3.0) * qc - real(2.0) * R;
        else if (over && (-(DL * DL)) / real(6.0) > DL * mid) R = real(3.0) * qc - real(2.0) * L;
    } else {  // REC_L04
        real mono[3];
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            real qm = q[m], q0 = q[m + 1], qp = q[m + 2];
            real dq = real(0.25) * (qp - qm);
            real dmin = O::fmx(O::fmx(qm, q0), qp) - q0;
            real dmax = q0 - O::fmn(O::fmn(qm, q0), qp);
            mono[m] = O::fmn(O::fmn(O::ab(dq), dmin), dmax) * fsign(dq);
        }
        R = real(0.5) * (q[3] + q[2]) - (mono[2] - mono[1]) / real(3.0);
        L = real(0.5) * (q[2] + q[1]) - (mono[1] - mono[0]) / real(3.0);
        const real q0 = q[2], m2 = real(2.0) * mono[1];
        L = q0 - O::fmn(real(2.0) * O::ab(mono[1]), O::ab(L - q0)) * fsign(m2);
        R = q0 + O::fmn(real(2.0) * O::ab(mono[1]), O::ab(R - q0)) * fsign(m2);
    }
}

// upwind PPM flux through an edge (flux.py:20-128).  w = the 5-point window around the
// upwind cell; gl, gr = metric at the cell's left/right edges, gc at its centre.
template <class real, int REC>
__device__ __forceinline__ real ppm_flux(const real w[5], bool upos, real ua, real c, real gl, real gr, real gc,
                                         real gedge, int mt) {
    real L, R;
    recon5<real, REC>(w, L, R);
    real q = w[2];
    if (mt == MT_0) {
        L = L * gl;
        R = R * gr;
        q = q * gc;
    }
    const real dq = R - L;
    const real q6 = real(6) * q - real(3) * (R + L);
    real f;
    if (upos) f = R + c * real(0.5) * (q6 - dq) - q6 * c * c / real(3.0);
    else f = L - c * real(0.5) * (q6 + dq) - q6 * c * c / real(3.0);
    f = f * ua;
    if (mt == MT_PL07) f = f * gedge;
    return f;
}

template <int TI, int TJ>
struct TileGeom {
    static constexpr int QI = TI + 6, QJ = TJ + 6;  // Q tile incl. 3 halo cells
};

template <class real, int REC, int TI, int TJ>
__global__ void __launch_bounds__(256) k_fused(FusedArgs a) {
    constexpr int QI = TI + 6, QJ = TJ + 6;
    // shared memory (dynamic): winds and metric (per tile), then per-tracer work arrays
    extern __shared__ __align__(16) unsigned char smem_raw[];
    real *sUa = (real *)smem_raw;           // [TI+1][QJ]   x-edge u_avg   rows I0.., cols J0-3..
    real *sVa = sUa + (TI + 1) * QJ;        // [QI][TJ+1]   y-edge v_avg   rows I0-3.., cols J0..
    real *sG = sVa + QI * (TJ + 1);         // [QI][QJ]     g at centres
    real *sQ = sG + QI * QJ;                // [QI][QJ]
    real *sFx = sQ + QI * QJ;               // [TI+1][QJ]
    real *sFy = sFx + (TI + 1) * QJ;        // [QI][TJ+1]
    real *sQx = sFy + QI * (TJ + 1);        // [TI][QJ]
    real *sQy = sQx + TI * QJ;              // [QI][TJ]
    unsigned char *sUp = (unsigned char *)(sQy + QI * TJ);  // [TI+1][QJ]
    unsigned char *sVp = sUp + (TI + 1) * QJ;                // [QI][TJ+1]
    __shared__ double red[256];

    const Dims d = a.d;
    const int tile = blockIdx.x % a.ntiles;
    const int p = blockIdx.x / a.ntiles;
    const int I0 = d.i0 + (tile / a.ntj) * TI, J0 = d.i0 + (tile % a.ntj) * TJ;
    const int ni = min(TI, d.iend - I0), nj = min(TJ, d.iend - J0);
    const real *ua = (const real *)a.ua, *va = (const real *)a.va;
    const real *gpc = (const real *)a.g_pc, *gpu = (const real *)a.g_pu, *gpv = (const real *)a.g_pv;
    const real rdt = (real)a.dt, rdx = (real)a.dx;
    const int tid = threadIdx.x, nth = blockDim.x;

    // ---- per-tile data shared by every tracer
    for (int t = tid; t < (TI + 1) * QJ; t += nth) {
        int ei = t / QJ, cj = t % QJ;
        int i = I0 + ei, j = J0 - 3 + cj;
        if (ei <= ni && cj < nj + 6) {
            sUa[t] = ua[at(d, p, i, j)];
            sUp[t] = (a.upos[(p * (long long)(d.n + 1) + i) * a.wpitch + (j >> 5)] >> (j & 31)) & 1u;
        }
    }
    for (int t = tid; t < QI * (TJ + 1); t += nth) {
        int ri = t / (TJ + 1), ej = t % (TJ + 1);
        int i = I0 - 3 + ri, j = J0 + ej;
        if (ri < ni + 6 && ej <= nj) {
            sVa[t] = va[at(d, p, i, j)];
            sVp[t] = (a.vpos[(p * (long long)(d.n + 1) + i) * a.wpitch + (j >> 5)] >> (j & 31)) & 1u;
        }
    }
    for (int t = tid; t < QI * QJ; t += nth) {
        int ri = t / QJ, cj = t % QJ;
        if (ri < ni + 6 && cj < nj + 6) sG[t] = gpc[at2(d, I0 - 3 + ri, J0 - 3 + cj)];
    }
    __syncthreads();

    for (int tr = 0; tr < a.T; ++tr) {
        const real *Qin = (const real *)a.Qin + (size_t)tr * d.field;
        real *Qout = (real *)a.Qout + (size_t)tr * d.field;
        const real corr = a.corr_in ? (real)a.corr_in[tr] : real(0);
        // A: load Q (+ pending correction on interior cells)
        for (int t = tid; t < QI * QJ; t += nth) {
            int ri = t / QJ, cj = t % QJ;
            if (ri < ni + 6 && cj < nj + 6) {
                int i = I0 - 3 + ri, j = J0 - 3 + cj;
                real v = Qin[at(d, p, i, j)];
                if (a.corr_in && i >= d.i0 && i < d.iend && j >= d.i0 && j < d.iend) v = v + sG[t] * corr;
                sQ[t] = v;
            }
        }
        __syncthreads();
        // B: first-pass fluxes
        for (int t = tid; t < (TI + 1) * QJ; t += nth) {  // x-edges: rows I0+ei, cols J0-3+cj
            int ei = t / QJ, cj = t % QJ;
            if (ei > ni || cj >= nj + 6) continue;
            const bool up = sUp[t];
            const int c = ei + (up ? 2 : 3);  // upwind cell's row in sQ
            real w[5];
#pragma unroll
            for (int m = 0; m < 5; ++m) w[m] = sQ[(c - 2 + m) * QJ + cj];
            const int ci = I0 - 3 + c, j = J0 - 3 + cj;
            const real u = sUa[t];
            const real cc = u * rdt / rdx;
            sFx[t] = ppm_flux<real, REC>(w, up, u, cc, gpu[at2(d, ci, j)], gpu[at2(d, ci + 1, j)], sG[c * QJ + cj],
                                         gpu[at2(d, I0 + ei, j)], a.mt);
        }
        for (int t = tid; t < QI * (TJ + 1); t += nth) {  // y-edges: rows I0-3+ri, cols J0+ej
            int ri = t / (TJ + 1), ej = t % (TJ + 1);
            if (ri >= ni + 6 || ej > nj) continue;
            const bool up = sVp[t];
            const int c = ej + (up ? 2 : 3);  // upwind cell's column in sQ
            real w[5];
#pragma unroll
            for (int m = 0; m < 5; ++m) w[m] = sQ[ri * QJ + c - 2 + m];
            const int i = I0 - 3 + ri, cjg = J0 - 3 + c;
            const real v = sVa[t];
            const real cc = v * rdt / rdx;
            sFy[t] = ppm_flux<real, REC>(w, up, v, cc, gpv[at2(d, i, cjg)], gpv[at2(d, i, cjg + 1)], sG[ri * QJ + c],
                                         gpv[at2(d, i, J0 + ej)], a.mt);
        }
        __syncthreads();
        // C: splitting
        for (int t = tid; t < TI * QJ; t += nth) {  // Qx: rows I0+ri, cols J0-3+cj
            int ri = t / QJ, cj = t % QJ;
            if (ri >= ni || cj >= nj + 6) continue;
            const int sq = (ri + 3) * QJ + cj;
            const real q = sQ[sq], g = sG[sq];
            real dF = -(sFx[(ri + 1) * QJ + cj] - sFx[ri * QJ + cj]);
            dF = dF * rdt / rdx;
            real out;
            if (a.split == SP_AVLT) {
                out = (q * g + real(0.5) * dF) / g;
            } else {
                const int j = J0 - 3 + cj;
                real c1 = gpu[at2(d, I0 + ri + 1, j)] * (sUa[(ri + 1) * QJ + cj] * rdt / rdx);
                real c2 = gpu[at2(d, I0 + ri, j)] * (sUa[ri * QJ + cj] * rdt / rdx);
                if (a.split == SP_L04) out = (q * g + real(0.5) * dF + real(0.5) * (c1 - c2) * q) / g;
                else out = real(0.5) * (q + (q + dF) / (real(1.0) - (c1 - c2)));
            }
            sQx[t] = out;
        }
        for (int t = tid; t < QI * TJ; t += nth) {  // Qy: rows I0-3+ri, cols J0+cj
            int ri = t / TJ, cj = t % TJ;
            if (ri >= ni + 6 || cj >= nj) continue;
            const int sq = ri * QJ + cj + 3;
            const real q = sQ[sq], g = sG[sq];
            real dF = -(sFy[ri * (TJ + 1) + cj + 1] - sFy[ri * (TJ + 1) + cj]);
            dF = dF * rdt / rdx;
            real out;
            if (a.split == SP_AVLT) {
                out = (q * g + real(0.5) * dF) / g;
            } else {
                const int i = I0 - 3 + ri;
                real c1 = gpv[at2(d, i, J0 + cj + 1)] * (sVa[ri * (TJ + 1) + cj + 1] * rdt / rdx);
                real c2 = gpv[at2(d, i, J0 + cj)] * (sVa[ri * (TJ + 1) + cj] * rdt / rdx);
                if (a.split == SP_L04) out = (q * g + real(0.5) * dF + real(0.5) * (c1 - c2) * q) / g;
                else out = real(0.5) * (q + (q + dF) / (real(1.0) - (c1 - c2)));
            }
            sQy[t] = out;
        }
        __syncthreads();
        // D: second-pass fluxes (x of Qy, y of Qx) on the tile's edges
        for (int t = tid; t < (TI + 1) * TJ; t += nth) {
            int ei = t / TJ, cj = t % TJ;
            if (ei > ni || cj >= nj) continue;
            const int wi = ei * QJ + cj + 3;  // wind index (cols offset by 3)
            const bool up = sUp[wi];
            const int c = ei + (up ? 2 : 3);  // upwind cell's row in sQy
            real w[5];
#pragma unroll
            for (int m = 0; m < 5; ++m) w[m] = sQy[(c - 2 + m) * TJ + cj];
            const int ci = I0 - 3 + c, j = J0 + cj;
            const real u = sUa[wi];
            const real cc = u * rdt / rdx;
            sFx[ei * QJ + cj + 3] = ppm_flux<real, REC>(w, up, u, cc, gpu[at2(d, ci, j)], gpu[at2(d, ci + 1, j)],
                                                        sG[c * QJ + cj + 3], gpu[at2(d, I0 + ei, j)], a.mt);
        }
        for (int t = tid; t < TI * (TJ + 1); t += nth) {
            int ri = t / (TJ + 1), ej = t % (TJ + 1);
            if (ri >= ni || ej > nj) continue;
            const int wi = (ri + 3) * (TJ + 1) + ej;
            const bool up = sVp[wi];
            const int c = ej + (up ? 2 : 3);  // upwind cell's column in sQx
            real w[5];
#pragma unroll
            for (int m = 0; m < 5; ++m) w[m] = sQx[ri * QJ + c - 2 + m];
            const int i = I0 + ri, cjg = J0 - 3 + c;
            const real v = sVa[wi];
            const real cc = v * rdt / rdx;
            sFy[(ri + 3) * (TJ + 1) + ej] = ppm_flux<real, REC>(w, up, v, cc, gpv[at2(d, i, cjg)],
                                                                gpv[at2(d, i, cjg + 1)], sG[(ri + 3) * QJ + c],
                                                                gpv[at2(d, i, J0 + ej)], a.mt);
        }
        __syncthreads();
        // E: divergence and update
        double acc = 0.0;
        for (int t = tid; t < TI * TJ; t += nth) {
            int ri = t / TJ, cj = t % TJ;
            if (ri >= ni || cj >= nj) continue;
            real dFx = -(sFx[(ri + 1) * QJ + cj + 3] - sFx[ri * QJ + cj + 3]);
            dFx = dFx * rdt / rdx;
            real dFy = -(sFy[(ri + 3) * (TJ + 1) + cj + 1] - sFy[(ri + 3) * (TJ + 1) + cj]);
            dFy = dFy * rdt / rdx;
            const int sq = (ri + 3) * QJ + cj + 3;
            const real g = sG[sq];
            const real dv = -(dFx + dFy) / (rdt * g);
            Qout[at(d, p, I0 + ri, J0 + cj)] = sQ[sq] - rdt * dv;
            if (a.mfpr) acc += (double)dv * (double)g;
        }
        if (a.mfpr) {
            red[tid] = acc;
            __syncthreads();
            for (int s = nth / 2; s > 0; s >>= 1) {
                if (tid < s) red[tid] += red[tid + s];
                __syncthreads();
            }
            if (tid == 0) a.partials[(size_t)tr * gridDim.x + blockIdx.x] = red[0];
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
    size_t reals = (size_t)(TI + 1) * QJ + QI * (TJ + 1) + QI * QJ + QI * QJ + (TI + 1) * QJ + QI * (TJ + 1) +
                   TI * QJ + QI * TJ;
    size_t bytes = reals * sizeof(real) + (size_t)(TI + 1) * QJ + QI * (TJ + 1);
    return (bytes + 15) / 16 * 16;
}

// tile shapes selectable per launch (the autotuner times them): {TI, TJ}
constexpr int FUSED_TILES[][2] = {{16, 32}, {32, 32}, {32, 64}, {64, 32}};
constexpr int FUSED_NTILE_CFG = 4;

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
    k_fused<real, REC, TI, TJ><<<NFACE * a.ntiles, 256, smem, st>>>(a);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

template <class real, int REC>
static int fused_tile(FusedArgs a, int tile, cudaStream_t st) {
    switch (tile) {
        case 0: return fused_go<real, REC, 16, 32>(a, st);
        case 1: return fused_go<real, REC, 32, 32>(a, st);
        case 2: return fused_go<real, REC, 32, 64>(a, st);
        default: return fused_go<real, REC, 64, 32>(a, st);
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

// number of CTAs of a launch with tile shape `tile`
inline int fused_blocks(const Dims &d, int tile) {
    int TI = FUSED_TILES[tile][0], TJ = FUSED_TILES[tile][1];
    return NFACE * ((d.N + TI - 1) / TI) * ((d.N + TJ - 1) / TJ);
}

}  // namespace csadv
