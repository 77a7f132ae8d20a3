// Paired-tracer line-marching step kernel of the FP32 form (k_sweep2).
//
// Same phases, tiles, work table and MF-PR bookkeeping as k_sweep (sweep.cuh), organised for
// instruction throughput, which is what bounds the FP32 step (its HBM traffic is a few percent of
// the bandwidth):
//   * The tracers of a solve are advanced two at a time.  A thread marches one grid line for a
//     pair of tracers (t, t+1) whose values of a cell sit in one 64-bit register (lanes x and y);
//     the arithmetic of both runs in Blackwell's packed FP32 instructions (add/sub/mul/fma
//     .f32x2), comparisons, minima and selections run per lane.
//   * What depends only on the wind and the metric (edge and cell records and their loads, the
//     Courant number, the upwind flag, the flux coefficients, addresses, loop control) is done
//     once for both tracers.
//   * Every operation is rounded once, in the packed and in the one-lane form alike (no
//     contraction is left to the compiler), so a solve's odd last tracer, marched alone, gets
//     the bits it would get as a member of a pair.
//   * Shared-memory row pitches are compile-time constants (61 and 55 cells: odd, so 8-byte
//     pairs are conflict-free along rows and along columns), the march loop is peeled so its
//     body carries no conditions, and its loads run one cell (smem, cell records) and two edges
//     (edge records) ahead; the reads past a line's end stay inside the tile buffers and the
//     padded global planes.
// Arithmetic follows the reference's formulas (reconstruction_1d.py:26-192, flux.py:20-128,
// discrete_operators.py:49-101), evaluated in FP32 with some products regrouped (e.g. c^2/3 is
// formed once per edge); the FP32 form's accuracy bounds are stated against the FP64 form.
#pragma once
#include "fused.cuh"
#include "halo.cuh"

namespace csadv {
namespace pairk {

typedef unsigned long long u64;

#ifndef CSADV_PAIR_UNROLL
#define CSADV_PAIR_UNROLL 0
#endif
#ifndef CSADV_UNROLL_LIGHT
#define CSADV_UNROLL_LIGHT 3
#endif
// march loop unrolling: 3 for the lighter reconstructions (PPM-0, PL07), 2 for the limited ones,
// whose longer bodies leave no registers for a third copy
template <int REC>
constexpr int pair_unroll() {
    return CSADV_PAIR_UNROLL ? CSADV_PAIR_UNROLL : (REC == REC_PPM0 || REC == REC_PL07) ? CSADV_UNROLL_LIGHT : 2;
}
#ifndef CSADV_EDGE_AHEAD
#define CSADV_EDGE_AHEAD 3
#endif
#ifndef CSADV_CELL_AHEAD
#define CSADV_CELL_AHEAD 2
#endif
// how far ahead of its use the march loads edge (2 or 3) and cell (1 or 2) records
constexpr int EDGE_AHEAD = CSADV_EDGE_AHEAD, CELL_AHEAD = CSADV_CELL_AHEAD;

// ------------------------------------------------------------------ one- and two-lane arithmetic
__device__ __forceinline__ float vadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float vsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float vmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float vfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }

__device__ __forceinline__ u64 &bits(float2 &v) { return reinterpret_cast<u64 &>(v); }
__device__ __forceinline__ float2 vadd(float2 a, float2 b) {
    float2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(bits(d)) : "l"(bits(a)), "l"(bits(b)));
    return d;
}
__device__ __forceinline__ float2 vsub(float2 a, float2 b) {
    float2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(bits(d)) : "l"(bits(a)), "l"(bits(b)));
    return d;
}
__device__ __forceinline__ float2 vmul(float2 a, float2 b) {
    float2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(bits(d)) : "l"(bits(a)), "l"(bits(b)));
    return d;
}
__device__ __forceinline__ float2 vfma(float2 a, float2 b, float2 c) {
    float2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(bits(d)) : "l"(bits(a)), "l"(bits(b)), "l"(bits(c)));
    return d;
}

// min(a, b, c) of three non-NaN floats, one three-input instruction (sm_100 and later)
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

template <class V> struct Lanes;
template <> struct Lanes<float> { static constexpr int n = 1; };
template <> struct Lanes<float2> { static constexpr int n = 2; };

template <class V> __device__ __forceinline__ V bc(float s);
template <> __device__ __forceinline__ float bc<float>(float s) { return s; }
template <> __device__ __forceinline__ float2 bc<float2>(float s) { return make_float2(s, s); }

__device__ __forceinline__ float lane(const float &v, int) { return v; }
__device__ __forceinline__ float lane(const float2 &v, int l) { return l ? v.y : v.x; }
__device__ __forceinline__ void set_lane(float &v, int, float x) { v = x; }
__device__ __forceinline__ void set_lane(float2 &v, int l, float x) {
    if (l) v.y = x;
    else v.x = x;
}

// ------------------------------------------------------------------ reconstructions
// The reconstructions work in doubled units: slopes, edge values and parabolas are carried as
// twice their value (2 L, 2 R, 2 q), which is exact, removes the halving constants from the
// packed arithmetic (every constant pair of a packed operation occupies two registers), and
// leaves every comparison of the limiters unchanged.  The flux folds the factor 1/2 into the
// wind (F = F2 u / 2).

// twice the CW84 limited slope of the cell between qm and qp (reconstruction_1d.py:64-100):
// with dp = qp - q0, dm = q0 - qm: copysign(min(|qp - qm|, 4|dp|, 4|dm|), qp - qm) when
// dp dm > 0, else 0; D1 = 4 dp and D2 = 4 dm are supplied (the march carries them)
template <class V>
__device__ __forceinline__ V cw84_slope2(V qm, V qp, V dp, V D1, V dm, V D2) {
    const V D0 = vsub(qp, qm);
    const V pr = vmul(dp, dm);
    V s;
#pragma unroll
    for (int l = 0; l < Lanes<V>::n; ++l) {
        const float m = fmin3(fabsf(lane(D0, l)), fabsf(lane(D1, l)), fabsf(lane(D2, l)));
        set_lane(s, l, lane(pr, l) > 0.f ? copysignf(m, lane(D0, l)) : 0.f);
    }
    return s;
}
template <class V>
__device__ __forceinline__ V times4(V x) {
    const V t = vadd(x, x);
    return vadd(t, t);
}
// CW84 monotonicity limiter (reconstruction_1d.py:102-153) on the doubled offsets U = 2 (R - q),
// Vv = 2 (q - L) of a cell's parabola: the reference's extremum test (R - q)(q - L) <= 0 flattens
// the cell (both offsets 0); otherwise (U, Vv of one sign; dq = u + v and q6 = 3 (v - u)) its
// overshoot tests |dq| < |q6| and dq (q - (R + L)/2) >< +-dq^2/6 hold exactly when |v| > 2|u|
// (L moves to 3q - 2R: v becomes 2u) or |u| > 2|v| (R moves to 3q - 2L: u becomes 2v).  At the
// ties a rounding could decide, both branches give the same parabola.
template <class V>
__device__ __forceinline__ void cw84_limit_ofs2(V U, V Vv, V &uo, V &vo) {
    const V U2 = vadd(U, U), V2 = vadd(Vv, Vv);
    const V pf = vmul(U, Vv);
#pragma unroll
    for (int l = 0; l < Lanes<V>::n; ++l) {
        const bool flat = lane(pf, l) <= 0.f;
        const bool ml = !flat && fabsf(lane(Vv, l)) > fabsf(lane(U2, l));
        const bool mr = !flat && fabsf(lane(U, l)) > fabsf(lane(V2, l));
        set_lane(uo, l, flat ? 0.f : (mr ? lane(V2, l) : lane(U, l)));
        set_lane(vo, l, flat ? 0.f : (ml ? lane(U2, l) : lane(Vv, l)));
    }
}
// twice the L04 monotone slope of the cell q0 between qm and qp (reconstruction_1d.py:155-172)
template <class V>
__device__ __forceinline__ V l04_mono2(V qm, V q0, V qp) {
    const V dq = vmul(vsub(qp, qm), bc<V>(0.5f));
    V r;
#pragma unroll
    for (int l = 0; l < Lanes<V>::n; ++l) {
        const float a = lane(qm, l), b = lane(q0, l), c = lane(qp, l);
        const float dmin = __fsub_rn(fmaxf(fmaxf(a, b), c), b);
        const float dmax = __fsub_rn(b, fminf(fminf(a, b), c));
        const float m = fminf(fminf(fabsf(lane(dq, l)), __fadd_rn(dmin, dmin)), __fadd_rn(dmax, dmax));
        set_lane(r, l, copysignf(m, lane(dq, l)));
    }
    return r;
}
// twice the L04 edge value: (qa + qb) - (Mb - Ma) / 3 with doubled slopes
template <class V>
__device__ __forceinline__ V l04_edge2(V qa, V qb, V Ma, V Mb) {
    return vfma(vsub(Mb, Ma), bc<V>(-1.0f / 3.0f), vadd(qa, qb));
}
// L04 limiter (reconstruction_1d.py:174-192) on doubled values: L = q - copysign(min(2|m|,
// |L - q|), m), R = q + copysign(min(2|m|, |R - q|), m)
template <class V>
__device__ __forceinline__ void l04_limit2(V Q2, V M2, V &L2, V &R2) {
    const V dL = vsub(L2, Q2), dR = vsub(R2, Q2);
#pragma unroll
    for (int l = 0; l < Lanes<V>::n; ++l) {
        const float m = lane(M2, l), a = __fadd_rn(fabsf(m), fabsf(m));
        set_lane(L2, l, __fsub_rn(lane(Q2, l), copysignf(fminf(a, fabsf(lane(dL, l))), m)));
        set_lane(R2, l, __fadd_rn(lane(Q2, l), copysignf(fminf(a, fabsf(lane(dR, l))), m)));
    }
}
// twice the PPM-0 4-point edge value between cells a and b (reconstruction_1d.py:33-44)
template <class V>
__device__ __forceinline__ V ppm0_edge2(V qam, V qa, V qb, V qbp) {
    return vfma(vadd(qb, qa), bc<V>(7.0f / 6.0f), vmul(vadd(qbp, qam), bc<V>(-1.0f / 6.0f)));
}

// Marching reconstruction: init() with the window q(ma-3..ma+1) prepares cell ma-1; cell() with
// the window w = q(m-2..m+2) gives the doubled parabola (L2, R2) of cell m and advances.
template <int REC, class V>
struct Recon {
    // doubled slope of the current cell; doubled left edge value (CW84: the doubled offset
    // 2 (q - L) of the current cell instead); q(m+1) - q(m), 4 times it
    V s, E, dp, D1;
    __device__ __forceinline__ void init(const V w[5]) {
        if (REC == REC_CW84) {
            const V dpa = vsub(w[2], w[1]), dma = vsub(w[1], w[0]);
            const V D1a = times4(dpa);
            const V sa = cw84_slope2(w[0], w[2], dpa, D1a, dma, times4(dma));
            dp = vsub(w[3], w[2]);
            D1 = times4(dp);
            s = cw84_slope2(w[1], w[3], dp, D1, dpa, D1a);
            E = vfma(vsub(s, sa), bc<V>(1.0f / 6.0f), dpa);  // 2 (q(m) - E(m - 1/2))
        } else if (REC == REC_L04) {
            const V sa = l04_mono2(w[0], w[1], w[2]);
            s = l04_mono2(w[1], w[2], w[3]);
            E = l04_edge2(w[1], w[2], sa, s);
        } else if (REC == REC_PPM0) {
            E = ppm0_edge2(w[0], w[1], w[2], w[3]);
        }
    }
    // the cell's doubled parabola (L, R); CW84: its doubled limited offsets (L <- 2 (q - L'),
    // R <- 2 (R' - q)).  With d = q(m+1) - q(m) and dS the doubled slopes' difference, the doubled
    // edge value between the cells gives 2 (E - q(m)) = d - dS/6 and 2 (q(m+1) - E) = d + dS/6.
    __device__ __forceinline__ void cell(const V w[5], V &L, V &R) {
        if (REC == REC_CW84) {
            const V dpn = vsub(w[4], w[3]);
            const V D1n = times4(dpn);
            const V sn = cw84_slope2(w[2], w[4], dpn, D1n, dp, D1);
            const V dS = vsub(sn, s);
            const V U = vfma(dS, bc<V>(-1.0f / 6.0f), dp), Vn = vfma(dS, bc<V>(1.0f / 6.0f), dp);
            cw84_limit_ofs2(U, E, R, L);
            s = sn;
            E = Vn;
            dp = dpn;
            D1 = D1n;
        } else if (REC == REC_L04) {
            const V sn = l04_mono2(w[2], w[3], w[4]);
            const V En = l04_edge2(w[2], w[3], s, sn);
            L = E;
            R = En;
            l04_limit2(vadd(w[2], w[2]), s, L, R);
            s = sn;
            E = En;
        } else if (REC == REC_PPM0) {
            const V En = ppm0_edge2(w[1], w[2], w[3], w[4]);
            L = E;
            R = En;
            E = En;
        } else {  // PL07 hybrid 5-point values (reconstruction_1d.py:46-62), doubled
            const V a1 = bc<V>(2.0f / 30.0f), a2 = bc<V>(-13.0f / 30.0f), a3 = bc<V>(47.0f / 30.0f),
                    a4 = bc<V>(27.0f / 30.0f), a5 = bc<V>(-3.0f / 30.0f);
            R = vfma(a5, w[4], vfma(a4, w[3], vfma(a3, w[2], vfma(a2, w[1], vmul(a1, w[0])))));
            L = vfma(a1, w[4], vfma(a2, w[3], vfma(a3, w[2], vfma(a4, w[1], vmul(a5, w[0])))));
        }
    }
};

// ------------------------------------------------------------------ the march
enum { M_SPLIT = 0, M_DIFF = 1, M_UPDATE = 2 };

// One grid line of the tile for one or two tracers.  Cell m (tile-local, 0 = the tile's first
// interior cell along the line) is at line[m * SS] in shared memory; the records of edge m (its
// left edge) and of cell m are erec[m * P] and crec[m * P] in global memory.  Cells [ma, mb) get
// outputs, from the fluxes through edges [ma, mb]:
//   M_SPLIT : split field of the first pass -> out[k * OS]             (discrete_operators.py:49-73)
//   M_DIFF  : flux difference F(k+1) - F(k) -> out[k * OS]
//   M_UPDATE: Q(k) - dt div(k) -> qo0/qo1[k * P] (lanes x/y), with the y-flux differences
//             dy[k * OS] and Q(k) at qc[k * PAIR_QJP]; sums of div g and of the new Q g per lane
//             into acc / accm (MF-PR, discrete_operators.py:80-101)
template <int REC, int SPL, int MODE, class V>
struct Marcher {
    static constexpr bool MT0 = SPL != SP_PL07;
    int SS, OS;             // strides of the line and of the output in shared memory (elements)
    const V *win;
    const float2 *ef, *cf;  // next edge / cell record to load
    int P;
    float dtdx;
    V w[5];
    Recon<REC, V> rc;
    float2 eA, eB, cC, cP;  // edges m, m+1; cells m, m-1
    float2 eC, cD;          // edge m+2, cell m+1 (deeper lookahead)
    V pU, pV, pQ, Fp;       // previous cell's (metric-weighted) parabola as offsets from its mean, the mean;
                            // flux through edge m-1
    float cmp;              // g u dt/dx at edge m-1 (SP-L04, SP-PL07)
    V *out;
    const V *dy, *qc;
    float *qo0, *qo1;
    V acc, accm;

    __device__ __forceinline__ void start(const V *line, int ss, int os, const float2 *erec, const float2 *crec, int P_,
                                          int ma) {
        SS = ss;
        OS = os;
        P = P_;
        const V *s = line + (ma - 3) * SS;
#pragma unroll
        for (int k = 0; k < 5; ++k) w[k] = s[k * SS];
        win = s + 5 * SS;
        rc.init(w);
        const float2 *e = erec + (long long)(ma - 1) * P;
        eA = __ldg(e);
        eB = __ldg(e + P);
        if (EDGE_AHEAD == 3) eC = __ldg(e + 2 * (long long)P);
        ef = e + EDGE_AHEAD * (long long)P;
        const float2 *c = crec + (long long)(ma - 1) * P;
        cC = __ldg(c);
        if (CELL_AHEAD == 2) cD = __ldg(c + P);
        cf = c + CELL_AHEAD * (long long)P;
    }

    // iteration m: parabola of cell m; with FLUX the flux through edge m; with OUT the output of
    // cell m - 1
    template <bool FLUX, bool OUT>
    __device__ __forceinline__ void step() {
        const V wn = *win;
        win += SS;
        const float2 eN = __ldg(ef);
        ef += P;
        const float2 cN = __ldg(cf);
        cf += P;

        V L, R;  // doubled (CW84: the doubled offsets, L <- 2 (q - L), R <- 2 (R - q))
        rc.cell(w, L, R);
        const float gl = fabsf(eA.y);
        // the (MT-0: metric-weighted, flux.py:28-31) parabola as offsets from its weighted mean:
        // cu = R - q, cv = q - L, doubled; cQ the weighted doubled mean
        V cu, cv, cQ;
        if (REC == REC_CW84) {
            const V Q2 = vadd(w[2], w[2]);
            if (MT0) {  // gR (q + u) - g q = gR u + (gR - g) q, g q - gL (q - v) = gL v + (g - gL) q
                const float gr = fabsf(eB.y), g = cC.x;
                cQ = vmul(Q2, bc<V>(g));
                cu = vfma(R, bc<V>(gr), vmul(Q2, bc<V>(__fsub_rn(gr, g))));
                cv = vfma(L, bc<V>(gl), vmul(Q2, bc<V>(__fsub_rn(g, gl))));
            } else {
                cQ = Q2;
                cu = R;
                cv = L;
            }
        } else {
            V cL = L, cR = R;
            if (MT0) {
                cL = vmul(L, bc<V>(gl));
                cR = vmul(R, bc<V>(fabsf(eB.y)));
                cQ = vmul(w[2], bc<V>(__fadd_rn(cC.x, cC.x)));
            } else {
                cQ = vadd(w[2], w[2]);
            }
            cu = vsub(cR, cQ);
            cv = vsub(cQ, cL);
        }
        if (FLUX) {
            // upwind PPM flux through edge m (flux.py:20-128): the parabola of cell m-1 when the
            // wind is >= 0, of cell m otherwise.  The reference's e + c/2 (q6 -+ dq) - q6 c^2/3 with
            // dq = u + v and q6 = 3 (v - u) in the upwind cell's offsets is q + A u + B v with
            // A = (1 - c)^2, B = c (1 - c) (wind >= 0) or A = c (1 + c), B = -(1 + c)^2; doubled
            // units, times u / 2
            const float u = eA.x;
            const bool up = !signbit(eA.y);
            const float c = __fmul_rn(u, dtdx);
            const float sc = up ? __fsub_rn(1.f, c) : __fadd_rn(1.f, c);
            const float ss = __fmul_rn(sc, sc), cs = __fmul_rn(c, sc);
            const float A = up ? ss : cs, B = up ? cs : -ss;
            // both cells' candidates in packed arithmetic, then one selection per lane
            const V Fu = vfma(pV, bc<V>(B), vfma(pU, bc<V>(A), pQ));
            const V Fd = vfma(cv, bc<V>(B), vfma(cu, bc<V>(A), cQ));
            V F;
#pragma unroll
            for (int l = 0; l < Lanes<V>::n; ++l) set_lane(F, l, up ? lane(Fu, l) : lane(Fd, l));
            F = vmul(F, bc<V>(MT0 ? __fmul_rn(0.5f, u) : __fmul_rn(__fmul_rn(0.5f, u), gl)));
            const float cm = __fmul_rn(gl, c);
            if (OUT) {
                const V dF = vsub(F, Fp);  // F(k+1) - F(k), k = m - 1
                if (MODE == M_SPLIT) {
                    const V q = w[1];
                    V o;
                    if (SPL == SP_AVLT) {  // Q + dF / 2 with dF = -(F(k+1) - F(k)) dt/dx / g
                        o = vfma(dF, bc<V>(__fmul_rn(cP.y, -0.5f * dtdx)), q);
                    } else if (SPL == SP_L04) {  // (Q g + dF / 2 + (c_k+1 - c_k) Q / 2) / g
                        const float a = __fadd_rn(cP.x, __fmul_rn(0.5f, __fsub_rn(cm, cmp)));
                        o = vmul(vfma(q, bc<V>(a), vmul(dF, bc<V>(-0.5f * dtdx))), bc<V>(cP.y));
                    } else {  // (Q + (Q + dF) / (1 - (c_k+1 - c_k))) / 2
                        const float r = __frcp_rn(__fsub_rn(1.f, __fsub_rn(cm, cmp)));
                        o = vmul(vadd(q, vmul(vfma(dF, bc<V>(-dtdx), q), bc<V>(r))), bc<V>(0.5f));
                    }
                    *out = o;
                    out += OS;
                } else if (MODE == M_DIFF) {
                    *out = dF;
                    out += OS;
                } else {
                    const V sdiv = vadd(dF, *dy);
                    dy += OS;
                    const V qn = vfma(sdiv, bc<V>(-__fmul_rn(dtdx, cP.y)), *qc);
                    qc += PAIR_QJP;
                    *qo0 = lane(qn, 0);
                    qo0 += P;
                    if (Lanes<V>::n == 2) {
                        *qo1 = lane(qn, 1);
                        qo1 += P;
                    }
                    // (accumulated unconditionally: a branch here would cost more than the sums)
                    acc = vfma(sdiv, bc<V>(__fmul_rn(cP.y, __fmul_rn(irdx, cP.x))), acc);
                    accm = vfma(qn, bc<V>(cP.x), accm);
                }
            }
            Fp = F;
            cmp = cm;
        }
        pU = cu;
        pV = cv;
        pQ = cQ;
        cP = cC;
        eA = eB;
        if (EDGE_AHEAD == 3) {
            eB = eC;
            eC = eN;
        } else {
            eB = eN;
        }
        if (CELL_AHEAD == 2) {
            cC = cD;
            cD = cN;
        } else {
            cC = cN;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) w[k] = w[k + 1];
        w[4] = wn;
    }
    float irdx;

    // march over cells [ma - 1, mb]
    __device__ __forceinline__ void run(int ma, int mb) {
        step<false, false>();
        step<true, false>();
        constexpr int U = pair_unroll<REC>();
#pragma unroll U
        for (int m = ma + 1; m <= mb; ++m) step<true, true>();
    }
};

// ------------------------------------------------------------------ one tile, one or two tracers
// Phases as in k_sweep: P0 Q (+ halo) -> shared; P1 first-pass x- and y-lines -> Qx, Qy;
// P2 y-lines of Qx -> dY; P3 x-lines of Qy -> div, update, MF-PR partial(s).  Every phase has
// at most one line segment per thread (the segment counts are chosen so).
template <int REC, int SPL, class V>
__device__ __forceinline__ void tile_pass(const SweepSolve &S, int p, int item, int tr, int I0, int ni, int J0, int nj,
                                          unsigned char *smem_raw, double *red) {
    constexpr int NL = Lanes<V>::n;
    constexpr int QJP = PAIR_QJP, TJP = PAIR_TJP;
    const int tid = threadIdx.x, lane_id = tid & 31, warp = tid >> 5;
    constexpr int NWARP = SWEEP_THREADS / 32;
    const Dims d = S.d;
    const int P = d.pitch;
    const long long pofs = (long long)p * d.plane;
    const PairSmem L = pair_smem(S.ti);
    V *sm = (V *)smem_raw;
    V *sQ = sm, *sQx = sm + L.oQx, *sQy = sm + L.oQy, *sDy = sm + L.oDy;
    const float dtdx = S.dtdx, irdx = S.irdx;
    const float2 *erx = (const float2 *)S.erx + pofs, *ery = (const float2 *)S.ery + pofs;
    const float2 *crx = (const float2 *)S.crx, *cry = (const float2 *)S.cry;
    const float *gpc = (const float *)S.gpc;
    const bool hc = S.corr_in != nullptr;

    // the pending MF-PR corrections of the pair, rounded to FP32 once per CTA (GB300 converts from
    // FP64 at the FP64 rate) and shared through shared memory
    float *scorr = (float *)(red + SWEEP_THREADS - 2);
    if (tid < NL) scorr[tid] = hc ? (float)S.corr_in[tr + tid] : 0.f;
    // The first-pass lines read the edge and cell records of the tile from global memory, one to
    // two cells ahead of their use; after the records have left L2 (the first pair of a step)
    // that is not far enough to hide a DRAM access, so every thread first asks L2 for a few
    // 128-byte lines of them (x-lines: rows I0-1 .. I0+ni+2 of erx, crx from column J0-3;
    // y-lines: the same of the transposed ery, cry), which then arrive while Q is loaded.
    if (tr == 0) {
        const int rx = ni + 4, ry = nj + 4, nl = 5;  // rows per array; lines per row (<= 61 records)
        const int total = 2 * (rx + ry) * nl;
        for (int k = tid; k < total; k += SWEEP_THREADS) {
            const int l = k % nl, rowk = k / nl;
            const float2 *base;
            if (rowk < 2 * rx) {
                const int row = rowk >> 1;
                base = ((rowk & 1) ? crx : erx) + (long long)(I0 - 1 + row) * P + (J0 - 3);
            } else {
                const int row = (rowk - 2 * rx) >> 1;
                base = ((rowk & 1) ? cry : ery) + (long long)(J0 - 1 + row) * P + (I0 - 3);
            }
            const char *a = (const char *)base + 128 * l;
            asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
        }
    }
    {   // the Q and metric rows that the tile load reads in its second round (rows 32..)
        const int r0 = 4 * (SWEEP_THREADS / 32), R = ni + 6, nrow = R > r0 ? R - r0 : 0;
        const int narr = Lanes<V>::n + (hc ? 1 : 0);
        for (int k = tid; k < nrow * narr * 3; k += SWEEP_THREADS) {
            const int l = k % 3, ra = k / 3, a = ra / nrow, r = r0 + ra % nrow;
            const float *base = (a < Lanes<V>::n ? (const float *)S.Qin + (long long)(tr + a) * d.field + pofs : gpc) +
                                (long long)(I0 - 3 + r) * P + (J0 - 3);
            const char *ad = (const char *)base + 128 * l;
            asm volatile("prefetch.global.L2 [%0];" ::"l"(ad));
        }
    }
    __syncthreads();

    // P0: Q on the tile + 3 halo cells; interior cells with the pending MF-PR correction.  Warp w
    // takes rows w, w + 8, ...; all loads of a thread are issued before its first store.
    {
        const float *Qt[2];
        float corr[2];
#pragma unroll
        for (int l = 0; l < NL; ++l) {
            Qt[l] = (const float *)S.Qin + (long long)(tr + l) * d.field + pofs;
            corr[l] = scorr[l];
        }
        // interior cells, and ghost cells as the ghost-cell kernel filled them (or, with inline
        // ghost cells, left for the evaluation below)
        const bool inl = S.lag_w != nullptr;
        constexpr int RR = 4, CC = (SWEEP_TMAX + 6 + 31) / 32;  // cells per batch: RR x CC
        for (int r0 = warp; r0 < ni + 6; r0 += RR * NWARP) {
            float q[RR][CC][NL], g[RR][CC];
#pragma unroll
            for (int a = 0; a < RR; ++a) {
                const int r = r0 + a * NWARP, i = I0 - 3 + r;
                const float *q0 = Qt[0] + (long long)i * P + J0 - 3 + lane_id;
#pragma unroll
                for (int b = 0; b < CC; ++b) {
                    if (r < ni + 6 && lane_id + 32 * b < nj + 6) {
#pragma unroll
                        for (int l = 0; l < NL; ++l) q[a][b][l] = __ldg(q0 + 32 * b + (l ? d.field : 0));
                        g[a][b] = hc ? __ldg(gpc + (q0 - Qt[0]) + 32 * b) : 0.f;
                    }
                }
            }
#pragma unroll
            for (int a = 0; a < RR; ++a) {
                const int r = r0 + a * NWARP, i = I0 - 3 + r;
#pragma unroll
                for (int b = 0; b < CC; ++b) {
                    const int c = lane_id + 32 * b, j = J0 - 3 + c;
                    const bool interior = i >= d.i0 && i < d.iend && j >= d.i0 && j < d.iend;
                    if (r < ni + 6 && c < nj + 6 && (interior || !inl)) {
                        V v;
#pragma unroll
                        for (int l = 0; l < NL; ++l)
                            set_lane(v, l, interior && hc ? corrected(q[a][b][l], g[a][b], corr[l]) : q[a][b][l]);
                        sQ[r * QJP + c] = v;
                    }
                }
            }
        }
        if (inl) {
            // inline ghost cells (ET-DG, interpolation.py:154-314): the part of the tile's 3-cell
            // ring outside the panel, from the neighbouring panels' interior values, with the
            // same device functions (and so the same bits) as the ghost-cell kernel.  Strips:
            // rows [-3, 0) / [ni, ni+3) over the full width at the panel's first / last row; then
            // columns [-3, 0) / [nj, nj+3) at its first / last column, over the ring's rows that
            // those row strips do not cover.
            const bool wr = I0 == d.i0, er = I0 + ni == d.iend;
            const int W6 = nj + 6, r_lo = wr ? 0 : -3, nr = (er ? ni : ni + 3) - r_lo;
            const int cw = wr ? 3 * W6 : 0, ce = er ? 3 * W6 : 0;
            const int cs = J0 == d.i0 ? 3 * nr : 0, cn = J0 + nj == d.iend ? 3 * nr : 0;
            for (int k = tid; k < cw + ce + cs + cn; k += SWEEP_THREADS) {
                int r, c;
                if (k < cw) {
                    r = -3 + k / W6;
                    c = -3 + k % W6;
                } else if (k < cw + ce) {
                    r = ni + (k - cw) / W6;
                    c = -3 + (k - cw) % W6;
                } else if (k < cw + ce + cs) {
                    r = r_lo + (k - cw - ce) / 3;
                    c = -3 + (k - cw - ce) % 3;
                } else {
                    r = r_lo + (k - cw - ce - cs) / 3;
                    c = nj + (k - cw - ce - cs) % 3;
                }
                V v;
                if constexpr (Lanes<V>::n == 2) {  // one table load serves both tracers
                    const float *F0 = (const float *)S.Qin + (long long)tr * d.field;
                    v = ghost_table_f2(F0, F0 + d.field, gpc, corr[0], corr[1], hc, d, S.gside, S.gcorner, p, I0 + r,
                                       J0 + c);
                } else {
                    const Src<float> src{(const float *)S.Qin + (long long)tr * d.field, gpc, corr[0], hc};
                    set_lane(v, 0, ghost_table_f(src, d, S.gside, S.gcorner, p, I0 + r, J0 + c));
                }
                sQ[(r + 3) * QJP + c + 3] = v;
            }
        }
    }
    __syncthreads();
    // P1: x-lines over columns c in [-3, nj+3), cells [0, ni) -> Qx;
    //     y-lines over rows r in [-3, ni+3), cells [0, nj) -> Qy
    // (one code path for both directions: the line's strides and records are arguments)
    {
        const int LX = nj + 6, LY = ni + 6;  // jobs packed densely: no idle lanes between lines
        const int jx = S.s1x * LX, job = tid;
        bool go = false;
        const V *line = nullptr;
        V *out = nullptr;
        const float2 *er = nullptr, *cr = nullptr;
        int ss = 1, os = 1, ma = 0, mb = 0;
        if (job < jx) {
            const int seg = job / LX, c = job - seg * LX - 3;
            ma = ni * seg / S.s1x;
            mb = ni * (seg + 1) / S.s1x;
            go = c < nj + 3 && ma < mb;
            const long long g0 = (long long)I0 * P + J0 + c;
            line = sQ + 3 * QJP + c + 3;
            ss = os = QJP;
            er = erx + g0;
            cr = crx + g0;
            out = sQx + ma * QJP + c + 3;
        } else if (job < jx + S.s1y * LY) {
            const int jj = job - jx;
            const int seg = jj / LY, r = jj - seg * LY - 3;
            ma = nj * seg / S.s1y;
            mb = nj * (seg + 1) / S.s1y;
            go = r < ni + 3 && ma < mb;
            const long long g0 = (long long)J0 * P + I0 + r;
            line = sQ + (r + 3) * QJP + 3;
            er = ery + g0;
            cr = cry + g0;
            out = sQy + (r + 3) * TJP + ma;
        }
        if (go) {
            Marcher<REC, SPL, M_SPLIT, V> mr;
            mr.dtdx = dtdx;
            mr.irdx = irdx;
            mr.start(line, ss, os, er, cr, P, ma);
            mr.out = out;
            mr.run(ma, mb);
        }
    }
    __syncthreads();
    // P2: y-lines of Qx over rows [0, ni): second-pass y-flux differences -> dY
    {
        const int LY = ni;
        const int job = tid;
        if (job < S.s2y * LY) {
            const int seg = job / LY, r = job - seg * LY;
            const int ma = nj * seg / S.s2y, mb = nj * (seg + 1) / S.s2y;
            if (r < ni && ma < mb) {
                const long long g0 = (long long)J0 * P + I0 + r;
                Marcher<REC, SPL, M_DIFF, V> mr;
                mr.dtdx = dtdx;
                mr.irdx = irdx;
                mr.start(sQx + r * QJP + 3, 1, 1, ery + g0, cry + g0, P, ma);
                mr.out = sDy + r * TJP + ma;
                mr.run(ma, mb);
            }
        }
    }
    __syncthreads();
    // P3: x-lines of Qy over columns [0, nj): second-pass x fluxes, div, update, MF-PR partials
    V acc = bc<V>(0.f), accm = bc<V>(0.f);
    {
        const int LX = nj;
        const int job = tid;
        if (job < S.s2x * LX) {
            const int seg = job / LX, c = job - seg * LX;
            const int ma = ni * seg / S.s2x, mb = ni * (seg + 1) / S.s2x;
            if (c < nj && ma < mb) {
                const long long g0 = (long long)I0 * P + J0 + c;
                Marcher<REC, SPL, M_UPDATE, V> mr;
                mr.dtdx = dtdx;
                mr.irdx = irdx;
                mr.start(sQy + 3 * TJP + c, TJP, TJP, erx + g0, crx + g0, P, ma);
                mr.dy = sDy + ma * TJP + c;
                mr.qc = sQ + (ma + 3) * QJP + c + 3;
                mr.qo0 = (float *)S.Qout + (long long)tr * d.field + pofs + g0 + (long long)ma * P;
                mr.qo1 = mr.qo0 + d.field;
                mr.acc = acc;
                mr.accm = accm;
                mr.run(ma, mb);
                acc = mr.acc;
                accm = mr.accm;
            }
        }
    }
    if (S.mfpr) {  // per tracer: FP32 within a warp (fixed butterfly order), FP64 across warps
        const bool anchor = S.mass_target != nullptr;
        const int nitems = NFACE * S.ntiles;
#pragma unroll
        for (int l = 0; l < NL; ++l) {
            float x = anchor ? lane(accm, l) : lane(acc, l);
            for (int o = 16; o > 0; o >>= 1) x = __fadd_rn(x, __shfl_xor_sync(0xffffffffu, x, o));
            if (lane_id == 0) red[l * NWARP + warp] = (double)x;
        }
        __syncthreads();
        if (tid < NL) {
            double s = 0.0;
            for (int w = 0; w < NWARP; ++w) s += red[tid * NWARP + w];
            S.partials[(long long)(tr + tid) * nitems + item] = s;
        }
    }
    __syncthreads();
}

// SPL: the splitting (SP_AVLT, SP_L04 with MT-0; SP_PL07 with MT-PL07), fixed per kernel
// TG: how the launch groups the tracers of its solves (SWEEP_TG_*): pairs only (every T even),
// one at a time (T = 1), or pairs and an odd last one (any T).  Each grouping is its own kernel so
// that the pair and single paths do not share one register allocation.
template <int REC, int SPL, int TG>
__global__ void __launch_bounds__(SWEEP_THREADS, 2) k_sweep2(const SweepSolve *__restrict__ solves,
                                                           const int2 *__restrict__ work, int nwork) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double red[SWEEP_THREADS];
    __shared__ int last;
    const int tid = threadIdx.x;

    for (int wk = blockIdx.x; wk < nwork; wk += gridDim.x) {
        const int2 it = work ? work[wk] : make_int2(0, wk);
        const SweepSolve &S = solves[it.x];
        const int ntiles = S.ntiles, nitems = NFACE * ntiles;
        const int tile = it.y % ntiles, p = it.y / ntiles;
        int I0, ni, J0, nj;
        sweep_tile(S, tile, I0, ni, J0, nj);
        const int T = S.T;
        if (TG == SWEEP_TG_PAIRS) {
            for (int tr = 0; tr + 1 < T; tr += 2) tile_pass<REC, SPL, float2>(S, p, it.y, tr, I0, ni, J0, nj, smem_raw, red);
        } else if (TG == SWEEP_TG_ONE) {
            for (int tr = 0; tr < T; ++tr) tile_pass<REC, SPL, float>(S, p, it.y, tr, I0, ni, J0, nj, smem_raw, red);
        } else {
            for (int tr = 0; tr < T; tr += 2) {
                if (tr + 1 < T)
                    tile_pass<REC, SPL, float2>(S, p, it.y, tr, I0, ni, J0, nj, smem_raw, red);
                else
                    tile_pass<REC, SPL, float>(S, p, it.y, tr, I0, ni, J0, nj, smem_raw, red);
            }
        }
        if (S.mfpr) {
            // the last item of the solve to finish sums its partials: corr = dt m0 / a2, or (FP32
            // mass anchor) the correction that restores the recorded mass
            if (tid == 0) {
                __threadfence();
                const unsigned int prev = atomicAdd(S.counter, 1u);
                last = prev == (unsigned int)nitems - 1u;
            }
            __syncthreads();
            if (last) {
                // fixed order: each thread sums items tid, tid + 256, ...; a warp butterfly (the
                // same bits in every lane); the 8 warp sums in warp order.  Tracers two at a time
                // (their partials read together), up to 32 per barrier.
                __threadfence();
                constexpr int NW = SWEEP_THREADS / 32, TB = SWEEP_THREADS / NW;
                const int lane_id = tid & 31, warp = tid >> 5;
                for (int t0 = 0; t0 < T; t0 += TB) {
                    const int nt = T - t0 < TB ? T - t0 : TB;
                    for (int k = 0; k < nt; k += 2) {
                        const bool two = k + 1 < nt;
                        const double *p0 = S.partials + (long long)(t0 + k) * nitems, *p1 = p0 + nitems;
                        double a0 = 0.0, a1 = 0.0;
                        for (int b = tid; b < nitems; b += SWEEP_THREADS) {
                            a0 = __dadd_rn(a0, __ldcg(p0 + b));
                            if (two) a1 = __dadd_rn(a1, __ldcg(p1 + b));
                        }
#pragma unroll
                        for (int o = 16; o > 0; o >>= 1) {
                            a0 = __dadd_rn(a0, __shfl_xor_sync(0xffffffffu, a0, o));
                            a1 = __dadd_rn(a1, __shfl_xor_sync(0xffffffffu, a1, o));
                        }
                        if (lane_id == 0) {
                            red[k * NW + warp] = a0;
                            if (two) red[(k + 1) * NW + warp] = a1;
                        }
                    }
                    __syncthreads();
                    if (tid < nt) {
                        double sum = 0.0;
#pragma unroll
                        for (int w = 0; w < NW; ++w) sum = __dadd_rn(sum, red[tid * NW + w]);
                        const int tr = t0 + tid;
                        S.corr_out[tr] = S.mass_target ? (S.mass_target[tr] - sum) / S.a2 : S.dt * sum / S.a2;
                    }
                    __syncthreads();
                }
                if (tid == 0) *S.counter = 0u;
            }
            __syncthreads();
        }
    }
}

template <int REC, int SPL, int TG>
int go(const SweepSolve *dsolves, const int2 *work, int nwork, int grid, size_t smem, cudaStream_t st) {
    if (st == (cudaStream_t)-1) {  // prepare only: allow the largest layout
        size_t mx = 0;
        for (int c = 0; c < SWEEP_NTILE_CFG; ++c) mx = mx > sweep_smem_bytes<float>(c) ? mx : sweep_smem_bytes<float>(c);
        CSADV_CUDA(cudaFuncSetAttribute(k_sweep2<REC, SPL, TG>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mx));
        return CSADV_OK;
    }
    k_sweep2<REC, SPL, TG><<<grid, SWEEP_THREADS, smem, st>>>(dsolves, work, nwork);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

template <int REC, int TG>
int split(int spl, const SweepSolve *dsolves, const int2 *work, int nwork, int grid, size_t smem, cudaStream_t st) {
    switch (spl) {
        case SP_AVLT: return go<REC, SP_AVLT, TG>(dsolves, work, nwork, grid, smem, st);
        case SP_L04: return go<REC, SP_L04, TG>(dsolves, work, nwork, grid, smem, st);
        default: return go<REC, SP_PL07, TG>(dsolves, work, nwork, grid, smem, st);
    }
}

// the kernels of one tracer grouping (each grouping is instantiated in its own translation unit)
template <int TG>
int launch_group(int recon, int spl, const SweepSolve *dsolves, const int2 *work, int nwork, int grid, size_t smem,
                 cudaStream_t st) {
    switch (recon) {
        case REC_PPM0: return split<REC_PPM0, TG>(spl, dsolves, work, nwork, grid, smem, st);
        case REC_CW84: return split<REC_CW84, TG>(spl, dsolves, work, nwork, grid, smem, st);
        case REC_PL07: return split<REC_PL07, TG>(spl, dsolves, work, nwork, grid, smem, st);
        default: return split<REC_L04, TG>(spl, dsolves, work, nwork, grid, smem, st);
    }
}

}  // namespace pairk
}  // namespace csadv
