// Line-marching step kernel of the fused engine (k_sweep).
//
// Same arithmetic as k_fused (the whole dimension-split divergence and the Q update of one
// step, all tracers), organised so that each quantity of the PPM sweeps is computed once
// per cell instead of once per edge:
//
//   * a thread owns a segment of one grid line through the tile and marches along it,
//     keeping the 5-cell window, the slope of the current cell and the edge value at its
//     left edge in registers.  A cell's slope and each edge value are computed once and
//     shared by the two cells (reconstruction_1d.py:64-192 computes them the same way,
//     as edge arrays); the limiter runs once per cell, and the upwind flux through an
//     edge selects the parabola of the cell on the upwind side (flux.py:46-66).
//   * x-lines (fixed column, marching rows) read consecutive columns across a warp; y-lines
//     (fixed row, marching columns) read consecutive rows across a warp, so their global
//     data (y-edge winds and flags, metric) is stored transposed (row j, column i).  Shared
//     memory rows have an odd pitch, so both directions are free of bank conflicts.
//
// Phases per tracer (one CTA = one tile of one panel of one solve):
//   P0  Q on the tile + 3 halo cells -> shared (pending MF-PR correction added on load)
//   P1  x-lines over the tile columns +-3: first-pass x fluxes -> split field Qx;
//       y-lines over the tile rows +-3:    first-pass y fluxes -> split field Qy
//       (discrete_operators.py:49-73)
//   P2  y-lines of Qx over the tile rows: second-pass y-flux differences -> shared
//   P3  x-lines of Qy over the tile columns: second-pass x fluxes; div and Q update,
//       written to global memory (coalesced), MF-PR block partial (discrete_operators.py:80-101)
//
// Work comes from a table of (solve, item) pairs; item = panel * tiles + tile.  One launch
// can therefore advance many solves of different sizes (each with its own descriptor), and
// a persistent grid may loop over the table.  The MF-PR sums use a fixed order that depends
// only on the solve and its tile shape, so a solve gives the same bits alone or in a batch.
#pragma once
#include "fused.cuh"
#include "halo.cuh"

namespace csadv {



template <class real>
__device__ __forceinline__ real csign(real a, real b) { return copysign(a, b); }
template <>
__device__ __forceinline__ float csign<float>(float a, float b) { return copysignf(a, b); }

// Decisions of the limiters.  GB300 runs FP64 arithmetic at 1/64 of the FP32 rate, so in FP64
// the comparisons and minima are taken on the bit patterns with integer instructions, leaving
// the FP64 pipe to the arithmetic.  The results equal the floating-point ones for finite
// inputs (the sign of a product differs only if the product of two non-zero values underflows
// to zero).
template <class real>
struct Pred {
    __device__ static __forceinline__ bool prod_pos(real a, real b) { return a * b > real(0); }
    __device__ static __forceinline__ bool prod_nonpos(real a, real b) { return a * b <= real(0); }
    __device__ static __forceinline__ bool abs_lt(real a, real b) { return RealOps<real>::ab(a) < RealOps<real>::ab(b); }
    // a, b >= 0
    __device__ static __forceinline__ real min_nonneg(real a, real b) { return RealOps<real>::fmn(a, b); }
    // p > d and p < -d, with d >= 0
    __device__ static __forceinline__ bool gt_nonneg(real p, real d) { return p > d; }
    __device__ static __forceinline__ bool lt_neg(real p, real d) { return -d > p; }
};
// FP64 helpers on the integer pipe.  GB300 issues FP64 arithmetic at 1/64 of the FP32 rate, so
// the FP64 kernel moves every operation that needs no FP64 rounding off the FP64 pipe: absolute
// values, sign transfers and selections on the bit patterns, exact scalings by powers of two on
// the exponent field, orderings of the bit patterns.  All of it works on the 32-bit halves of the
// patterns: measured on GB300, 64-bit integer comparisons run as FP64-pipe instructions (they
// counted as DADD), so a 64-bit compare would cost as much as the arithmetic it replaces.
struct Bits {  // a double as its two 32-bit words
    int h;       // sign, exponent, high mantissa
    unsigned l;  // low mantissa
    __device__ __forceinline__ explicit Bits(double x) {
        h = __double2hiint(x);
        l = (unsigned)__double2loint(x);
    }
    __device__ __forceinline__ Bits(int h_, unsigned l_) {
        h = h_;
        l = l_;
    }
    __device__ __forceinline__ double d() const { return __hiloint2double(h, (int)l); }
    __device__ __forceinline__ int mh() const { return h & 0x7fffffff; }  // high word of |x|
    __device__ __forceinline__ bool zero() const { return (mh() | (int)l) == 0; }
};
// |x| < |y| (magnitudes compared word by word)
__device__ __forceinline__ bool mag_lt(const Bits &x, const Bits &y) {
    return x.mh() < y.mh() || (x.mh() == y.mh() && x.l < y.l);
}
// c ? a : b on the bit patterns
__device__ __forceinline__ Bits bsel(bool c, const Bits &a, const Bits &b) { return Bits(c ? a.h : b.h, c ? a.l : b.l); }
__device__ __forceinline__ double dsel(bool c, double a, double b) { return bsel(c, Bits(a), Bits(b)).d(); }
// -x by the sign bit
__device__ __forceinline__ double neg_d(double x) { return Bits(Bits(x).h ^ (int)0x80000000, Bits(x).l).d(); }
__device__ __forceinline__ float dsel(bool c, float a, float b) { return c ? a : b; }
// the order of finite values (+0 and -0 equal): x > y
__device__ __forceinline__ bool ord_gt(const Bits &x, const Bits &y) {
    const bool nx = x.h < 0 && !x.zero(), ny = y.h < 0 && !y.zero();
    if (nx != ny) return ny;                  // exactly one of them negative (zeros count as +0)
    const bool gt_mag = mag_lt(y, x), lt_mag = mag_lt(x, y);
    return nx ? lt_mag : gt_mag;              // both negative: the smaller magnitude is greater
}
template <>
struct Pred<double> {
    __device__ static __forceinline__ bool prod_pos(double x, double y) {
        const Bits a(x), b(y);
        return (a.h ^ b.h) >= 0 && !a.zero() && !b.zero();
    }
    __device__ static __forceinline__ bool prod_nonpos(double x, double y) { return !prod_pos(x, y); }
    __device__ static __forceinline__ bool abs_lt(double x, double y) { return mag_lt(Bits(x), Bits(y)); }
    // a, b >= 0
    __device__ static __forceinline__ double min_nonneg(double x, double y) {
        const Bits a(x), b(y);
        return bsel(mag_lt(a, b), a, b).d();
    }
    // p > d and p < -d, with d >= 0
    __device__ static __forceinline__ bool gt_nonneg(double p, double d) {
        const Bits a(p), b(d);
        return a.h >= 0 && mag_lt(b, a);
    }
    __device__ static __forceinline__ bool lt_neg(double p, double d) {
        const Bits a(p), b(d);
        return a.h < 0 && mag_lt(b, a);
    }
};

// |x| 2^K on the pattern of a magnitude m (sign bit clear): equal to the FP64 product whenever that
// is a normal number (every value of an advected field); results below the normal range become
// 0, and m is returned unchanged when it is infinite, NaN or so large (> 2^1022) that the product
// would overflow
template <int K>
__device__ __forceinline__ Bits mag_scale(const Bits &m) {
    const int e = m.h >> 20;
    constexpr int EMIN = K < 0 ? 1 - K : 1, EMAX = K > 0 ? 0x7fe - K : 0x7fe;
    if (e < EMIN) return Bits(0, 0u);
    return Bits(e <= EMAX ? m.h + K * (1 << 20) : m.h, m.l);
}
// x 2^K for a double of either sign, as mag_scale (the sign kept)
template <int K>
__device__ __forceinline__ double pow2_scale(double x) {
    const Bits b(x);
    const Bits m = mag_scale<K>(Bits(b.mh(), b.l));
    return Bits(m.h | (b.h & (int)0x80000000), m.l).d();
}

// x / 2 (exact: on the exponent for FP64, an FP32 product otherwise)
__device__ __forceinline__ double half_of(double x) { return pow2_scale<-1>(x); }
__device__ __forceinline__ float half_of(float x) { return 0.5f * x; }

// --------------------------------------------------------------------------- reconstructions
// CW84 limited slope of the cell q0 between qm and qp (reconstruction_1d.py:64-100);
// min(...) * sign(d0) written as copysign: equal for every finite input
template <class real>
__device__ __forceinline__ real cw84_slope(real qm, real q0, real qp) {
    using O = RealOps<real>;
    const real d0 = real(0.5) * (qp - qm);
    const real d1 = real(2.0) * (qp - q0);
    const real d2 = real(2.0) * (q0 - qm);
    using B = Pred<real>;
    const real s = csign(B::min_nonneg(B::min_nonneg(O::ab(d0), O::ab(d1)), O::ab(d2)), d0);
    return B::prod_pos(qp - q0, q0 - qm) ? s : real(0);
}
// value at the edge between cells a and b from their values and slopes
template <class real>
__device__ __forceinline__ real cw84_edge(real qa, real qb, real sa, real sb) {
    return real(0.5) * (qb + qa) - Div<real>::by(sb - sa, real(6.0), real(1.0 / 6.0));
}
// CW84 monotonicity limiter of the parabola (L, R) of a cell with mean qc (reconstruction_1d.py:102-153)
template <class real>
__device__ __forceinline__ void cw84_limit(real qc, real &L, real &R) {
    using B = Pred<real>;
    const real dq = R - L;
    const real q6 = real(6) * qc - real(3) * (R + L);
    const bool flat = B::prod_nonpos(R - qc, qc - L);
    R = flat ? qc : R;
    L = flat ? qc : L;
    const bool over = B::abs_lt(dq, q6);
    const real DL = R - L;
    const real mid = qc - real(0.5) * (R + L);
    const real d2 = Div<real>::by(DL * DL, real(6.0), real(1.0 / 6.0));
    const real prod = DL * mid;
    const bool ml = over && B::gt_nonneg(prod, d2);
    const bool mr = over && !ml && B::lt_neg(prod, d2);
    const real Ln = real(3.0) * qc - real(2.0) * R;
    const real Rn = real(3.0) * qc - real(2.0) * L;
    L = ml ? Ln : L;
    R = mr ? Rn : R;
}
// L04 monotone slope (reconstruction_1d.py:155-172)
template <class real>
__device__ __forceinline__ real l04_mono(real qm, real q0, real qp) {
    using O = RealOps<real>;
    const real dq = real(0.25) * (qp - qm);
    const real dmin = O::fmx(O::fmx(qm, q0), qp) - q0;
    const real dmax = q0 - O::fmn(O::fmn(qm, q0), qp);
    using B = Pred<real>;
    return csign(B::min_nonneg(B::min_nonneg(O::ab(dq), dmin), dmax), dq);
}
template <class real>
__device__ __forceinline__ real l04_edge(real qa, real qb, real ma, real mb) {
    return real(0.5) * (qb + qa) - Div<real>::by(mb - ma, real(3.0), real(1.0 / 3.0));
}
// L04 limiter (reconstruction_1d.py:174-192)
template <class real>
__device__ __forceinline__ void l04_limit(real q0, real mono, real &L, real &R) {
    using O = RealOps<real>;
    using B = Pred<real>;
    const real m2 = real(2.0) * mono;
    L = q0 - csign(B::min_nonneg(real(2.0) * O::ab(mono), O::ab(L - q0)), m2);
    R = q0 + csign(B::min_nonneg(real(2.0) * O::ab(mono), O::ab(R - q0)), m2);
}
// PPM-0 4-point edge value between cells a and b (reconstruction_1d.py:33-44)
template <class real>
__device__ __forceinline__ real ppm0_edge(real qam, real qa, real qb, real qbp) {
    return real(7.0 / 12.0) * (qb + qa) - Div<real>::by(qbp + qam, real(12.0), real(1.0 / 12.0));
}

// The FP64 CW84 reconstruction with its FP64 operations cut to the ones that round: the limited
// slope from a = qp - qm, b = qp - q0, c = q0 - qm (reconstruction_1d.py:64-100) is
// sign(a) min(|a|/2, 2 min(|b|, |c|)) when b c > 0, with the scalings exact on the exponent; the
// edge value 0.5 (qa + qb) - (sb - sa)/6; the limiter (reconstruction_1d.py:102-153) with the
// monotonicity test as an ordering of the bit patterns (R - qc and qc - L have the signs of
// those comparisons) and the flattened case's DL = 0, mid = 0 selected.
__device__ __forceinline__ double cw84_slope_d(double a, double b, double c) {
    const Bits A(a), B(b), C(c);
    const Bits mb(B.mh(), B.l), mc(C.mh(), C.l);
    const Bits m = mag_scale<1>(bsel(mag_lt(mb, mc), mb, mc));   // 2 min(|b|, |c|)
    const Bits h = mag_scale<-1>(Bits(A.mh(), A.l));                // |a| / 2
    const Bits v = bsel(mag_lt(h, m), h, m);
    const bool pos = (B.h ^ C.h) >= 0 && !B.zero() && !C.zero();  // b c > 0
    return pos ? Bits(v.h | (A.h & (int)0x80000000), v.l).d() : 0.0;
}
__device__ __forceinline__ double cw84_edge_d(double qa, double qb, double sa, double sb) {
    return fma(-(sb - sa), 1.0 / 6.0, pow2_scale<-1>(qb + qa));
}
// The limiter in the offsets u = R - qc, v = qc - L of a cell's parabola.  The reference's tests
// (reconstruction_1d.py:102-153) with dq = u + v and q6 = 3 (v - u): flattened when u v <= 0 (the
// extremum test); for a cell that is not flattened (u, v of one sign) the overshoot tests
// |dq| < |q6| and dq (qc - (R + L)/2) >< +-dq^2/6 hold exactly when |v| > 2|u| (L moves to
// 3 qc - 2 R, i.e. v becomes 2u) or |u| > 2|v| (R moves to 3 qc - 2 L, u becomes 2v).  At the
// ties a rounding could decide, both branches give the same parabola.  No FP64 instruction: the
// tests, 2|u|, 2|v| and the selections are integer work on the bit patterns.
__device__ __forceinline__ void cw84_limit_ofs(double u, double v, double &uo, double &vo) {
    const Bits bu(u), bv(v);
    const bool flat = !((bu.h ^ bv.h) >= 0 && !bu.zero() && !bv.zero());  // u v <= 0
    const Bits mu(bu.mh(), bu.l), mv(bv.mh(), bv.l);                     // |u|, |v|
    const bool ml = mag_lt(mag_scale<1>(mu), mv);                        // |v| > 2|u|
    const bool mr = mag_lt(mag_scale<1>(mv), mu);                        // |u| > 2|v|
    uo = dsel(flat, 0.0, dsel(mr, pow2_scale<1>(v), u));
    vo = dsel(flat, 0.0, dsel(ml, pow2_scale<1>(u), v));
}

// Marching reconstruction: init() with the window of the first cell, then cell() once per
// cell (window w[0..4] = q[m-2..m+2]) gives the cell's (L, R) and advances.
template <class real, int REC>
struct March;
// FP64 CW84 in offsets: per cell the limited u' = R - q and v' = q - L (cw84_limit_ofs) instead
// of the edge values.  With d = q(m+1) - q(m) and ds = s(m+1) - s(m) the edge value between them,
// E = (q(m) + q(m+1))/2 - ds/6, gives u(m) = E - q(m) = d/2 - ds/6 and v(m+1) = q(m+1) - E =
// d/2 + ds/6: two fused operations per edge, and the limiter needs no FP64 arithmetic.
template <>
struct March<double, REC_CW84> {
    double s, dd, vm;  // slope of the current cell; w[3] - w[2]; q(m) - E(m - 1/2) of the current cell
    __device__ __forceinline__ void init(const double w[5]) {
        const double d01 = w[1] - w[0], d12 = w[2] - w[1], d23 = w[3] - w[2];
        const double sp = cw84_slope_d(w[2] - w[0], d12, d01);
        s = cw84_slope_d(w[3] - w[1], d23, d12);
        vm = fma(s - sp, 1.0 / 6.0, pow2_scale<-1>(d12));
        dd = d23;
    }
    // the limited offsets (uo, vo) of the window's centre cell; advances
    __device__ __forceinline__ void cell(const double w[5], double &uo, double &vo) {
        const double b = w[4] - w[3];
        const double sn = cw84_slope_d(w[4] - w[2], b, dd);
        const double ds = sn - s, hd = pow2_scale<-1>(dd);
        const double u = fma(-ds, 1.0 / 6.0, hd);
        const double vn = fma(ds, 1.0 / 6.0, hd);
        cw84_limit_ofs(u, vm, uo, vo);
        s = sn;
        vm = vn;
        dd = b;
    }
};
template <class real, int REC>
struct March {
    real s, E;  // slope of the current cell; edge value at its left edge
    __device__ __forceinline__ void init(const real w[5]) {
        if (REC == REC_CW84) {
            const real sp = cw84_slope(w[0], w[1], w[2]);
            s = cw84_slope(w[1], w[2], w[3]);
            E = cw84_edge(w[1], w[2], sp, s);
        } else if (REC == REC_L04) {
            const real sp = l04_mono(w[0], w[1], w[2]);
            s = l04_mono(w[1], w[2], w[3]);
            E = l04_edge(w[1], w[2], sp, s);
        } else if (REC == REC_PPM0) {
            E = ppm0_edge(w[0], w[1], w[2], w[3]);
        }
    }
    __device__ __forceinline__ void cell(const real w[5], real &L, real &R) {
        if (REC == REC_CW84) {
            const real sn = cw84_slope(w[2], w[3], w[4]);
            const real En = cw84_edge(w[2], w[3], s, sn);
            L = E;
            R = En;
            cw84_limit(w[2], L, R);
            s = sn;
            E = En;
        } else if (REC == REC_L04) {
            const real sn = l04_mono(w[2], w[3], w[4]);
            const real En = l04_edge(w[2], w[3], s, sn);
            L = E;
            R = En;
            l04_limit(w[2], s, L, R);
            s = sn;
            E = En;
        } else if (REC == REC_PPM0) {
            const real En = ppm0_edge(w[1], w[2], w[3], w[4]);
            L = E;
            R = En;
            E = En;
        } else {  // PL07 hybrid 5-point values (reconstruction_1d.py:46-62)
            const real a1 = real(2.0 / 60.0), a2 = real(-13.0 / 60.0), a3 = real(47.0 / 60.0),
                       a4 = real(27.0 / 60.0), a5 = real(-3.0 / 60.0);
            R = a1 * w[0] + a2 * w[1] + a3 * w[2] + a4 * w[3] + a5 * w[4];
            L = a5 * w[0] + a4 * w[1] + a3 * w[2] + a2 * w[3] + a1 * w[4];
        }
    }
};

// One grid line through a tile.  Cell m (tile-local, 0 = first interior cell of the tile
// along the line) is at s[m * ss] in shared memory; the record of edge m (left edge of cell
// m) is e[m * P] and that of cell m is c[m * P] in global memory.
template <class real>
struct Line {
    using V = typename Vec2<real>::type;
    const real *s;
    int ss;
    const V *e, *c;
    const V *f;     // flux coefficients of edge m: {alpha, beta} at f[m * P], {gamma, sigma} at f[m * P + fo]
    long long fo;   // (flux_coefs and put_record, wind.cu)
};

enum { MARCH_SPLIT = 0, MARCH_DIFF = 1, MARCH_UPDATE = 2 };

// per-line sums of the update (MF-PR): div * g and the new Q * g
template <class real>
struct LineSums {
    real div, mass;
};

#ifndef CSADV_SWEEP_UNROLL
#define CSADV_SWEEP_UNROLL 1
#endif
// march loop unrolling: 1, measured best for the FP64 form since the march works in edge offsets
// (0.297 ms per N=384 two-tracer step against 0.303 ms unrolled 2x and 0.304 ms 3x: fewer spilled
// values; the FP64 pipe is the bound either way)
constexpr int SWEEP_UNROLL = CSADV_SWEEP_UNROLL;

// March over cells [ma - 1, mb]: fluxes through edges [ma, mb], outputs for cells [ma, mb).
//   MARCH_SPLIT : split field of the first pass -> out[k * os]
//   MARCH_DIFF  : flux difference F(k+1) - F(k) -> out[k * os]
//   MARCH_UPDATE: Q(k) - dt div(k) -> qout[k * P], with the y-flux differences dY[k * os]
//                 and Q(k) at Qc[k * qs]; returns the line's sums of div * g and of the new
//                 Q * g (MF-PR)
// Loads run one iteration ahead of the arithmetic (edge records and flux coefficients, cell
// records, the shared-memory window), so the global (L1/L2) latency overlaps the work.
template <class real, int REC, int MODE>
__device__ __forceinline__ LineSums<real> march(const Line<real> &ln, int P, int ma, int mb, real dtdx, real irdx,
                                                int mt, int split, bool mfpr, real *out, int os, const real *dY,
                                                const real *Qc, int qs, real *qout) {
    using O = RealOps<real>;
    using V = typename Vec2<real>::type;
    // FP64 with AVLT splitting: the cell records carry dt/dx (1/g) (k_cell_records), and the
    // split's (dt/dx / 2)(1/g) is half of it, exactly
    const bool HDT = sizeof(real) == 8 && split == SP_AVLT;
    // FP64 CW84: the cells' parabolas as limited offsets (u', v') from the mean, and the flux as
    // sigma mean + alpha u' - beta v' with sigma = alpha + beta + gamma (the record's second word)
    constexpr bool OFS = sizeof(real) == 8 && REC == REC_CW84;
    real w[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) w[k] = ln.s[(ma - 3 + k) * ln.ss];
    March<real, REC> rc;
    rc.init(w);
    V eA = ln.e[(ma - 1) * P], eN = eA;                          // edge m (m+1 loaded in the loop)
    V fA = ln.f[(ma - 1) * P], fN = fA;                          // its flux coefficients
    real gA = OFS ? ln.f[(ma - 1) * P + ln.fo].y : ln.f[(ma - 1) * P + ln.fo].x, gN = gA;
    V cC = ln.c[(ma - 1) * P], cN = cC;                          // cell m
    real nw4 = real(0);
    real pL = real(0), pR = real(0), pQ = real(0);  // previous cell's parabola
    real Fp = real(0), cp = real(0), gcp = real(0), igp = real(0), accm = real(0);
    real Fa = real(0);  // the flux through edge ma (the MF-PR sum telescopes to F(mb) - F(ma))
#pragma unroll SWEEP_UNROLL
    for (int m = ma - 1; m <= mb; ++m) {
        if (m < mb) {
            nw4 = ln.s[(m + 3) * ln.ss];
            eN = ln.e[(m + 1) * P];
            fN = ln.f[(m + 1) * P];
            gN = OFS ? ln.f[(m + 1) * P + ln.fo].y : ln.f[(m + 1) * P + ln.fo].x;
            cN = ln.c[(m + 1) * P];
        }
        const real gl = O::ab(eA.y), gcm = cC.x;
        real L, R;  // the cell's parabola (OFS: R holds u', L holds v')
        rc.cell(w, OFS ? R : L, OFS ? L : R);
        if (m >= ma) {
            // upwind PPM flux through edge m (flux.py:20-128) from the parabola (q_L, q_R, mean) of
            // the upwind cell (m-1 when the wind is >= 0): F = alpha q_R + beta q_L + gamma mean,
            // the reference's u (e -+ c/2 (q6 -+ dq) - q6 c^2/3) with its metric weights
            // (flux.py:28-31 for MT-0, the edge metric for MT-PL07) multiplied out per edge
            // (flux_coefs, wind.cu)
            const real u = eA.x;
            const bool up = !signbit(eA.y);
            const real ig = igp;
            const real eL = dsel(up, pL, L), eR = dsel(up, pR, R), eQ = dsel(up, pQ, w[2]);
            // OFS: (eR, eL) are the upwind cell's (u', v')
            const real F = OFS ? fma(fA.x, eR, fma(-fA.y, eL, gA * eQ)) : fma(gA, eQ, fma(fA.y, eL, fA.x * eR));
            const real cm = split == SP_AVLT ? real(0) : gl * (u * dtdx);  // g u dt/dx at edge m (SP-L04, SP-PL07)
            if (m > ma) {
                const int k = m - 1;
                if (MODE == MARCH_SPLIT) {
                    const real q = w[1];
                    const real dF = -(F - Fp) * dtdx;
                    real o;
                    if (split == SP_AVLT)  // q + dF / (2 g), dF = -(F - Fp) dt/dx
                        o = fma(-(F - Fp), HDT ? half_of(ig) : (real(0.5) * dtdx) * ig, q);
                    else if (split == SP_L04)
                        o = (q * gcp + real(0.5) * dF + real(0.5) * (cm - cp) * q) * ig;
                    else
                        o = real(0.5) * (q + (q + dF) / (real(1.0) - (cm - cp)));
                    out[k * os] = o;
                } else if (MODE == MARCH_DIFF) {
                    out[k * os] = F - Fp;
                } else {
                    const real sdiv = (F - Fp) + dY[k * os];
                    const real qn = fma(-sdiv, HDT ? ig : dtdx * ig, Qc[k * qs]);
                    qout[(long long)k * P] = qn;
                }
            }
            if (m == ma) Fa = F;
            Fp = F;
            cp = cm;
        }
        pL = L;
        pR = R;
        pQ = w[2];
        gcp = gcm;
        igp = cC.y;
        eA = eN;
        fA = fN;
        gA = gN;
        cC = cN;
        w[0] = w[1];
        w[1] = w[2];
        w[2] = w[3];
        w[3] = w[4];
        w[4] = nw4;
    }
    // MF-PR: sum(div g) = sum(sdiv) / dx (div = sdiv / (dx g)), and over a segment the x part of
    // sdiv = (F(k+1) - F(k)) + dY(k) sums to F(mb) - F(ma); the y-flux differences dY are summed the
    // same way by the P2 lines that form them (MARCH_DIFF), so no per-cell addition is needed
    const real tele = mfpr && MODE != MARCH_SPLIT ? Fp - Fa : real(0);
    return LineSums<real>{tele * irdx, accm};
}

// CTAs per SM the register allocation is sized for: two, so that the FP64 pipe (on GB300 its
// results arrive on the short scoreboard, long after issue) has twice the warps to choose from
// (measured: 533 -> 517 us on the N=384 two-tracer step)
#ifndef CSADV_SWEEP_MINB
template <class real> struct SweepMinBlocks { static constexpr int value = 2; };
template <> struct SweepMinBlocks<double> { static constexpr int value = 2; };
#else
template <class real> struct SweepMinBlocks { static constexpr int value = CSADV_SWEEP_MINB; };
#endif

// SPL: the splitting (SP_AVLT, SP_L04 with MT-0; SP_PL07 with MT-PL07), fixed per kernel so
// the march loop carries no scheme branches
template <class real, int REC, int SPL>
__global__ void __launch_bounds__(SWEEP_THREADS, SweepMinBlocks<real>::value) k_sweep(const SweepSolve *__restrict__ solves,
                                                         const int2 *__restrict__ work, int nwork) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    real *sm = (real *)smem_raw;
    __shared__ double red[SWEEP_THREADS];
    __shared__ int last;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NWARP = SWEEP_THREADS / 32;

    for (int wk = blockIdx.x; wk < nwork; wk += gridDim.x) {
        const int2 it = work ? work[wk] : make_int2(0, wk);
        const SweepSolve &S = solves[it.x];
        const Dims d = S.d;
        const int ti = S.ti, tj = S.tj, ntiles = S.ntiles, nitems = NFACE * ntiles;
        const int tile = it.y % ntiles, p = it.y / ntiles;
        int I0, ni, J0, nj;
        sweep_tile(S, tile, I0, ni, J0, nj);
        const SweepSmem L = sweep_smem(ti, tj);
        real *sQ = sm, *sQx = sm + L.oQx, *sQy = sm + L.oQy, *sDy = sm + L.oDy;
        const int P = d.pitch;
        const long long pofs = (long long)p * d.plane;
        const real dtdx = (real)(S.dt / S.dx);
        const real irdx = real(1) / (real)S.dx;
        constexpr int split = SPL, mt = SPL == SP_PL07 ? MT_PL07 : MT_0;
        const bool mfpr = S.mfpr != 0;
        using V = typename Vec2<real>::type;
        const V *erx = (const V *)S.erx + pofs, *ery = (const V *)S.ery + pofs;
        const V *efx = erx + S.ecofs, *efy = ery + S.ecofs;
        const V *crx = (const V *)S.crx, *cry = (const V *)S.cry;
        const real *gpc = (const real *)S.gpc;

        for (int tr = 0; tr < S.T; ++tr) {
            const real *Qin = (const real *)S.Qin + (long long)tr * d.field + pofs;
            real *Qout = (real *)S.Qout + (long long)tr * d.field + pofs;
            const bool hc = S.corr_in != nullptr;
            const real corr = hc ? (real)S.corr_in[tr] : real(0);
            // P0: Q on the tile + halo: interior cells with the pending mass-fixer correction;
            // ghost cells as filled by the ghost-cell kernel, or (lag_w set) interpolated here
            // from the neighbouring panels (ET-DG, from the corrected interior values)
            const Src<real> src{(const real *)S.Qin + (long long)tr * d.field, gpc, corr, hc};
            const bool inline_ghosts = S.lag_w != nullptr;
            for (int r = warp; r < ni + 6; r += NWARP) {
                const int i = I0 - 3 + r;
                const bool irow = i >= d.i0 && i < d.iend;
                for (int c = lane; c < nj + 6; c += 32) {
                    const int j = J0 - 3 + c;
                    real v;
                    if (irow && j >= d.i0 && j < d.iend) {
                        v = Qin[(long long)i * P + j];
                        if (hc) v = corrected(v, gpc[(long long)i * P + j], corr);
                    } else if (!inline_ghosts) {
                        v = Qin[(long long)i * P + j];
                    } else {
                        v = (real)ghost_value(src, d, S.lag_w, S.lag_k, p, i, j);
                    }
                    sQ[r * L.QJp + c] = v;
                }
            }
            __syncthreads();
            // P1: first pass.  x-lines: columns c in [-3, nj+3), cells [0, ni) -> Qx;
            //                  y-lines: rows r in [-3, ni+3), cells [0, nj) -> Qy
            {
                // jobs packed densely (no idle lanes between lines); x- and y-lines share one code path
                const int LX = nj + 6, LY = ni + 6;
                const int jx = S.s1x * LX, jy = S.s1y * LY;
                for (int job = tid; job < jx + jy; job += SWEEP_THREADS) {
                    const bool xl = job < jx;
                    const int jj = xl ? job : job - jx, nl = xl ? LX : LY, ns = xl ? S.s1x : S.s1y, len = xl ? ni : nj;
                    const int seg = jj / nl, o = jj - seg * nl - 3;  // o: column (x-lines) or row (y-lines)
                    const int ma = len * seg / ns, mb = len * (seg + 1) / ns;
                    if (ma >= mb) continue;
                    const long long g0 = xl ? (long long)I0 * P + J0 + o : (long long)J0 * P + I0 + o;
                    Line<real> ln{xl ? sQ + 3 * L.QJp + o + 3 : sQ + (o + 3) * L.QJp + 3, xl ? L.QJp : 1,
                                  (xl ? erx : ery) + g0, (xl ? crx : cry) + g0, (xl ? efx : efy) + g0, S.ecofs};
                    march<real, REC, MARCH_SPLIT>(ln, P, ma, mb, dtdx, irdx, mt, split, false,
                                                  xl ? sQx + o + 3 : sQy + (o + 3) * L.TJp, xl ? L.QJp : 1, nullptr,
                                                  nullptr, 0, nullptr);
                }
            }
            __syncthreads();
            real acc = real(0);  // MF-PR: this thread's share of the tile's sum(div g) (P2 and P3 lines)
            // P2: y-lines of Qx over rows [0, ni): y-flux differences -> sDy
            {
                const int LY = ni;  // jobs packed densely
                const int jy = S.s2y * LY;
                for (int job = tid; job < jy; job += SWEEP_THREADS) {
                    const int seg = job / LY, r = job - seg * LY;
                    const int ma = nj * seg / S.s2y, mb = nj * (seg + 1) / S.s2y;
                    if (r >= ni || ma >= mb) continue;
                    const long long g0 = (long long)J0 * P + I0 + r;
                    Line<real> ln{sQx + r * L.QJp + 3, 1, ery + g0, cry + g0, efy + g0, S.ecofs};
                    acc += march<real, REC, MARCH_DIFF>(ln, P, ma, mb, dtdx, irdx, mt, split, mfpr, sDy + r * L.TJp,
                                                        1, nullptr, nullptr, 0, nullptr).div;
                }
            }
            __syncthreads();
            // P3: x-lines of Qy over columns [0, nj): x fluxes, div, update, MF-PR partials
            {
                const int LX = nj;  // jobs packed densely
                const int jx = S.s2x * LX;
                for (int job = tid; job < jx; job += SWEEP_THREADS) {
                    const int seg = job / LX, c = job - seg * LX;
                    const int ma = ni * seg / S.s2x, mb = ni * (seg + 1) / S.s2x;
                    if (c >= nj || ma >= mb) continue;
                    const long long g0 = (long long)I0 * P + J0 + c;
                    Line<real> ln{sQy + 3 * L.TJp + c, L.TJp, erx + g0, crx + g0, efx + g0, S.ecofs};
                    const LineSums<real> ls = march<real, REC, MARCH_UPDATE>(
                        ln, P, ma, mb, dtdx, irdx, mt, split, mfpr, nullptr, L.TJp, sDy + c, sQ + 3 * L.QJp + c + 3,
                        L.QJp, Qout + g0);
                    acc += ls.div;
                }
            }
            if (mfpr) {  // FP64 across threads, in a fixed order
                double dacc = (double)acc;  // the FP64 form has no mass target (the reference's projection)
                for (int o = 16; o > 0; o >>= 1) dacc += __shfl_xor_sync(0xffffffffu, dacc, o);
                if (lane == 0) red[warp] = dacc;
                __syncthreads();
                if (tid == 0) {
                    double s = 0.0;
                    for (int w = 0; w < NWARP; ++w) s += red[w];
                    S.partials[(long long)tr * nitems + it.y] = s;
                }
            }
            __syncthreads();
        }
        if (mfpr) {
            // the last item of the solve to finish sums its partials: corr = dt m0 / a2
            if (tid == 0) {
                __threadfence();
                const unsigned int prev = atomicAdd(S.counter, 1u);
                last = prev == (unsigned int)nitems - 1u;
            }
            __syncthreads();
            if (last) {
                __threadfence();
                for (int tr = 0; tr < S.T; ++tr) {
                    double a = 0.0;
                    const volatile double *pp = S.partials + (long long)tr * nitems;
                    for (int b = tid; b < nitems; b += SWEEP_THREADS) a += pp[b];
                    red[tid] = a;
                    __syncthreads();
                    for (int s = SWEEP_THREADS / 2; s > 0; s >>= 1) {
                        if (tid < s) red[tid] += red[tid + s];
                        __syncthreads();
                    }
                    // projection (discrete_operators.py:98-101): corr = dt m0 / a2; anchored FP32
                    // form: the correction that brings sum(Q g) back to the target mass
                    if (tid == 0)
                        S.corr_out[tr] = S.mass_target ? (S.mass_target[tr] - red[0]) / S.a2 : S.dt * red[0] / S.a2;
                    __syncthreads();
                }
                if (tid == 0) *S.counter = 0u;
            }
            __syncthreads();
        }
    }
}



template <class real, int REC, int SPL>
int sweep_go(const SweepSolve *dsolves, const int2 *work, int nwork, int grid, size_t smem, cudaStream_t st) {
    if (st == (cudaStream_t)-1) {  // prepare only: allow the largest layout
        size_t mx = 0;
        for (int c = 0; c < SWEEP_NTILE_CFG; ++c) mx = mx > sweep_smem_bytes<real>(c) ? mx : sweep_smem_bytes<real>(c);
        CSADV_CUDA(cudaFuncSetAttribute(k_sweep<real, REC, SPL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mx));
        return CSADV_OK;
    }
    k_sweep<real, REC, SPL><<<grid, SWEEP_THREADS, smem, st>>>(dsolves, work, nwork);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

template <class real, int REC>
int sweep_split(int split, const SweepSolve *dsolves, const int2 *work, int nwork, int grid, size_t smem,
                cudaStream_t st) {
    switch (split) {
        case SP_AVLT: return sweep_go<real, REC, SP_AVLT>(dsolves, work, nwork, grid, smem, st);
        case SP_L04: return sweep_go<real, REC, SP_L04>(dsolves, work, nwork, grid, smem, st);
        default: return sweep_go<real, REC, SP_PL07>(dsolves, work, nwork, grid, smem, st);
    }
}

template <class real>
int sweep_launch(int recon, int split, const SweepSolve *dsolves, const int2 *work, int nwork, int grid, size_t smem,
                 cudaStream_t st, int) {
    switch (recon) {
        case REC_PPM0: return sweep_split<real, REC_PPM0>(split, dsolves, work, nwork, grid, smem, st);
        case REC_CW84: return sweep_split<real, REC_CW84>(split, dsolves, work, nwork, grid, smem, st);
        case REC_PL07: return sweep_split<real, REC_PL07>(split, dsolves, work, nwork, grid, smem, st);
        default: return sweep_split<real, REC_L04>(split, dsolves, work, nwork, grid, smem, st);
    }
}

}  // namespace csadv
