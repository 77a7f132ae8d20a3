// Ghost-cell values of the ET-DG edge treatment (interpolation.py:154-314 with
// halo_data.py:15-185), as device functions shared by the ghost-cell kernel (halo.cu) and the
// line-marching step kernel, which evaluates the ghost cells of its tiles in place.
// Products and sums are rounded explicitly (no contraction), as numpy rounds them, so every
// translation unit computes the same bits whatever its FMA setting.
#pragma once
#include "common.cuh"

namespace csadv {

// the true state Q* + g corr of a cell with a pending MF-PR correction, one fused rounding (the
// same function everywhere the correction is applied: on load, in the ghost cells, on read-out)
__device__ __forceinline__ float corrected(float v, float g, float corr) { return __fmaf_rn(g, corr, v); }
__device__ __forceinline__ double corrected(double v, double g, double corr) { return __fma_rn(g, corr, v); }

// Source values of the ghost-cell interpolation.  With a pending MF-PR correction
// (fused engine) the stored interior value is Q* and the true value is Q* + g corr,
// formed in the state's precision exactly as the fused kernel forms it on load.
template <class real>
struct Src {
    const real *F;
    const real *g;  // metric plane (real), used only with corr
    real corr;
    bool has_corr;
    __device__ __forceinline__ real value(const Dims &d, int q, int i, int j) const {
        real v = F[at(d, q, i, j)];
        if (has_corr) v = corrected(v, g[at2(d, i, j)], corr);
        return v;
    }
    __device__ __forceinline__ double interior(const Dims &d, int q, int i, int j) const {
        return (double)value(d, q, i, j);
    }
};

// value of the ghost cell at depth `dep` outside side s of panel p, along index k
// (k inside the edge's interior range); computed in FP64 from interior cells only
template <class real>
__device__ __forceinline__ double side_ghost(const Src<real> &S, const Dims &d, const double *__restrict__ W,
                                             const int *__restrict__ K, int p, int s, int dep, int k) {
    const Conn c = c_conn[p][s];
    const int n = d.n;
    const int k0 = K[dep * n + k];
    const double *w = W + ((long long)dep * n + k) * 4;
    double prod[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        int kk = k0 + m;
        int along = c.rev ? n - 1 - kk : kk;
        int i, j;
        inside_ij(d, c.qs, dep, along, i, j);
        prod[m] = __dmul_rn(S.interior(d, c.q, i, j), w[m]);
    }
    return __dadd_rn(__dadd_rn(__dadd_rn(prod[0], prod[1]), prod[2]), prod[3]);
}

// value of cell (i, j) of panel q where (i, j) is interior or in a side strip (not a corner);
// one call site of side_ghost, so that the four calls of a corner cell inline into straight-line
// code whose loads the compiler can issue together
template <class real>
__device__ __forceinline__ double cell_or_side_ghost(const Src<real> &S, const Dims &d, const double *__restrict__ W,
                                                     const int *__restrict__ K, int q, int i, int j) {
    int s = -1, dep = 0, k = 0;
    if (i >= d.iend) {
        s = SIDE_E;
        dep = i - d.iend;
        k = j;
    } else if (i < d.i0) {
        s = SIDE_W;
        dep = d.i0 - 1 - i;
        k = j;
    } else if (j >= d.iend) {
        s = SIDE_N;
        dep = j - d.iend;
        k = i;
    } else if (j < d.i0) {
        s = SIDE_S;
        dep = d.i0 - 1 - j;
        k = i;
    }
    if (s < 0) return S.interior(d, q, i, j);
    return (double)(real)side_ghost(S, d, W, K, q, s, dep, k);
}

// value of the ghost cell (i, j) of panel p (not interior: i or j outside [i0, iend), both in
// [0, n)); the corner blocks as the reference fills them, from the neighbour's refreshed halo
template <class real>
__device__ __forceinline__ double ghost_value(const Src<real> &S, const Dims &d, const double *__restrict__ W,
                                              const int *__restrict__ K, int p, int i, int j) {
    if (i < d.i0 || i >= d.iend) {
        const int s = i >= d.iend ? SIDE_E : SIDE_W;
        const int dep = s == SIDE_E ? i - d.iend : d.i0 - 1 - i;
        if (is_interior(d, j)) return side_ghost(S, d, W, K, p, s, dep, j);
        const Conn c = c_conn[p][s];
        const int n = d.n;
        const int k0 = K[dep * n + j];
        const double *w = W + ((long long)dep * n + j) * 4;
        double prod[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            int kk = k0 + m;
            int along = c.rev ? n - 1 - kk : kk;
            int qi, qj;
            inside_ij(d, c.qs, dep, along, qi, qj);
            prod[m] = __dmul_rn(cell_or_side_ghost(S, d, W, K, c.q, qi, qj), w[m]);
        }
        return __dadd_rn(__dadd_rn(__dadd_rn(prod[0], prod[1]), prod[2]), prod[3]);
    }
    const int s = j >= d.iend ? SIDE_N : SIDE_S;
    const int dep = s == SIDE_N ? j - d.iend : d.i0 - 1 - j;
    return side_ghost(S, d, W, K, p, s, dep, i);
}

// ---------------------------------------------------------------- FP32 form: stencil tables
// The FP32 form keeps the Lagrange weights at FP64 accuracy but evaluates the interpolation on
// the FP32 pipe: GB300 runs FP64 at 1/64 of the FP32 rate, with long latency, and the ghost cells
// are on the critical path of every step.  Each ghost cell's interpolation is flattened, once per
// grid, into a list of terms {source cell, weight}: 4 for a side-strip cell, 16 for a corner-block
// cell (the outer weights times the inner stencils of the neighbour's side strip, formed in FP64,
// instead of the reference's two levels).  A weight is stored as hi + lo (two FP32 words, about
// 48 significant bits); each product q w is carried as an unevaluated sum (the FMA gives the
// rounding error of q hi exactly: Dekker's product) and the terms are summed with Knuth's
// two-sum, then rounded once to FP32.  Every evaluation is one level of table loads and one of
// source loads, without branches on the panel connectivity.
struct __align__(16) GhostTerm {
    int o;      // source cell: offset in one tracer's field (panel plane, row, column)
    int o2;     // the same cell in the single metric plane
    float2 w;   // weight: hi + lo
};
constexpr int GHOST_CORNER_TERMS = 16;

struct DFloat {
    float hi, lo;
};
__device__ __forceinline__ DFloat df_prod(float q, float2 w) {
    const float p = __fmul_rn(q, w.x);
    return DFloat{p, __fmaf_rn(q, w.y, __fmaf_rn(q, w.x, -p))};
}
__device__ __forceinline__ DFloat df_add(DFloat a, DFloat b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float v = __fsub_rn(s, a.hi);
    const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(b.hi, v));
    const float t = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    const float h = __fadd_rn(s, t);
    return DFloat{h, __fsub_rn(t, __fsub_rn(h, s))};
}
__device__ __forceinline__ float df_round(DFloat a) { return __fadd_rn(a.hi, a.lo); }

// sum of NT terms: all table loads, then all source loads, then the arithmetic
template <int NT>
__device__ __forceinline__ float ghost_terms_f(const Src<float> &S, const GhostTerm *__restrict__ t) {
    GhostTerm x[NT];
#pragma unroll
    for (int m = 0; m < NT; ++m) x[m] = t[m];
    float v[NT];
#pragma unroll
    for (int m = 0; m < NT; ++m) v[m] = S.has_corr ? corrected(S.F[x[m].o], S.g[x[m].o2], S.corr) : S.F[x[m].o];
    DFloat acc = df_prod(v[0], x[0].w);
#pragma unroll
    for (int m = 1; m < NT; ++m) acc = df_add(acc, df_prod(v[m], x[m].w));
    return df_round(acc);
}

// the stencil-table row of the ghost cell (i, j) of panel p (not interior; both within the 4 ghost
// layers): side rows [p][s][dep][k - i0] x 4 terms, corner rows [p][corner][di][dj] x 16
__device__ __forceinline__ const GhostTerm *ghost_row(const Dims &d, const GhostTerm *__restrict__ side,
                                                      const GhostTerm *__restrict__ corner, int p, int i, int j,
                                                      bool &is_corner) {
    const bool io = i < d.i0 || i >= d.iend, jo = j < d.i0 || j >= d.iend;
    is_corner = io && jo;
    if (is_corner) {
        const int cc = (i >= d.iend ? 2 : 0) + (j >= d.iend ? 1 : 0);
        const int di = i >= d.iend ? i - d.iend : d.i0 - 1 - i, dj = j >= d.iend ? j - d.iend : d.i0 - 1 - j;
        return corner + (((p * 4 + cc) * NG + di) * NG + dj) * GHOST_CORNER_TERMS;
    }
    int s, dep, k;
    if (io) {
        s = i >= d.iend ? SIDE_E : SIDE_W;
        dep = s == SIDE_E ? i - d.iend : d.i0 - 1 - i;
        k = j;
    } else {
        s = j >= d.iend ? SIDE_N : SIDE_S;
        dep = s == SIDE_N ? j - d.iend : d.i0 - 1 - j;
        k = i;
    }
    return side + ((((p * 4 + s) * NG + dep) * d.N) + (k - d.i0)) * 4;
}

// the ghost cell (i, j) of panel p for the FP32 form, from the stencil tables
__device__ __forceinline__ float ghost_table_f(const Src<float> &S, const Dims &d, const GhostTerm *__restrict__ side,
                                               const GhostTerm *__restrict__ corner, int p, int i, int j) {
    bool cn;
    const GhostTerm *t = ghost_row(d, side, corner, p, i, j, cn);
    return cn ? ghost_terms_f<GHOST_CORNER_TERMS>(S, t) : ghost_terms_f<4>(S, t);
}

// Two fields at once (the two tracers of a pair in the FP32 step kernel; F1 = F0 + one field):
// each table entry and metric value is loaded once for both.  Per field the arithmetic is
// ghost_terms_f's, term by term, so each result has ghost_table_f's bits.  Terms are taken
// 8 at a time (loads of a chunk, then its arithmetic) to bound the registers held.
template <int NT>
__device__ __forceinline__ float2 ghost_terms_f2(const float *__restrict__ F0, const float *__restrict__ F1,
                                                 const float *__restrict__ g, float c0, float c1, bool has_corr,
                                                 const GhostTerm *__restrict__ t) {
    constexpr int CH = NT < 8 ? NT : 8;
    DFloat a0{0.f, 0.f}, a1{0.f, 0.f};
#pragma unroll
    for (int m0 = 0; m0 < NT; m0 += CH) {
        GhostTerm x[CH];
#pragma unroll
        for (int m = 0; m < CH; ++m) x[m] = t[m0 + m];
        float v0[CH], v1[CH];
#pragma unroll
        for (int m = 0; m < CH; ++m) {
            v0[m] = F0[x[m].o];
            v1[m] = F1[x[m].o];
            if (has_corr) {
                const float gg = g[x[m].o2];
                v0[m] = corrected(v0[m], gg, c0);
                v1[m] = corrected(v1[m], gg, c1);
            }
        }
#pragma unroll
        for (int m = 0; m < CH; ++m) {
            if (m0 + m == 0) {
                a0 = df_prod(v0[0], x[0].w);
                a1 = df_prod(v1[0], x[0].w);
            } else {
                a0 = df_add(a0, df_prod(v0[m], x[m].w));
                a1 = df_add(a1, df_prod(v1[m], x[m].w));
            }
        }
    }
    return make_float2(df_round(a0), df_round(a1));
}

__device__ __forceinline__ float2 ghost_table_f2(const float *F0, const float *F1, const float *g, float c0, float c1,
                                                 bool has_corr, const Dims &d, const GhostTerm *__restrict__ side,
                                                 const GhostTerm *__restrict__ corner, int p, int i, int j) {
    bool cn;
    const GhostTerm *t = ghost_row(d, side, corner, p, i, j, cn);
    return cn ? ghost_terms_f2<GHOST_CORNER_TERMS>(F0, F1, g, c0, c1, has_corr, t)
              : ghost_terms_f2<4>(F0, F1, g, c0, c1, has_corr, t);
}

// The ghost-cell value in the state's precision: FP64 sums in the reference's order for FP64
// state, the stencil tables for FP32 state
template <class real>
__device__ __forceinline__ real ghost_cell(const Src<real> &S, const Dims &d, const double *__restrict__ W,
                                           const int *__restrict__ K, const GhostTerm *__restrict__ side,
                                           const GhostTerm *__restrict__ corner, int p, int i, int j);
template <>
__device__ __forceinline__ double ghost_cell<double>(const Src<double> &S, const Dims &d, const double *__restrict__ W,
                                                     const int *__restrict__ K, const GhostTerm *__restrict__,
                                                     const GhostTerm *__restrict__, int p, int i, int j) {
    return ghost_value(S, d, W, K, p, i, j);
}
template <>
__device__ __forceinline__ float ghost_cell<float>(const Src<float> &S, const Dims &d, const double *__restrict__,
                                                   const int *__restrict__, const GhostTerm *__restrict__ side,
                                                   const GhostTerm *__restrict__ corner, int p, int i, int j) {
    return ghost_table_f(S, d, side, corner, p, i, j);
}

}  // namespace csadv
