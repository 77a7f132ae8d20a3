// Ghost-cell values of the ET-DG edge treatment (interpolation.py:154-314 with
// halo_data.py:15-185), as device functions shared by the ghost-cell kernel (halo.cu) and the
// line-marching step kernel, which evaluates the ghost cells of its tiles in place.
// Products and sums are rounded explicitly (no contraction), as numpy rounds them, so every
// translation unit computes the same bits whatever its FMA setting.
#pragma once
#include "common.cuh"

namespace csadv {

// the true state Q* + g corr of a cell with a pending MF-PR correction, rounded as the
// reference rounds Q - dt (div - g m0/a2) split into its two parts
__device__ __forceinline__ float corrected(float v, float g, float corr) { return __fadd_rn(v, __fmul_rn(g, corr)); }
__device__ __forceinline__ double corrected(double v, double g, double corr) {
    return __dadd_rn(v, __dmul_rn(g, corr));
}

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

// ---------------------------------------------------------------- FP32 form: double-float sums
// The FP32 form keeps the Lagrange weights at FP64 accuracy but evaluates the interpolation on
// the FP32 pipe: GB300 runs FP64 at 1/64 of the FP32 rate, with long latency, and the ghost cells
// are on the critical path of every step.  A weight is carried as hi + lo (two FP32 words, about
// 48 significant bits), each product q w as an unevaluated sum p + e (the FMA gives the rounding
// error of q hi exactly, Dekker's product), and the four products are summed with Knuth's
// two-sum; the result is rounded once to FP32.  It equals the FP64 evaluation rounded to FP32
// except when that value lies within ~2^-47 of a rounding boundary.  The order of the terms
// and the two-level corner rule are those of the FP64 functions above.
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

// side_ghost for the FP32 form (weights as hi + lo pairs)
__device__ __forceinline__ float side_ghost_f(const Src<float> &S, const Dims &d, const float2 *__restrict__ W,
                                              const int *__restrict__ K, int p, int s, int dep, int k) {
    const Conn c = c_conn[p][s];
    const int n = d.n;
    const int k0 = K[dep * n + k];
    const float2 *w = W + ((long long)dep * n + k) * 4;
    DFloat prod[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        int kk = k0 + m;
        int along = c.rev ? n - 1 - kk : kk;
        int i, j;
        inside_ij(d, c.qs, dep, along, i, j);
        prod[m] = df_prod(S.value(d, c.q, i, j), w[m]);
    }
    return df_round(df_add(df_add(df_add(prod[0], prod[1]), prod[2]), prod[3]));
}

__device__ __forceinline__ float cell_or_side_ghost_f(const Src<float> &S, const Dims &d, const float2 *__restrict__ W,
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
    if (s < 0) return S.value(d, q, i, j);
    return side_ghost_f(S, d, W, K, q, s, dep, k);
}

// ghost_value for the FP32 form
__device__ __forceinline__ float ghost_value_f(const Src<float> &S, const Dims &d, const float2 *__restrict__ W,
                                               const int *__restrict__ K, int p, int i, int j) {
    if (i < d.i0 || i >= d.iend) {
        const int s = i >= d.iend ? SIDE_E : SIDE_W;
        const int dep = s == SIDE_E ? i - d.iend : d.i0 - 1 - i;
        if (is_interior(d, j)) return side_ghost_f(S, d, W, K, p, s, dep, j);
        const Conn c = c_conn[p][s];
        const int n = d.n;
        const int k0 = K[dep * n + j];
        const float2 *w = W + ((long long)dep * n + j) * 4;
        DFloat prod[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            int kk = k0 + m;
            int along = c.rev ? n - 1 - kk : kk;
            int qi, qj;
            inside_ij(d, c.qs, dep, along, qi, qj);
            prod[m] = df_prod(cell_or_side_ghost_f(S, d, W, K, c.q, qi, qj), w[m]);
        }
        return df_round(df_add(df_add(df_add(prod[0], prod[1]), prod[2]), prod[3]));
    }
    const int s = j >= d.iend ? SIDE_N : SIDE_S;
    const int dep = s == SIDE_N ? j - d.iend : d.i0 - 1 - j;
    return side_ghost_f(S, d, W, K, p, s, dep, i);
}

// The ghost-cell value in the state's precision: FP64 sums for FP64 state, double-float sums
// (weights Wf) for FP32 state
template <class real>
__device__ __forceinline__ real ghost_cell(const Src<real> &S, const Dims &d, const double *__restrict__ W,
                                           const float2 *__restrict__ Wf, const int *__restrict__ K, int p, int i,
                                           int j);
template <>
__device__ __forceinline__ double ghost_cell<double>(const Src<double> &S, const Dims &d, const double *__restrict__ W,
                                                     const float2 *__restrict__, const int *__restrict__ K, int p,
                                                     int i, int j) {
    return ghost_value(S, d, W, K, p, i, j);
}
template <>
__device__ __forceinline__ float ghost_cell<float>(const Src<float> &S, const Dims &d, const double *__restrict__,
                                                   const float2 *__restrict__ Wf, const int *__restrict__ K, int p,
                                                   int i, int j) {
    return ghost_value_f(S, d, Wf, K, p, i, j);
}
template <class real>
__device__ __forceinline__ real side_cell(const Src<real> &S, const Dims &d, const double *__restrict__ W,
                                          const float2 *__restrict__ Wf, const int *__restrict__ K, int p, int s,
                                          int dep, int k);
template <>
__device__ __forceinline__ double side_cell<double>(const Src<double> &S, const Dims &d, const double *__restrict__ W,
                                                    const float2 *__restrict__, const int *__restrict__ K, int p,
                                                    int s, int dep, int k) {
    return side_ghost(S, d, W, K, p, s, dep, k);
}
template <>
__device__ __forceinline__ float side_cell<float>(const Src<float> &S, const Dims &d, const double *__restrict__,
                                                  const float2 *__restrict__ Wf, const int *__restrict__ K, int p,
                                                  int s, int dep, int k) {
    return side_ghost_f(S, d, Wf, K, p, s, dep, k);
}

}  // namespace csadv
