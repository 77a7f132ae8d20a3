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
    __device__ __forceinline__ double interior(const Dims &d, int q, int i, int j) const {
        real v = F[at(d, q, i, j)];
        if (has_corr) v = corrected(v, g[at2(d, i, j)], corr);
        return (double)v;
    }
};

// value of the ghost cell at depth `dep` outside side s of panel p, along index k
// (k inside the edge's interior range); computed in FP64 from interior cells only
template <class real>
__device__ double side_ghost(const Src<real> &S, const Dims &d, const double *__restrict__ W,
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

// value of cell (i, j) of panel q where (i, j) is interior or in a side strip (not a corner)
template <class real>
__device__ double cell_or_side_ghost(const Src<real> &S, const Dims &d, const double *__restrict__ W,
                                     const int *__restrict__ K, int q, int i, int j) {
    if (i >= d.iend) return (double)(real)side_ghost(S, d, W, K, q, SIDE_E, i - d.iend, j);
    if (i < d.i0) return (double)(real)side_ghost(S, d, W, K, q, SIDE_W, d.i0 - 1 - i, j);
    if (j >= d.iend) return (double)(real)side_ghost(S, d, W, K, q, SIDE_N, j - d.iend, i);
    if (j < d.i0) return (double)(real)side_ghost(S, d, W, K, q, SIDE_S, d.i0 - 1 - j, i);
    return S.interior(d, q, i, j);
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

}  // namespace csadv
