// Shared device definitions for the csadv kernels.
//
// Layout in HBM ("native" layout).  A cell-centred field of one tracer is 6 panel planes;
// plane p holds rows i (x direction, 0..n-1) of `pitch` elements, columns j (y direction,
// contiguous).  n = N + 8 (4 ghost cells per side, interior [4, N+4) in both directions,
// as cs_datastruct.py:225-237).  Edge fields use the same planes with one extra row
// (x-edges, pu: rows 0..n) or one extra column (y-edges, pv: columns 0..n); every plane
// therefore has n+1 rows.  The pitch is a multiple of 32 elements so every row starts on
// a 256-byte boundary.  The reference's A[i, j, p] (p fastest) is converted to and from
// this layout only at the host boundary.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace csadv {

constexpr int NG = 4;        // ghost cells per side
constexpr int NFACE = 6;     // panels
constexpr int SIDE_E = 0, SIDE_W = 1, SIDE_N = 2, SIDE_S = 3;

struct Dims {
    int N;          // cells per panel edge
    int n;          // N + 8
    int pitch;      // elements per row
    int i0, iend;   // interior [i0, iend) in both directions
    long long plane;  // elements per panel plane = (n + 1) * pitch
    long long field;  // elements per field = 6 * plane
};

inline Dims make_dims(int N) {
    Dims d;
    d.N = N;
    d.n = N + 2 * NG;
    d.pitch = ((d.n + 1 + 31) / 32) * 32;
    d.i0 = NG;
    d.iend = NG + N;
    d.plane = (long long)(d.n + 1) * d.pitch;
    d.field = NFACE * d.plane;
    return d;
}

__host__ __device__ __forceinline__ long long at(const Dims &d, int p, int i, int j) {
    return p * d.plane + (long long)i * d.pitch + j;
}
// single metric plane (identical for every panel: cs_datastruct.py:417,430,445)
__host__ __device__ __forceinline__ long long at2(const Dims &d, int i, int j) {
    return (long long)i * d.pitch + j;
}

// Panel connectivity: for panel p and side s, {neighbour q, side of q, reversed}.
// Derived from the reference's halo gathers (halo_data.py:33-182).  A ghost cell at depth
// d outside side s of p maps to the cell at depth d inside side qs of q; the along-edge
// index k maps to n-1-k when `reversed`.
struct Conn {
    int8_t q, qs, rev;
};
#define CSADV_CONN_TABLE                                                          \
    {                                                                             \
        /* 0 */ {{1, SIDE_W, 0}, {3, SIDE_E, 0}, {4, SIDE_S, 0}, {5, SIDE_N, 0}},  \
        /* 1 */ {{2, SIDE_W, 0}, {0, SIDE_E, 0}, {4, SIDE_E, 0}, {5, SIDE_E, 1}},  \
        /* 2 */ {{3, SIDE_W, 0}, {1, SIDE_E, 0}, {4, SIDE_N, 1}, {5, SIDE_S, 1}},  \
        /* 3 */ {{0, SIDE_W, 0}, {2, SIDE_E, 0}, {4, SIDE_W, 1}, {5, SIDE_W, 0}},  \
        /* 4 */ {{1, SIDE_N, 0}, {3, SIDE_N, 1}, {2, SIDE_N, 1}, {0, SIDE_N, 0}},  \
        /* 5 */ {{1, SIDE_S, 1}, {3, SIDE_S, 0}, {0, SIDE_S, 0}, {2, SIDE_S, 1}},  \
    }
// one copy per translation unit (no relocatable device code)
static __constant__ Conn c_conn[NFACE][4] = CSADV_CONN_TABLE;
static const Conn h_conn[NFACE][4] = CSADV_CONN_TABLE;

// +1 when the outward normal of a side is the positive coordinate direction (E, N)
__host__ __device__ __forceinline__ int side_sign(int s) { return (s == SIDE_E || s == SIDE_N) ? 1 : -1; }
// sign between p's and q's coordinate directions across the shared edge (vector quantities)
__host__ __device__ __forceinline__ int vec_sign(int s, int qs) { return -side_sign(s) * side_sign(qs); }

// (i, j) of the cell at depth d inside side s, along-edge index k
__host__ __device__ __forceinline__ void inside_ij(const Dims &d, int s, int dep, int k, int &i, int &j) {
    switch (s) {
        case SIDE_W: i = d.i0 + dep; j = k; break;
        case SIDE_E: i = d.iend - 1 - dep; j = k; break;
        case SIDE_S: i = k; j = d.i0 + dep; break;
        default: i = k; j = d.iend - 1 - dep; break;
    }
}
// (i, j) of the ghost cell at depth d outside side s, along-edge index k
__host__ __device__ __forceinline__ void ghost_ij(const Dims &d, int s, int dep, int k, int &i, int &j) {
    switch (s) {
        case SIDE_E: i = d.iend + dep; j = k; break;
        case SIDE_W: i = d.i0 - 1 - dep; j = k; break;
        case SIDE_N: i = k; j = d.iend + dep; break;
        default: i = k; j = d.i0 - 1 - dep; break;
    }
}
__host__ __device__ __forceinline__ bool is_interior(const Dims &d, int k) { return k >= d.i0 && k < d.iend; }

// Device-resident grid of one resolution N (FP64, built by build_grid).
struct Grid {
    Dims d;
    double dx;
    // metric tensor sqrt(g) at centres / x-edges / y-edges: one plane each
    const double *g_pc, *g_pu, *g_pv;
    // lon/lat at centres and edges: 6 planes each
    const double *lon_pc, *lat_pc, *lon_pu, *lat_pu, *lon_pv, *lat_pv;
    // lat-lon <-> contravariant coefficients: [0] ex.elon [1] ex.elat [2] ey.elon [3] ey.elat [4] det
    const double *cu[5], *cv[5], *cc[4];
    // Lagrange ghost-cell weights [depth][k][m] and stencil starts [depth][k] (lagrange.py:28-163)
    const double *lag_w;
    const int *lag_k;
    // the FP32 form's ghost-cell stencils, flattened per ghost cell (halo.cuh, built by grid.cu):
    // side-strip rows [panel][side][depth][k] of 4 terms, corner-block rows of 16
    const struct GhostTerm *gside, *gcorner;
    double a2;  // sum over the interior of g_pc^2, all panels (MF-PR denominator)
};

// Wind state, shared by every tracer of a plan, in the state's precision (see wind.cu).
struct Winds {
    int esize = 8;                // bytes per element (8: float64, 4: float32)
    void *u_pu = nullptr, *v_pv = nullptr;      // contravariant wind at x-edges / y-edges
    void *u_old = nullptr, *v_old = nullptr;    // previous step (RK2)
    void *u_avg = nullptr, *v_avg = nullptr;    // departure-point (time-averaged) winds
    void *ulon_pc = nullptr, *vlat_pc = nullptr;  // lat-lon wind at centres (ET-DG halo), contiguous
    void *tab[2] = {nullptr, nullptr};  // time-independent wind coefficients (x-, y-edges)
    int tkind = 0;                // 0: static wind, 1: deformational (6 coefs), 2: separable (1 coef)
    void *clock = nullptr;        // device clock (step count, time of the current wind)
    // fused engine: the time-dependent wind as coefficient fields of a time basis on every
    // edge (ghost edges included), nbasis fields per direction; 0 = not used
    void *btab[2] = {nullptr, nullptr};
    void *btabT = nullptr;        // FP32: the y-edge coefficients transposed ([j][i], as the y-edge records)
    int nbasis = 0;
};

__host__ __device__ __forceinline__ int ceil_div(long long a, int b) { return (int)((a + b - 1) / b); }

}  // namespace csadv
