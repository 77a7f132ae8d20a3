// Launch descriptors and tile geometry of the fused engine's step kernels, shared by the
// host code and the kernels.  No kernels here: the kernel templates live in fused.cuh and
// sweep.cuh and are instantiated only in fused_f32/f64.cu and sweep_f32/f64.cu (one device
// copy of each kernel in the library).
#pragma once
#include <cstddef>
#include <cstdint>

#include "common.cuh"

namespace csadv {

// a pair of the state's precision (edge and cell records of the line-marching kernel)
template <class real> struct Vec2;
template <> struct Vec2<float> { using type = float2; };
template <> struct Vec2<double> { using type = double2; };

// ---------------------------------------------------------------- per-edge tile kernel (k_fused)
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

// tile shapes selectable per launch (the autotuner times them): {TI, TJ}
constexpr int FUSED_TILES[][2] = {{16, 58}, {32, 58}, {16, 26}, {32, 26}};
constexpr int FUSED_NTILE_CFG = 4;

// number of CTAs of a launch with tile shape `tile`
inline int fused_blocks(const Dims &d, int tile) {
    int TI = FUSED_TILES[tile][0], TJ = FUSED_TILES[tile][1];
    return NFACE * ((d.N + TI - 1) / TI) * ((d.N + TJ - 1) / TJ);
}

// ---------------------------------------------------------------- line-marching kernel (k_sweep)
// One solve's part of a sweep launch (device memory; one per solve and buffer parity).
struct SweepSolve {
    Dims d;
    int T;                  // tracers
    int ti, tj;             // tile shape (interior cells); ti + 6 <= 64, tj + 6 <= 64
    int ntj, ntiles;        // tiles along j; tiles per panel (items = 6 ntiles)
    int s1x, s1y, s2y, s2x; // segments per line in P1 (x, y), P2, P3
    double dt, dx, a2;
    float dtdx, irdx;       // dt / dx and 1 / dx rounded to FP32 (the FP32 kernel's step constants)
    const void *Qin;        // T fields, ghost cells filled
    void *Qout;             // T fields, interior written
    const double *corr_in;  // [T] pending MF-PR correction of Qin, or null
    double *corr_out;       // [T] correction of Qout (MF-PR)
    double *partials;       // [T][6 ntiles]
    unsigned int *counter;  // arrival counter (MF-PR)
    // edge records {departure-point wind, +-metric at the edge; the sign is the upwind flag,
    // + when the wind is >= 0}: x-edges natural (row i, column j), y-edges transposed (row j,
    // column i); per panel plane, element type vec2 of the state's precision.  FP64: the edges'
    // flux coefficients {alpha, beta} at erx + ecofs and {gamma, alpha + beta + gamma} at erx + 2 ecofs (units of
    // double2; flux_coefs and put_record in wind.cu); ecofs 0 in the FP32 form, which has none
    const void *erx, *ery;
    long long ecofs;
    // cell records {metric, 1 / metric}: natural and transposed (one plane)
    const void *crx, *cry;
    const void *gpc;        // metric at the centres (state precision), for the pending correction
    int split, mt, mfpr;
    const double *mass_target;  // FP32 form: per-tracer sum(Q g) that the MF-PR correction restores
                                // (partials then hold sum(Q g)); null: the reference's projection
    const double *lag_w;    // ET-DG ghost-cell weights and stencil starts: when set, the kernel
    const int *lag_k;       // evaluates the ghost cells of its tiles itself; else it reads them
    const double *hlag_w;   // the same tables for the batched ghost-cell kernel (always set)
    const int *hlag_k;
    const struct GhostTerm *gside, *gcorner;  // the FP32 form's flattened ghost-cell stencils
};

// offset (vec2 units) of the flux coefficients behind the edge records of one direction: the
// FP64 line-marching kernel reads them, the FP32 one forms the same terms itself
template <class real>
__host__ __device__ inline long long record_coef_offset(const Dims &d) { return sizeof(real) == 8 ? d.field : 0; }

// blocks of the batched ghost-cell kernel per tracer of a solve (128 ghost-cell columns each)
__host__ __device__ inline int halo_blocks(const Dims &d) { return (NFACE * 4 * NG * d.n + 127) / 128; }

constexpr int SWEEP_THREADS = 256;
// tracer grouping of an FP32 step-kernel launch: tracers of every solve in pairs (all T even), one
// at a time (T = 1), or pairs and an odd last one (any T)
constexpr int SWEEP_TG_ANY = 0, SWEEP_TG_PAIRS = 1, SWEEP_TG_ONE = 2;
inline int sweep_tgroup(int T) { return T == 1 ? SWEEP_TG_ONE : T % 2 == 0 ? SWEEP_TG_PAIRS : SWEEP_TG_ANY; }
// largest tile shapes of the sweep kernels: {ti, tj}; the N cells of each direction are split into
// nearly equal tiles no larger than these (sweep_tile)
constexpr int SWEEP_TILES[][2] = {{55, 55}, {55, 26}, {26, 55}, {26, 26}};
constexpr int SWEEP_NTILE_CFG = 4;
constexpr int SWEEP_TMAX = 55;  // largest ti, tj of any shape

__host__ __device__ __forceinline__ int odd_up(int x) { return x | 1; }
__host__ __device__ __forceinline__ int round32(int x) { return (x + 31) & ~31; }

// shared-memory layout for tile shape (ti, tj), in elements
struct SweepSmem {
    int QJp, TJp;           // row pitches (odd): Q/Qx rows hold tj+6 cells, Qy/dY rows tj cells
    int oQx, oQy, oDy, total;
};
__host__ __device__ __forceinline__ SweepSmem sweep_smem(int ti, int tj) {
    SweepSmem s;
    s.QJp = odd_up(tj + 6);
    s.TJp = odd_up(tj);
    s.oQx = (ti + 6) * s.QJp;
    s.oQy = s.oQx + ti * s.QJp;
    s.oDy = s.oQy + (ti + 6) * s.TJp;
    s.total = s.oDy + ti * s.TJp;
    return s;
}

// tile configuration of a solve: shape and segments per line (about 256 threads per phase,
// segments of at least ~10 cells).  The step kernels number a phase's jobs densely (line l,
// segment s at job s * lines + l), so lanes past the last line do not idle inside a warp; the
// counts below, sized with lines rounded up to 32, stay within 256 jobs either way.
inline void sweep_config(SweepSolve &s, int cfg) {
    s.ti = SWEEP_TILES[cfg][0];
    s.tj = SWEEP_TILES[cfg][1];
    const int N = s.d.N;
    const int ti = s.ti < N ? s.ti : N, tj = s.tj < N ? s.tj : N;
    auto segs = [](int threads_per_seg, int len) {
        int k = SWEEP_THREADS / (threads_per_seg > 0 ? threads_per_seg : 1);
        int kmax = len / 10 > 1 ? len / 10 : 1;
        if (k > kmax) k = kmax;
        return k > 0 ? k : 1;
    };
    s.s1x = segs(round32(tj + 6) + round32(ti + 6), ti);
    s.s1y = segs(round32(tj + 6) + round32(ti + 6), tj);
    s.s2y = segs(round32(ti), tj);
    s.s2x = segs(round32(tj), ti);
    s.ntj = (N + s.tj - 1) / s.tj;
    s.ntiles = ((N + s.ti - 1) / s.ti) * s.ntj;
}

// Rows [I0, I0 + ni) and columns [J0, J0 + nj) (panel indices) of tile `tile` of a solve.  The
// N interior cells of each direction are split into nearly equal parts (sizes differ by at
// most one and never exceed the configured shape), so no CTA carries a full tile while another
// carries a ragged remainder.
__host__ __device__ __forceinline__ void sweep_tile(const SweepSolve &s, int tile, int &I0, int &ni, int &J0,
                                                    int &nj) {
    const int N = s.d.N, nti = s.ntiles / s.ntj;
    const int a = tile / s.ntj, b = tile - a * s.ntj;
    const int ia = N * a / nti, ib = N * (a + 1) / nti;
    const int ja = N * b / s.ntj, jb = N * (b + 1) / s.ntj;
    I0 = s.d.i0 + ia;
    ni = ib - ia;
    J0 = s.d.i0 + ja;
    nj = jb - ja;
}

// Shared-memory layout of the paired-tracer FP32 kernel (k_sweep2): one 8-byte pair of
// tracer values per cell, row pitches fixed at compile time for every tile shape (odd numbers of
// pairs: conflict-free along rows and along columns), ti rows.  Units: pairs.
constexpr int PAIR_QJP = SWEEP_TMAX + 6;  // rows of the Q and Qx tiles (tj + 6 cells)
constexpr int PAIR_TJP = SWEEP_TMAX;      // rows of the Qy and dY tiles (tj cells)
struct PairSmem {
    int oQx, oQy, oDy, total;
};
__host__ __device__ __forceinline__ PairSmem pair_smem(int ti) {
    PairSmem s;
    s.oQx = (ti + 6) * PAIR_QJP;
    s.oQy = s.oQx + ti * PAIR_QJP;
    s.oDy = s.oQy + (ti + 6) * PAIR_TJP;
    s.total = s.oDy + ti * PAIR_TJP + 8;  // + a few pairs: the marching loads run one cell past a line
    return s;
}

template <class real>
inline size_t sweep_smem_bytes(int cfg) {
    return (size_t)sweep_smem(SWEEP_TILES[cfg][0], SWEEP_TILES[cfg][1]).total * sizeof(real);
}
// the FP32 form runs the paired-tracer kernel
template <>
inline size_t sweep_smem_bytes<float>(int cfg) {
    return (size_t)pair_smem(SWEEP_TILES[cfg][0]).total * 2 * sizeof(float);
}

}  // namespace csadv
