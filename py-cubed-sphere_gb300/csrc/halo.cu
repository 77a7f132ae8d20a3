// Ghost cells of cell-centred fields across the cube edges.
//
// k_halo_dg       -- ET-DG: degree-3 Lagrange interpolation along the neighbour panel's
//                    edge (interpolation.py:154-314 with halo_data.py:15-185).  The
//                    reference fills the four side strips first and then the 4x4 corner
//                    blocks from the refreshed halo of the east/west neighbours.  Here one
//                    launch does both: a corner thread recomputes the neighbour's side-strip
//                    values it needs (same operations, same bits) instead of waiting for
//                    them, so no grid-wide barrier is needed and no thread reads a ghost cell
//                    that another thread writes.
// k_halo_adjacent -- ET-S72 / ET-PL07: copy of the neighbour's cells (interpolation.py:320-340,
//                    halo_data.py:191-400).  Only the strips along the interior of each edge
//                    are written; the reference also writes the corner blocks, but with
//                    these edge treatments no corner value reaches an interior result.
//
// Both are compiled without FMA contraction: each product and sum is rounded as in numpy,
// so the FP64 form reproduces the reference's halo values bit for bit.
#include "common.cuh"
#include "halo.cuh"
#include "internal.h"
#include "tiles.h"

namespace csadv {

// blockIdx.y = tracer (fields `fstride` elements apart); corr[tracer] optional
template <class real>
__global__ void k_halo_dg(real *F0, long long fstride, Dims d, const double *__restrict__ W,
                          const int *__restrict__ K, const GhostTerm *__restrict__ gside,
                          const GhostTerm *__restrict__ gcorner, const double *__restrict__ corr,
                          const real *__restrict__ g) {
    const int n = d.n;
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= NFACE * 4 * NG * n) return;
    real *F = F0 + blockIdx.y * fstride;
    Src<real> S{F, g, corr ? (real)corr[blockIdx.y] : real(0), corr != nullptr};
    int k = tid % n;
    int dep = (tid / n) % NG;
    int s = (tid / (n * NG)) % 4;
    int p = tid / (n * NG * 4);
    int gi, gj;
    ghost_ij(d, s, dep, k, gi, gj);
    if (!is_interior(d, k) && (s == SIDE_N || s == SIDE_S)) return;  // corner blocks: from the E/W sides
    F[at(d, p, gi, gj)] = ghost_cell(S, d, W, K, gside, gcorner, p, gi, gj);
}

// ghost cells of many solves in one launch: item (s, b) of the work table is block b % nb of
// tracer b / nb of solve s (descriptor s: its input buffer and pending correction), nb =
// halo_blocks; the same work per thread as k_halo_dg
template <class real>
__global__ void k_halo_batch(const SweepSolve *__restrict__ solves, const int2 *__restrict__ work, int nwork) {
    for (int wk = blockIdx.x; wk < nwork; wk += gridDim.x) {
        const int2 it = work[wk];
        const SweepSolve &S = solves[it.x];
        const Dims d = S.d;
        const int n = d.n, nb = halo_blocks(d);
        const int tr = it.y / nb;
        const int tid = (it.y % nb) * 128 + threadIdx.x;
        if (tid >= NFACE * 4 * NG * n) continue;
        real *F = (real *)S.Qin + (long long)tr * d.field;
        const bool hc = S.corr_in != nullptr;
        Src<real> src{F, (const real *)S.gpc, hc ? (real)S.corr_in[tr] : real(0), hc};
        const int k = tid % n, dep = (tid / n) % NG, s = (tid / (n * NG)) % 4, p = tid / (n * NG * 4);
        int gi, gj;
        ghost_ij(d, s, dep, k, gi, gj);
        if (is_interior(d, k) || s == SIDE_E || s == SIDE_W) {  // corner blocks, from the E/W sides
            F[at(d, p, gi, gj)] = ghost_cell(src, d, S.hlag_w, S.hlag_k, S.gside, S.gcorner, p, gi, gj);
        }
    }
}

template <class real>
int launch_halo_batch(const SweepSolve *dsolves, const int2 *work, int nwork, cudaStream_t st) {
    if (nwork <= 0) return CSADV_OK;
    k_halo_batch<real><<<nwork, 128, 0, st>>>(dsolves, work, nwork);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}
template int launch_halo_batch<double>(const SweepSolve *, const int2 *, int, cudaStream_t);
template int launch_halo_batch<float>(const SweepSolve *, const int2 *, int, cudaStream_t);

template <class real>
__global__ void k_halo_adjacent(real *Qx, real *Qy, Dims d) {
    const int N = d.N;
    int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= NFACE * 4 * NG * N) return;
    int k = d.i0 + tid % N;
    int dep = (tid / N) % NG;
    int s = (tid / (N * NG)) % 4;
    int p = tid / (N * NG * 4);
    const Conn c = c_conn[p][s];
    real *dst = (s == SIDE_E || s == SIDE_W) ? Qy : Qx;
    const real *src = (c.qs == SIDE_E || c.qs == SIDE_W) ? Qy : Qx;
    int along = c.rev ? d.n - 1 - k : k;
    int si, sj, gi, gj;
    inside_ij(d, c.qs, dep, along, si, sj);
    ghost_ij(d, s, dep, k, gi, gj);
    dst[at(d, p, gi, gj)] = src[at(d, c.q, si, sj)];
}

template <class real>
int launch_halo_dg(real *F, const Grid &g, cudaStream_t st) {
    int tot = NFACE * 4 * NG * g.d.n;
    k_halo_dg<real><<<ceil_div(tot, 128), 128, 0, st>>>(F, 0, g.d, g.lag_w, g.lag_k, g.gside, g.gcorner, nullptr,
                                                        nullptr);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

template <class real>
int launch_halo_dg_tracers(real *F, int T, const Grid &g, const double *corr, const real *greal, cudaStream_t st) {
    int tot = NFACE * 4 * NG * g.d.n;
    dim3 grid(ceil_div(tot, 128), T);
    k_halo_dg<real><<<grid, 128, 0, st>>>(F, g.d.field, g.d, g.lag_w, g.lag_k, g.gside, g.gcorner, corr, greal);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

template <class real>
int launch_halo_adjacent(real *Qx, real *Qy, const Grid &g, cudaStream_t st) {
    int tot = NFACE * 4 * NG * g.d.N;
    k_halo_adjacent<real><<<ceil_div(tot, 128), 128, 0, st>>>(Qx, Qy, g.d);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

template int launch_halo_dg<double>(double *, const Grid &, cudaStream_t);
template int launch_halo_dg<float>(float *, const Grid &, cudaStream_t);
template int launch_halo_dg_tracers<double>(double *, int, const Grid &, const double *, const double *,
                                            cudaStream_t);
template int launch_halo_dg_tracers<float>(float *, int, const Grid &, const double *, const float *, cudaStream_t);
template int launch_halo_adjacent<double>(double *, double *, const Grid &, cudaStream_t);
template int launch_halo_adjacent<float>(float *, float *, const Grid &, cudaStream_t);

}  // namespace csadv
