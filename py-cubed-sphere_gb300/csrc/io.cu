// Tracer initialisation, host-layout conversion and FP64 diagnostics.
//
//  init_tracer  -- q0_adv (advection_ic.py:208-210) at the interior cell centres
//                  (a point value, as advection_vars.py:105)
//  tracer_io    -- reference layout A[i][j][p] (full or interior) <-> native pitched planes
//  diag_mass    -- mass_computation (diagnostics.py:14-26)
//  diag_errors  -- compute_errors vs qexact_adv (errors.py:99-113)
// All sums are FP64 with a fixed reduction order (block partials, then one block).
#include <cmath>

#include "cases.cuh"
#include "common.cuh"
#include "halo.cuh"
#include "internal.h"

namespace csadv {

constexpr int RB = 256;  // reduction block

// maximum that propagates NaN, as numpy.max does in the reference's compute_errors (fmax would
// drop a NaN and report a finite Linf for a state that holds one)
__device__ __forceinline__ double max_nan(double a, double b) { return (a > b || a != a) ? a : b; }

template <class real>
__global__ void k_init(Grid g, int ic, int vf, IcParams prm, real *Q) {
    const Dims d = g.d;
    const int N = d.N;
    long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= (long long)NFACE * N * N) return;
    int j = d.i0 + (int)(tid % N), i = d.i0 + (int)((tid / N) % N), p = (int)(tid / ((long long)N * N));
    long long o = at(d, p, i, j);
    Q[o] = (real)qexact(ic, prm.ic, vf, prm.wind, g.lon_pc[o], g.lat_pc[o], 0.0);
}

// host index (reference layout) of cell (p, i, j) of the native layout
__device__ __forceinline__ long long host_index(const Dims &d, int layout, int p, int i, int j) {
    if (layout == CSADV_LAYOUT_FULL) return ((long long)i * d.n + j) * NFACE + p;
    return ((long long)(i - d.i0) * d.N + (j - d.i0)) * NFACE + p;
}

// Reference layout A[i][j][p] (p fastest) <-> native planes, IO_B cells per block: the block's
// 6 IO_B host values form one contiguous range, copied between the host array and shared memory
// with consecutive lanes on consecutive addresses (16 bytes per lane when the host array is
// 16-byte aligned), so the interconnect sees whole lines; each thread then moves the six panel
// values of one cell, consecutive threads on consecutive columns of each plane.  `host` may be a
// device buffer or page-locked host memory mapped into the device.  `x` adds the work on the
// fused engine's state (the pending correction, the mass record) to the same pass.
__device__ __forceinline__ double block_sum(double v, double *ws) {
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, s));
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
#pragma unroll
        for (int w = 0; w < IO_B / 32; ++w) t = __dadd_rn(t, ws[w]);
    __syncthreads();
    return t;  // thread 0
}

template <class real, bool VEC>
__global__ void __launch_bounds__(IO_B) k_io(Dims d, real *Q, double *host, int layout, int to_native, IoLazy<real> x) {
    __shared__ __align__(16) double s[IO_B * NFACE];
    __shared__ double ws[IO_B / 32];
    __shared__ int last;
    const int m = layout == CSADV_LAYOUT_FULL ? d.n : d.N;
    const int off = layout == CSADV_LAYOUT_FULL ? 0 : d.i0;
    const long long cell0 = (long long)blockIdx.x * IO_B, ncell = (long long)m * m;
    const int nc = (int)(ncell - cell0 < IO_B ? ncell - cell0 : IO_B);
    double *h = host + cell0 * NFACE;
    const int tid = threadIdx.x;
    const long long cell = cell0 + tid;
    const int i = off + (int)(cell / m), j = off + (int)(cell % m);
    const long long o = at2(d, i, j);
    const bool inner = tid < nc && i >= d.i0 && i < d.iend && j >= d.i0 && j < d.iend;
    if (to_native) {
        if (VEC)
            for (int e = tid; e < nc * NFACE / 2; e += IO_B) ((double2 *)s)[e] = ((const double2 *)h)[e];
        else
            for (int e = tid; e < nc * NFACE; e += IO_B) s[e] = h[e];
        __syncthreads();
        double mp = 0.0;
        const double gw = x.mass && inner ? (double)x.g[o] : 0.0;
        if (tid < nc)
#pragma unroll
            for (int p = 0; p < NFACE; ++p) {
                const real v = (real)s[tid * NFACE + p];
                Q[p * d.plane + o] = v;
                if (x.mass && inner) mp = __dadd_rn(mp, __dmul_rn((double)v, gw));
            }
        if (x.corr && blockIdx.x == 0 && tid == 0) *x.corr = 0.0;
        if (x.mass) {  // the same for every block
            mp = block_sum(mp, ws);
            if (tid == 0) {
                x.part[blockIdx.x] = mp;
                __threadfence();
                last = atomicAdd(x.count, 1u) == gridDim.x - 1;
            }
            __syncthreads();
            if (last) {
                __threadfence();
                double a = 0.0;
                // each thread adds its partials in block order; the loads of a batch are issued
                // together (one L2 round trip per 8 partials, not one per partial)
                constexpr int BATCH = 8;
                for (int b0 = tid; b0 < (int)gridDim.x; b0 += BATCH * IO_B) {
                    double v[BATCH];
#pragma unroll
                    for (int k = 0; k < BATCH; ++k) {
                        const int b = b0 + k * IO_B;
                        v[k] = b < (int)gridDim.x ? __ldcg(x.part + b) : 0.0;
                    }
#pragma unroll
                    for (int k = 0; k < BATCH; ++k)
                        if (b0 + k * IO_B < (int)gridDim.x) a = __dadd_rn(a, v[k]);
                }
                a = block_sum(a, ws);
                if (tid == 0) {
                    *x.mass = a;
                    *x.count = 0u;
                }
            }
        }
    } else {
        if (tid < nc) {
            const bool fix = x.corr && inner;
            const real c = fix ? (real)*x.corr : real(0), gc = fix ? x.g[o] : real(0);
#pragma unroll
            for (int p = 0; p < NFACE; ++p) {
                const real v = Q[p * d.plane + o];
                s[tid * NFACE + p] = (double)(fix ? corrected(v, gc, c) : v);
            }
        }
        __syncthreads();
        if (VEC)
            for (int e = tid; e < nc * NFACE / 2; e += IO_B) ((double2 *)h)[e] = ((const double2 *)s)[e];
        else
            for (int e = tid; e < nc * NFACE; e += IO_B) h[e] = s[e];
    }
}

template <class real>
__global__ void k_mass_part(Dims d, const real *__restrict__ Q, const double *__restrict__ g, double dx,
                            double *part) {
    __shared__ double red[RB];
    const int N = d.N;
    long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    double v = 0.0;
    if (tid < (long long)NFACE * N * N) {
        int j = d.i0 + (int)(tid % N), i = d.i0 + (int)((tid / N) % N), p = (int)(tid / ((long long)N * N));
        v = (double)Q[at(d, p, i, j)] * g[at2(d, i, j)] * dx * dx;
    }
    red[threadIdx.x] = v;
    __syncthreads();
    for (int s = RB / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

template <class real>
__global__ void k_err_part(Grid g, const real *__restrict__ Q, int ic, int vf, IcParams prm, double t, double *part) {
    __shared__ double rmax[RB], rs1[RB], rs2[RB];
    const Dims d = g.d;
    const int N = d.N;
    long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    double e = 0.0;
    if (tid < (long long)NFACE * N * N) {
        int j = d.i0 + (int)(tid % N), i = d.i0 + (int)((tid / N) % N), p = (int)(tid / ((long long)N * N));
        long long o = at(d, p, i, j);
        double qe = qexact(ic, prm.ic, vf, prm.wind, g.lon_pc[o], g.lat_pc[o], t);
        e = fabs(qe - (double)Q[o]);
    }
    rmax[threadIdx.x] = e;
    rs1[threadIdx.x] = e;
    rs2[threadIdx.x] = e * e;
    __syncthreads();
    for (int s = RB / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            rmax[threadIdx.x] = max_nan(rmax[threadIdx.x], rmax[threadIdx.x + s]);
            rs1[threadIdx.x] += rs1[threadIdx.x + s];
            rs2[threadIdx.x] += rs2[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[3 * blockIdx.x + 0] = rmax[0];
        part[3 * blockIdx.x + 1] = rs1[0];
        part[3 * blockIdx.x + 2] = rs2[0];
    }
}

// fixed-order reduction of `np` groups of `w` partials (w = 1: sum; w = 3: max, sum, sum)
__global__ void k_reduce(const double *__restrict__ part, int np, int w, double *out) {
    __shared__ double r0[1024], r1[1024], r2[1024];
    double a = w == 3 ? 0.0 : 0.0, b = 0.0, c = 0.0;
    for (int t = threadIdx.x; t < np; t += blockDim.x) {
        if (w == 1) {
            a += part[t];
        } else {
            a = max_nan(a, part[3 * t]);
            b += part[3 * t + 1];
            c += part[3 * t + 2];
        }
    }
    r0[threadIdx.x] = a;
    r1[threadIdx.x] = b;
    r2[threadIdx.x] = c;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            r0[threadIdx.x] = w == 1 ? r0[threadIdx.x] + r0[threadIdx.x + s] : max_nan(r0[threadIdx.x], r0[threadIdx.x + s]);
            r1[threadIdx.x] += r1[threadIdx.x + s];
            r2[threadIdx.x] += r2[threadIdx.x + s];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = r0[0];
        out[1] = r1[0];
        out[2] = r2[0];
    }
}

int diag_partials(const Grid &g) { return ceil_div((long long)NFACE * g.d.N * g.d.N, RB); }

template <class real>
int init_tracer(const Grid &g, int ic, int vf, const IcParams &prm, real *Q, cudaStream_t st) {
    long long tot = (long long)NFACE * g.d.N * g.d.N;
    k_init<real><<<ceil_div(tot, 128), 128, 0, st>>>(g, ic, vf, prm, Q);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

template <class real>
int tracer_io(const Grid &g, real *Q, double *dev_stage, int layout, bool to_native, cudaStream_t st,
              const IoLazy<real> *lazy) {
    const int m = layout == CSADV_LAYOUT_FULL ? g.d.n : g.d.N;
    const long long tot = (long long)m * m;
    const IoLazy<real> x = lazy ? *lazy : IoLazy<real>{};
    if (((uintptr_t)dev_stage & 15) == 0)
        k_io<real, true><<<ceil_div(tot, IO_B), IO_B, 0, st>>>(g.d, Q, dev_stage, layout, to_native ? 1 : 0, x);
    else
        k_io<real, false><<<ceil_div(tot, IO_B), IO_B, 0, st>>>(g.d, Q, dev_stage, layout, to_native ? 1 : 0, x);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

template <class real>
int diag_mass(const Grid &g, const real *Q, double *tmp, double &mass, cudaStream_t st) {
    int np = diag_partials(g);
    k_mass_part<real><<<np, RB, 0, st>>>(g.d, Q, g.g_pc, g.dx, tmp);
    k_reduce<<<1, 1024, 0, st>>>(tmp, np, 1, tmp + 3 * np);
    CSADV_CUDA(cudaGetLastError());
    double h[3];
    CSADV_CUDA(cudaMemcpyAsync(h, tmp + 3 * np, sizeof(h), cudaMemcpyDeviceToHost, st));
    CSADV_CUDA(cudaStreamSynchronize(st));
    mass = h[0];
    return CSADV_OK;
}

template <class real>
int diag_errors(const Grid &g, const real *Q, int ic, int vf, const IcParams &prm, double t, double *tmp,
                double out[3], cudaStream_t st) {
    int np = diag_partials(g);
    k_err_part<real><<<np, RB, 0, st>>>(g, Q, ic, vf, prm, t, tmp);
    k_reduce<<<1, 1024, 0, st>>>(tmp, np, 3, tmp + 3 * np);
    CSADV_CUDA(cudaGetLastError());
    double h[3];
    CSADV_CUDA(cudaMemcpyAsync(h, tmp + 3 * np, sizeof(h), cudaMemcpyDeviceToHost, st));
    CSADV_CUDA(cudaStreamSynchronize(st));
    const double n = (double)NFACE * g.d.N * g.d.N;
    out[0] = h[0];
    out[1] = h[1] / n;
    out[2] = sqrt(h[2] / n);
    return CSADV_OK;
}

#define INST(real)                                                                                       \
    template int init_tracer<real>(const Grid &, int, int, const IcParams &, real *, cudaStream_t);     \
    template int tracer_io<real>(const Grid &, real *, double *, int, bool, cudaStream_t, const IoLazy<real> *); \
    template int diag_mass<real>(const Grid &, const real *, double *, double &, cudaStream_t);         \
    template int diag_errors<real>(const Grid &, const real *, int, int, const IcParams &, double, double *, \
                                   double *, cudaStream_t);
INST(double)
INST(float)
#undef INST

}  // namespace csadv
