// Lat-lon output of a cubed-sphere field (the reference's plotting path, made headless).
//
//  ll2cs             -- for points (X, Y, Z) on the unit sphere, the panel and the (i, j) of
//                       the cubed-sphere cell each falls in (interpolation.py:38-140): the
//                       panel is the face whose axis has the largest |coordinate| (Lauritzen
//                       et al. 2015), the point is mapped back to the panel's angles by the
//                       inverse equiangular gnomonic map (cs_transform.py:101-126), and the
//                       angles are binned on the N cells of [-pi/4, pi/4].
//  nearest_neighbour -- the field at those cells (interpolation.py:145-150).
//
// Integer results: the panel rule reproduces the reference's order of masks (a later panel
// wins a tie of |coordinates|), the angle is binned with the reference's floating-point
// expression floor((x + a) / dx).  Host arrays that are page-locked are read and written in
// place; pageable ones go through stream-ordered device buffers.
#include <cmath>
#include <cstdint>

#include "common.cuh"
#include "internal.h"
#include "plan.h"

namespace csadv {

__global__ void k_ll2cs(int N, const double *__restrict__ X, const double *__restrict__ Y,
                        const double *__restrict__ Z, long long n, uint32_t *ci, uint32_t *cj, uint32_t *cp) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= n) return;
    const double x = X[t], y = Y[t], z = Z[t];
    const double ax = fabs(x), ay = fabs(y), az = fabs(z);
    const double pm = fmax(fmax(ax, ay), az);
    // masks in the reference's order; the last one that holds sets the panel
    uint32_t p = 0;
    if (pm == ax && x > 0.0) p = 0;
    if (pm == ay && y > 0.0) p = 1;
    if (pm == ax && x < 0.0) p = 2;
    if (pm == ay && y < 0.0) p = 3;
    if (pm == az && z > 0.0) p = 4;
    if (pm == az && z <= 0.0) p = 5;
    double tx, ty;  // cs_transform.py:101-126
    switch (p) {
        case 0: tx = y / x; ty = z / x; break;
        case 1: tx = -x / y; ty = z / y; break;
        case 2: tx = y / x; ty = -z / x; break;
        case 3: tx = -x / y; ty = -z / y; break;
        case 4: tx = y / z; ty = -x / z; break;
        default: tx = -y / z; ty = -x / z; break;
    }
    const double a = (3.141592653589793 * 0.5) * 0.5, dx = 2.0 * a / N, xmin = -a;  // pio4 (constants.py:20-22)
    const double fi = floor((atan(tx) - xmin) / dx), fj = floor((atan(ty) - xmin) / dx);
    ci[t] = (uint32_t)(long long)fi;
    cj[t] = (uint32_t)(long long)fj;
    cp[t] = p;
}

// out[t] = Q(i0 + ci[t], i0 + cj[t], cp[t]); an index out of range gives NaN and sets *bad
template <class real>
__global__ void k_nearest(const real *__restrict__ Q, Dims d, const uint32_t *__restrict__ ci,
                          const uint32_t *__restrict__ cj, const uint32_t *__restrict__ cp, long long n, double *out,
                          int *bad) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= n) return;
    const uint32_t i = ci[t], j = cj[t], p = cp[t];
    if (i >= (uint32_t)d.N || j >= (uint32_t)d.N || p >= (uint32_t)NFACE) {
        out[t] = nan("");
        *bad = 1;
        return;
    }
    out[t] = (double)Q[at(d, (int)p, d.i0 + (int)i, d.i0 + (int)j)];
}

}  // namespace csadv

using namespace csadv;

extern "C" {

int csadv_ll2cs(int N, const double *X, const double *Y, const double *Z, long long n, uint32_t *i, uint32_t *j,
                uint32_t *panel, void *stream) {
    if (N < 1 || n < 0 || !X || !Y || !Z || !i || !j || !panel) return CSADV_ERR_ARG;
    if (n == 0) return CSADV_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t bd = (size_t)n * sizeof(double), bu = (size_t)n * sizeof(uint32_t);
    DevArray ax, ay, az, oi, oj, op;
    int rc = dev_in(X, bd, st, ax);
    if (!rc) rc = dev_in(Y, bd, st, ay);
    if (!rc) rc = dev_in(Z, bd, st, az);
    if (!rc) rc = dev_out(i, bu, st, oi);
    if (!rc) rc = dev_out(j, bu, st, oj);
    if (!rc) rc = dev_out(panel, bu, st, op);
    if (!rc) {
        k_ll2cs<<<ceil_div(n, 256), 256, 0, st>>>(N, (const double *)ax.dev, (const double *)ay.dev,
                                                 (const double *)az.dev, n, (uint32_t *)oi.dev, (uint32_t *)oj.dev,
                                                 (uint32_t *)op.dev);
        if (cudaGetLastError() != cudaSuccess) rc = CSADV_ERR_CUDA;
    }
    if (!rc) rc = dev_back(i, bu, st, oi);
    if (!rc) rc = dev_back(j, bu, st, oj);
    if (!rc) rc = dev_back(panel, bu, st, op);
    for (DevArray *a : {&ax, &ay, &az, &oi, &oj, &op}) dev_free(*a, st);
    if (cudaStreamSynchronize(st) != cudaSuccess && !rc) rc = CSADV_ERR_CUDA;
    return rc;
}

int csadv_nearest_neighbour(csadv_plan *pl, int tracer, const uint32_t *i, const uint32_t *j, const uint32_t *panel,
                            long long n, double *out, void *stream) {
    if (!pl || tracer < 0 || tracer >= pl->T || n < 0 || !i || !j || !panel || !out) return CSADV_ERR_ARG;
    if (n == 0) return CSADV_OK;
    cudaStream_t st = (cudaStream_t)stream;
    int rc = plan_select_device(pl);
    if (!rc) rc = plan_settle(pl, st);  // the stored state is the true state
    if (rc) return rc;
    const size_t bu = (size_t)n * sizeof(uint32_t), bd = (size_t)n * sizeof(double);
    DevArray ai, aj, ap, ao, flag;
    rc = dev_in(i, bu, st, ai);
    if (!rc) rc = dev_in(j, bu, st, aj);
    if (!rc) rc = dev_in(panel, bu, st, ap);
    if (!rc) rc = dev_out(out, bd, st, ao);
    if (!rc) {
        if (cudaMallocAsync(&flag.dev, sizeof(int), st) != cudaSuccess) rc = CSADV_ERR_CUDA;
        flag.owned = true;
        if (!rc && cudaMemsetAsync(flag.dev, 0, sizeof(int), st) != cudaSuccess) rc = CSADV_ERR_CUDA;
    }
    if (!rc) {
        const Dims d = pl->grid.d;
        if (pl->opt.precision == 64)
            k_nearest<double><<<ceil_div(n, 256), 256, 0, st>>>((const double *)pl->tracer(tracer), d,
                                                                (const uint32_t *)ai.dev, (const uint32_t *)aj.dev,
                                                                (const uint32_t *)ap.dev, n, (double *)ao.dev,
                                                                (int *)flag.dev);
        else
            k_nearest<float><<<ceil_div(n, 256), 256, 0, st>>>((const float *)pl->tracer(tracer), d,
                                                               (const uint32_t *)ai.dev, (const uint32_t *)aj.dev,
                                                               (const uint32_t *)ap.dev, n, (double *)ao.dev,
                                                               (int *)flag.dev);
        if (cudaGetLastError() != cudaSuccess) rc = CSADV_ERR_CUDA;
    }
    if (!rc) rc = dev_back(out, bd, st, ao);
    int bad = 0;
    if (!rc && cudaMemcpyAsync(&bad, flag.dev, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        rc = CSADV_ERR_CUDA;
    for (DevArray *a : {&ai, &aj, &ap, &ao, &flag}) dev_free(*a, st);
    if (cudaStreamSynchronize(st) != cudaSuccess && !rc) rc = CSADV_ERR_CUDA;
    if (!rc && bad) rc = CSADV_ERR_ARG;
    return rc;
}

}  // extern "C"
