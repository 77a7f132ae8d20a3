// Grid generation: gnomonic equiangular cubed sphere, FP64, on the device.
//
// Restates cs_datastruct.py:197-493 (points, tangent vectors, metric tensor, lat-lon /
// contravariant coefficients) with cs_transform.py:41-96 (equiangular map), :245-397
// (tangent vectors) and sphgeo.py:29-33, 72-88.  The 1-D angular coordinates follow
// numpy.linspace exactly (host side) so every later rounding matches the reference's
// sequence of operations; transcendental functions are CUDA's (within 2 ulp of libm).
//
// The Lagrange ghost-cell tables (lagrange.py:28-163) are built on the host from the
// same formulas (they are tiny: 4 x (N+8) entries).
#include <cmath>
#include <cstdio>
#include <vector>

#include "common.cuh"
#include "halo.cuh"
#include "internal.h"

namespace csadv {



// numpy.linspace(start, stop, num): arange(num) * step + start, last element = stop
std::vector<double> linspace(double start, double stop, int num) {
    std::vector<double> y(num);
    double step = (stop - start) / (double)(num - 1);
    for (int i = 0; i < num; ++i) y[i] = (double)i * step + start;
    y[num - 1] = stop;
    return y;
}

void angular_axes(int N, std::vector<double> &xc, std::vector<double> &xe, double &dx) {
    const double a = M_PI / 4.0;
    dx = (a - (-a)) / N;
    xe = linspace(-a - NG * dx, a + NG * dx, N + 1 + 2 * NG);
    xc = linspace(-a + dx / 2.0 - NG * dx, a - dx / 2.0 + NG * dx, N + 2 * NG);
}

// ---------------------------------------------------------------- device geometry
__host__ __device__ inline void panel_xyz(int p, double invD, double XoD, double YoD, double &X, double &Y,
                                          double &Z) {
    switch (p) {  // cs_transform.py:63-91
        case 0: X = invD; Y = XoD; Z = YoD; break;
        case 1: X = -XoD; Y = invD; Z = YoD; break;
        case 2: X = -invD; Y = -XoD; Z = YoD; break;
        case 3: X = XoD; Y = -invD; Z = YoD; break;
        case 4: X = -YoD; Y = XoD; Z = invD; break;
        default: X = YoD; Y = XoD; Z = -invD; break;
    }
}

// equiangular tangent vectors (cs_transform.py:245-397): the equidistant tangent at
// (a tan x, a tan y) scaled by a / cos^2, from the per-axis values tx = tan x, sx = a / cos^2 x
// (and ty, sy); |r|^3 is formed as r^2 |r|
__device__ inline void tangents(int p, double tx, double sx, double ty, double sy, double ex[3], double ey[3]) {
    const double a = 1.0 / sqrt(3.0);
    double xe = a * tx, ye = a * ty;
    double r2 = a * a + xe * xe + ye * ye;
    double invr = 1.0 / (r2 * sqrt(r2));
    double a2 = a * a, ax = a * xe, ay = a * ye, xy = xe * ye;
    double bx = (a2 + ye * ye) * invr, by = (a2 + xe * xe) * invr;
    double axr = ax * invr, ayr = ay * invr, xyr = xy * invr;
    switch (p) {
        case 0: ex[0] = -axr; ex[1] = bx; ex[2] = -xyr; ey[0] = -ayr; ey[1] = -xyr; ey[2] = by; break;
        case 1: ex[0] = -bx; ex[1] = -axr; ex[2] = -xyr; ey[0] = xyr; ey[1] = -ayr; ey[2] = by; break;
        case 2: ex[0] = axr; ex[1] = -bx; ex[2] = -xyr; ey[0] = ayr; ey[1] = xyr; ey[2] = by; break;
        case 3: ex[0] = bx; ex[1] = axr; ex[2] = -xyr; ey[0] = -xyr; ey[1] = ayr; ey[2] = by; break;
        case 4: ex[0] = xyr; ex[1] = bx; ex[2] = -axr; ey[0] = -by; ey[1] = -xyr; ey[2] = -ayr; break;
        default: ex[0] = -xyr; ex[1] = bx; ex[2] = axr; ey[0] = by; ey[1] = -xyr; ey[2] = ayr; break;
    }
    for (int c = 0; c < 3; ++c) {
        ex[c] = ex[c] * sx;
        ey[c] = ey[c] * sy;
    }
}
// the per-axis values of `tangents` for angle x
__host__ __device__ inline void axis_values(double x, double &t, double &sc) {
    const double c = cos(x);
    t = tan(x);
    sc = (1.0 / sqrt(3.0)) / (c * c);
}
// the same vectors with the reference's sequence of operations per point (r^3 as a power, the
// scaling as a division): the grid file's tangent arrays, compared element by element
__device__ inline void tangents_file(int p, double x, double y, double ex[3], double ey[3]) {
    const double a = 1.0 / sqrt(3.0);
    double xe = a * tan(x), ye = a * tan(y);
    double r2 = a * a + xe * xe + ye * ye;
    double invr = 1.0 / pow(sqrt(r2), 3.0);
    double a2 = a * a, ax = a * xe, ay = a * ye, xy = xe * ye;
    double bx = (a2 + ye * ye) * invr, by = (a2 + xe * xe) * invr;
    double axr = ax * invr, ayr = ay * invr, xyr = xy * invr;
    switch (p) {
        case 0: ex[0] = -axr; ex[1] = bx; ex[2] = -xyr; ey[0] = -ayr; ey[1] = -xyr; ey[2] = by; break;
        case 1: ex[0] = -bx; ex[1] = -axr; ex[2] = -xyr; ey[0] = xyr; ey[1] = -ayr; ey[2] = by; break;
        case 2: ex[0] = axr; ex[1] = -bx; ex[2] = -xyr; ey[0] = ayr; ey[1] = xyr; ey[2] = by; break;
        case 3: ex[0] = bx; ex[1] = axr; ex[2] = -xyr; ey[0] = -xyr; ey[1] = ayr; ey[2] = by; break;
        case 4: ex[0] = xyr; ex[1] = bx; ex[2] = -axr; ey[0] = -by; ey[1] = -xyr; ey[2] = -ayr; break;
        default: ex[0] = -xyr; ex[1] = bx; ex[2] = axr; ey[0] = by; ey[1] = -xyr; ey[2] = ayr; break;
    }
    double cx = cos(x), cy = cos(y);
    double c2x = cx * cx, c2y = cy * cy;
    for (int c = 0; c < 3; ++c) {
        ex[c] = a * ex[c] / c2x;
        ey[c] = a * ey[c] / c2y;
    }
}

struct PointOut {
    double *lon, *lat;   // 6 planes
    double *coef[5];     // ex.elon ex.elat ey.elon ey.elat det (det may be null)
    double *metric;      // single plane
};

// One thread per point (panel p, row i, column j) of a family of points over the axes with
// per-axis tables {tan, a / cos^2} (ax[2 i], ax[2 i + 1]; ay likewise): position, lon/lat, the
// tangent vectors' lon/lat components, and (panel 0) the metric.  The unit vectors
// e_lon = (-sin lon, cos lon, 0) and e_lat = (-sin lat cos lon, -sin lat sin lon, cos lat) are
// formed from the position itself (cos lon = X/h, sin lon = Y/h, cos lat = h, sin lat = Z with
// h = hypot(X, Y)), not from sines and cosines of the angles; on the polar axis (h = 0) from the
// angles as atan2 gives them.
__global__ void k_grid_points(Dims d, const double *__restrict__ ax, int nx, const double *__restrict__ ay, int ny,
                              PointOut out) {
    long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    long long total = (long long)NFACE * nx * ny;
    if (tid >= total) return;
    int j = (int)(tid % ny);
    int i = (int)((tid / ny) % nx);
    int p = (int)(tid / ((long long)nx * ny));
    const double tx = ax[2 * i], sx = ax[2 * i + 1], ty = ay[2 * j], sy = ay[2 * j + 1];
    double D = sqrt(1.0 + tx * tx + ty * ty);
    double invD = 1.0 / D;
    double X, Y, Z;
    panel_xyz(p, invD, invD * tx, invD * ty, X, Y, Z);
    const double h = hypot(X, Y);
    double lon = atan2(Y, X);
    double lat = atan2(Z, h);
    long long o = at(d, p, i, j);
    out.lon[o] = lon;
    out.lat[o] = lat;
    double ex[3], ey[3];
    tangents(p, tx, sx, ty, sy, ex, ey);
    double sl, cl, sp, cp;
    if (h > 0.0) {
        const double ih = 1.0 / h;
        sl = Y * ih;
        cl = X * ih;
        sp = Z;
        cp = h;
    } else {
        sl = sin(lon);
        cl = cos(lon);
        sp = sin(lat);
        cp = cos(lat);
    }
    double elon[3] = {-sl, cl, 0.0};
    double elat[3] = {-sp * cl, -sp * sl, cp};
    double exlon = ex[0] * elon[0] + ex[1] * elon[1] + ex[2] * elon[2];
    double exlat = ex[0] * elat[0] + ex[1] * elat[1] + ex[2] * elat[2];
    double eylon = ey[0] * elon[0] + ey[1] * elon[1] + ey[2] * elon[2];
    double eylat = ey[0] * elat[0] + ey[1] * elat[1] + ey[2] * elat[2];
    out.coef[0][o] = exlon;
    out.coef[1][o] = exlat;
    out.coef[2][o] = eylon;
    out.coef[3][o] = eylat;
    if (out.coef[4]) out.coef[4][o] = exlon * eylat - eylon * exlat;
    if (p == 0) {  // metric tensor of panel 0, used for every panel (cs_datastruct.py:407-446)
        double dot = ex[0] * ey[0] + ex[1] * ey[1] + ex[2] * ey[2];
        double nx2 = ex[0] * ex[0] + ex[1] * ex[1] + ex[2] * ex[2];
        double ny2 = ey[0] * ey[0] + ey[1] * ey[1] + ey[2] * ey[2];
        out.metric[at2(d, i, j)] = sqrt(-(dot * dot) + nx2 * ny2);
    }
}

// The arrays of the reference's grid file (plot.py:522-660, read back by cs_datastruct.py:45-195)
// for one family of points over the axes (xs, ys): P[i][j][panel][5] = X, Y, Z, lon, lat of the
// point (the arithmetic of k_grid_points), EX and EY its tangent vectors d/dx and d/dy in the same
// layout (X, Y, Z; their lon, lat entries stay 0, as the reference leaves them).  Any output may
// be null.
__global__ void k_grid_file(const double *__restrict__ xs, int nx, const double *__restrict__ ys, int ny, double *P,
                            double *EX, double *EY) {
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (tid >= (long long)NFACE * nx * ny) return;
    const int p = (int)(tid % NFACE);
    const long long ij = tid / NFACE;
    const double x = xs[ij / ny], y = ys[ij % ny];
    const long long o = tid * 5;
    if (P) {
        const double tx = tan(x), ty = tan(y);
        const double invD = 1.0 / sqrt(1.0 + tx * tx + ty * ty);
        double X, Y, Z;
        panel_xyz(p, invD, invD * tx, invD * ty, X, Y, Z);
        P[o + 0] = X;
        P[o + 1] = Y;
        P[o + 2] = Z;
        P[o + 3] = atan2(Y, X);
        P[o + 4] = atan2(Z, hypot(X, Y));
    }
    if (EX || EY) {
        double ex[3], ey[3];
        tangents_file(p, x, y, ex, ey);
        for (int c = 0; c < 5; ++c) {
            if (EX) EX[o + c] = c < 3 ? ex[c] : 0.0;
            if (EY) EY[o + c] = c < 3 ? ey[c] : 0.0;
        }
    }
}

// sum of g_pc^2 over the interior of all panels (discrete_operators.py:99), fixed order: block b
// of G2_BLOCKS sums cells b*256 + tid, stepping by the grid, into part[b]; then part in block order
constexpr int G2_BLOCKS = 64;
__global__ void k_sum_g2(Dims d, const double *__restrict__ g, double *part) {
    __shared__ double red[256];
    double acc = 0.0;
    const long long cnt = (long long)d.N * d.N;
    for (long long t = blockIdx.x * 256LL + threadIdx.x; t < cnt; t += (long long)gridDim.x * 256) {
        int i = d.i0 + (int)(t / d.N), j = d.i0 + (int)(t % d.N);
        double v = g[at2(d, i, j)];
        acc += v * v;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}
__global__ void k_sum_g2_final(const double *__restrict__ part, int n, double *out) {
    double s = 0.0;
    for (int b = 0; b < n; ++b) s += part[b];
    *out = 6.0 * s;
}

// ---------------------------------------------------------------- Lagrange tables (host)
// lagrange.py:28-163: degree-3 weights at the ghost-cell centres of panel 0's east side,
// in panel 1's angular coordinate, reused for every panel and side.
int lagrange_tables(int N, const std::vector<double> &xc, double dx, std::vector<double> &w, std::vector<int> &kmin) {
    const int n = N + 2 * NG, i0 = NG, iend = NG + N, order = 4, degree = 3;
    std::vector<double> yg(NG * n), ysup(NG * n);
    for (int g = 0; g < NG; ++g) {
        for (int k = 0; k < n; ++k) {
            // ghost centre of panel 0 (x = xc[iend+g], y = xc[k]); panel-1 inverse tan y = Z/Y
            double tx = tan(xc[iend + g]), ty = tan(xc[k]);
            double invD = 1.0 / sqrt(1.0 + tx * tx + ty * ty);
            yg[g * n + k] = atan((invD * ty) / (invD * tx));
            // support centre of panel 1 (x = xc[i0+g], y = xc[k]): Y = invD, Z = invD tan y
            tx = tan(xc[i0 + g]);
            invD = 1.0 / sqrt(1.0 + tx * tx + ty * ty);
            ysup[g * n + k] = atan((invD * ty) / invD);
        }
    }
    w.assign((size_t)NG * n * order, 0.0);
    kmin.assign((size_t)NG * n, 0);
    for (int g = 0; g < NG; ++g) {
        for (int k = 0; k < n; ++k) {
            double K = (yg[g * n + k] - ysup[g * n + 0]) / dx;
            double kmax = K + 2.0;  // ceil(order / 2)
            double kmn = kmax - order + 1;
            if (k >= i0 && k < iend) {
                if (kmax >= iend) {
                    kmax = iend - 1;
                    kmn = kmax - order + 1;
                } else if (kmn < i0) {
                    kmn = i0;
                    kmax = kmn + order - 1;
                }
            } else if (k >= iend) {
                if (kmax >= n) {
                    kmax = n - 1;
                    kmn = kmax - order + 1;
                }
            } else if (kmn < 0) {
                kmn = 0;
                kmax = kmn + order - 1;
            }
            int a = (int)kmn, b = (int)kmax;  // truncation, as ndarray.astype(int)
            if (b - a != degree || a < 0 || b >= n) return CSADV_ERR_ARG;
            if (k >= i0 && k < iend && (a < i0 || b > iend)) return CSADV_ERR_ARG;
            kmin[g * n + k] = a;
            const double x = yg[g * n + k];
            for (int l = 0; l < order; ++l) {
                double L = 1.0;
                for (int m = 0; m < order; ++m)
                    if (m != l) L = L * (x - ysup[g * n + a + m]) / (ysup[g * n + a + l] - ysup[g * n + a + m]);
                w[((size_t)g * n + k) * order + l] = L;
            }
        }
    }
    return CSADV_OK;
}

// Build every FP64 geometry array of resolution N into `mem` (device) and fill `grid`.
// ---------------------------------------------------------------- FP32 ghost-cell stencil tables
__device__ GhostTerm ghost_term(const Dims &d, int q, int i, int j, double w) {
    GhostTerm t;
    t.o = (int)at(d, q, i, j);
    t.o2 = (int)at2(d, i, j);
    const float hi = (float)w;
    t.w = make_float2(hi, (float)(w - (double)hi));
    return t;
}

// the 4 terms of the side-strip ghost cell at depth dep outside side s of panel p, along-edge
// index k, every weight times `scale` (the index rules of side_ghost, halo.cuh)
__device__ void side_terms(const Dims &d, const double *__restrict__ W, const int *__restrict__ K, int p, int s,
                           int dep, int k, double scale, GhostTerm *out) {
    const Conn c = c_conn[p][s];
    const int n = d.n;
    const int k0 = K[dep * n + k];
    const double *w = W + ((long long)dep * n + k) * 4;
    for (int m = 0; m < 4; ++m) {
        const int kk = k0 + m, along = c.rev ? n - 1 - kk : kk;
        int i, j;
        inside_ij(d, c.qs, dep, along, i, j);
        out[m] = ghost_term(d, c.q, i, j, scale * w[m]);
    }
}

// One thread per table row: side rows [p][s][dep][k - i0] (4 terms), then corner rows
// [p][corner][di][dj] (16 terms: for each of the 4 outer points of the E/W interpolation
// (ghost_value, halo.cuh), the neighbour's cell itself or its side-strip stencil, weights
// multiplied in FP64; unused slots have weight 0)
__global__ void k_ghost_tables(Dims d, const double *__restrict__ W, const int *__restrict__ K, GhostTerm *side,
                               GhostTerm *corner) {
    const int N = d.N, n = d.n;
    const long long nside = (long long)NFACE * 4 * NG * N;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < nside) {
        const int kk = (int)(t % N), dep = (int)((t / N) % NG), s = (int)((t / ((long long)N * NG)) % 4);
        const int p = (int)(t / ((long long)N * NG * 4));
        side_terms(d, W, K, p, s, dep, d.i0 + kk, 1.0, side + 4 * t);
        return;
    }
    const long long r = t - nside;
    if (r >= (long long)NFACE * 4 * NG * NG) return;
    const int dj = (int)(r % NG), di = (int)((r / NG) % NG), cc = (int)((r / (NG * NG)) % 4);
    const int p = (int)(r / (NG * NG * 4));
    const int gj = (cc & 1) ? d.iend + dj : d.i0 - 1 - dj;
    const int s = (cc & 2) ? SIDE_E : SIDE_W, dep = di;
    const Conn c = c_conn[p][s];
    const int k0 = K[dep * n + gj];
    const double *w = W + ((long long)dep * n + gj) * 4;
    GhostTerm *out = corner + GHOST_CORNER_TERMS * r;
    for (int m = 0; m < 4; ++m) {
        const int kk = k0 + m, along = c.rev ? n - 1 - kk : kk;
        int qi, qj;
        inside_ij(d, c.qs, dep, along, qi, qj);
        // the cell (qi, qj) of panel c.q: interior, or in a side strip (cell_or_side_ghost, halo.cuh)
        int s2 = -1, dep2 = 0, k2 = 0;
        if (qi >= d.iend) {
            s2 = SIDE_E; dep2 = qi - d.iend; k2 = qj;
        } else if (qi < d.i0) {
            s2 = SIDE_W; dep2 = d.i0 - 1 - qi; k2 = qj;
        } else if (qj >= d.iend) {
            s2 = SIDE_N; dep2 = qj - d.iend; k2 = qi;
        } else if (qj < d.i0) {
            s2 = SIDE_S; dep2 = d.i0 - 1 - qj; k2 = qi;
        }
        if (s2 < 0) {
            out[4 * m] = ghost_term(d, c.q, qi, qj, w[m]);
            for (int e = 1; e < 4; ++e) out[4 * m + e] = ghost_term(d, c.q, qi, qj, 0.0);
        } else {
            side_terms(d, W, K, c.q, s2, dep2, k2, w[m], out + 4 * m);
        }
    }
}

int build_grid(int N, DeviceArena &mem, Grid &grid, cudaStream_t st) {
    Dims d = make_dims(N);
    grid.d = d;
    std::vector<double> xc, xe;
    double dx;
    angular_axes(N, xc, xe, dx);
    grid.dx = dx;
    const long long P1 = d.plane, P6 = d.field;
    double *g_pc = mem.alloc<double>(P1), *g_pu = mem.alloc<double>(P1), *g_pv = mem.alloc<double>(P1);
    double *lon_pc = mem.alloc<double>(P6), *lat_pc = mem.alloc<double>(P6);
    double *lon_pu = mem.alloc<double>(P6), *lat_pu = mem.alloc<double>(P6);
    double *lon_pv = mem.alloc<double>(P6), *lat_pv = mem.alloc<double>(P6);
    double *cu[5], *cv[5], *cc[4];
    for (int c = 0; c < 5; ++c) { cu[c] = mem.alloc<double>(P6); cv[c] = mem.alloc<double>(P6); }
    for (int c = 0; c < 4; ++c) cc[c] = mem.alloc<double>(P6);
    // per-axis {tan, a / cos^2} of the centre and edge angles (the grid points' 1-D factors)
    std::vector<double> axes(2 * (xc.size() + xe.size()));
    for (size_t k = 0; k < xc.size(); ++k) axis_values(xc[k], axes[2 * k], axes[2 * k + 1]);
    for (size_t k = 0; k < xe.size(); ++k)
        axis_values(xe[k], axes[2 * (xc.size() + k)], axes[2 * (xc.size() + k) + 1]);
    double *xs_dev = mem.alloc<double>(axes.size());
    double *a2 = mem.alloc<double>(1 + G2_BLOCKS);  // the sum, then the blocks' partials
    std::vector<double> lw;
    std::vector<int> lk;
    int rc = lagrange_tables(N, xc, dx, lw, lk);
    if (rc != CSADV_OK) return rc;
    double *lag_w = mem.alloc<double>(lw.size());
    int *lag_k = mem.alloc<int>(lk.size());
    const long long nside = (long long)NFACE * 4 * NG * N, ncorner = (long long)NFACE * 4 * NG * NG;
    GhostTerm *gside = mem.alloc<GhostTerm>(4 * nside);
    GhostTerm *gcorner = mem.alloc<GhostTerm>(GHOST_CORNER_TERMS * ncorner);
    if (!mem.ok()) return CSADV_ERR_OOM;
    for (double *g : {g_pc, g_pu, g_pv}) CSADV_CUDA(cudaMemsetAsync(g, 0, P1 * sizeof(double), st));
    CSADV_CUDA(cudaMemcpyAsync(xs_dev, axes.data(), axes.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    CSADV_CUDA(cudaMemcpyAsync(lag_w, lw.data(), lw.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    CSADV_CUDA(cudaMemcpyAsync(lag_k, lk.data(), lk.size() * sizeof(int), cudaMemcpyHostToDevice, st));
    k_ghost_tables<<<ceil_div(nside + ncorner, 128), 128, 0, st>>>(d, lag_w, lag_k, gside, gcorner);
    const double *xcd = xs_dev, *xed = xs_dev + 2 * xc.size();
    const int n = d.n;
    PointOut o;
    o.lon = lon_pc; o.lat = lat_pc; o.metric = g_pc;
    for (int c = 0; c < 4; ++c) o.coef[c] = cc[c];
    o.coef[4] = nullptr;
    long long tot = (long long)NFACE * n * n;
    k_grid_points<<<ceil_div(tot, 128), 128, 0, st>>>(d, xcd, n, xcd, n, o);
    o.lon = lon_pu; o.lat = lat_pu; o.metric = g_pu;
    for (int c = 0; c < 5; ++c) o.coef[c] = cu[c];
    tot = (long long)NFACE * (n + 1) * n;
    k_grid_points<<<ceil_div(tot, 128), 128, 0, st>>>(d, xed, n + 1, xcd, n, o);
    o.lon = lon_pv; o.lat = lat_pv; o.metric = g_pv;
    for (int c = 0; c < 5; ++c) o.coef[c] = cv[c];
    k_grid_points<<<ceil_div(tot, 128), 128, 0, st>>>(d, xcd, n, xed, n + 1, o);
    k_sum_g2<<<G2_BLOCKS, 256, 0, st>>>(d, g_pc, a2 + 1);
    k_sum_g2_final<<<1, 1, 0, st>>>(a2 + 1, G2_BLOCKS, a2);
    CSADV_CUDA(cudaGetLastError());
    double a2h = 0.0;
    CSADV_CUDA(cudaMemcpyAsync(&a2h, a2, sizeof(double), cudaMemcpyDeviceToHost, st));
    CSADV_CUDA(cudaStreamSynchronize(st));
    grid.g_pc = g_pc; grid.g_pu = g_pu; grid.g_pv = g_pv;
    grid.lon_pc = lon_pc; grid.lat_pc = lat_pc;
    grid.lon_pu = lon_pu; grid.lat_pu = lat_pu;
    grid.lon_pv = lon_pv; grid.lat_pv = lat_pv;
    for (int c = 0; c < 5; ++c) { grid.cu[c] = cu[c]; grid.cv[c] = cv[c]; }
    for (int c = 0; c < 4; ++c) grid.cc[c] = cc[c];
    grid.lag_w = lag_w;
    grid.lag_k = lag_k;
    grid.gside = gside;
    grid.gcorner = gcorner;
    grid.a2 = a2h;
    return CSADV_OK;
}

}  // namespace csadv

using namespace csadv;

extern "C" int csadv_grid_points(int N, int kind, double *P, double *EX, double *EY, void *stream) {
    if (N < 1 || kind < 0 || kind > 3 || (!P && !EX && !EY)) return CSADV_ERR_ARG;
    std::vector<double> xc, xe;
    double dx;
    angular_axes(N, xc, xe, dx);
    // po: (x edges, y edges), pc: (centres, centres), pu: (x edges, centres), pv: (centres, y edges)
    const std::vector<double> &xs = kind == 0 || kind == 2 ? xe : xc;
    const std::vector<double> &ys = kind == 0 || kind == 3 ? xe : xc;
    const int nx = (int)xs.size(), ny = (int)ys.size();
    const size_t bytes = (size_t)nx * ny * NFACE * 5 * sizeof(double);
    cudaStream_t st = (cudaStream_t)stream;
    DevArray ax, ay, op, oex, oey;
    int rc = dev_in(xs.data(), nx * sizeof(double), st, ax);
    if (!rc) rc = dev_in(ys.data(), ny * sizeof(double), st, ay);
    if (!rc && P) rc = dev_out(P, bytes, st, op);
    if (!rc && EX) rc = dev_out(EX, bytes, st, oex);
    if (!rc && EY) rc = dev_out(EY, bytes, st, oey);
    if (!rc) {
        const long long tot = (long long)NFACE * nx * ny;
        k_grid_file<<<ceil_div(tot, 128), 128, 0, st>>>((const double *)ax.dev, nx, (const double *)ay.dev, ny,
                                                         (double *)op.dev, (double *)oex.dev, (double *)oey.dev);
        if (cudaGetLastError() != cudaSuccess) rc = CSADV_ERR_CUDA;
    }
    if (!rc && P) rc = dev_back(P, bytes, st, op);
    if (!rc && EX) rc = dev_back(EX, bytes, st, oex);
    if (!rc && EY) rc = dev_back(EY, bytes, st, oey);
    for (DevArray *a : {&ax, &ay, &op, &oex, &oey}) dev_free(*a, st);
    if (cudaStreamSynchronize(st) != cudaSuccess && !rc) rc = CSADV_ERR_CUDA;
    return rc;
}
