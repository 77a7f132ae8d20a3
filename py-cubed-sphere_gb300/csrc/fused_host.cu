// Host side of the fused engine: buffers, wind preparation, step sequencing, and the
// lazy MF-PR correction.
#include <vector>

#include "halo.cuh"
#include "internal.h"
#include "tiles.h"

namespace csadv {

constexpr int ANCHOR_BLOCKS = 512;  // blocks of k_anchor_mass

int fused_supported(const Options &o) { return o.et == ET_DG && o.mf != MF_AF; }

__global__ void k_plane_to_float(const double *__restrict__ src, float *dst, long long n) {
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < n) dst[t] = (float)src[t];
}

// dst(j, i) = src(i, j) (transpose) or dst(i, j) = 1 / src(i, j) (recip), or both, for i < rows,
// j < cols of one plane; entries outside are set to zero
template <class real>
__global__ void k_plane_xform(const real *__restrict__ src, real *dst, Dims d, int rows, int cols, int transpose,
                              int recip) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= d.plane) return;
    const int a = (int)(t / d.pitch), b = (int)(t % d.pitch);  // destination row, column
    const int i = transpose ? b : a, j = transpose ? a : b;      // source row, column
    real v = real(0);
    if (i < rows && j < cols) {
        v = src[(long long)i * d.pitch + j];
        if (recip) v = real(1) / v;
    }
    dst[t] = v;
}

// cell records {g, 1/g} of the n x n centres, natural (dst(i, j)) or transposed (dst(j, i));
// zero outside.  dtdx != 0: {g, dtdx (1/g)}, the factor of the update (FP64 with AVLT splitting:
// the kernel's per-cell product dt/dx * (1/g), made once per plan with the same two roundings)
template <class real>
__global__ void k_cell_records(const real *__restrict__ g, typename Vec2<real>::type *dst, Dims d, int n,
                               int transpose, real dtdx) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= d.plane) return;
    const int a = (int)(t / d.pitch), b = (int)(t % d.pitch);
    const int i = transpose ? b : a, j = transpose ? a : b;
    typename Vec2<real>::type v;
    v.x = real(0);
    v.y = real(0);
    if (i < n && j < n) {
        v.x = g[(long long)i * d.pitch + j];
        v.y = real(1) / v.x;
        if (dtdx != real(0)) v.y = dtdx * v.y;
    }
    dst[t] = v;
}

// Q* + g corr on interior cells of every tracer (the true state); blockIdx.y = tracer
template <class real>
__global__ void k_materialize(real *Q0, Dims d, const real *__restrict__ g, const double *__restrict__ corr) {
    const int N = d.N;
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)NFACE * N * N) return;
    int j = d.i0 + (int)(t % N), i = d.i0 + (int)((t / N) % N), p = (int)(t / ((long long)N * N));
    real *Q = Q0 + blockIdx.y * d.field;
    long long o = at(d, p, i, j);
    Q[o] = corrected(Q[o], g[at2(d, i, j)], (real)corr[blockIdx.y]);
}

// copy every non-interior cell of the n x n cell planes from `src` to `dst` (all tracers)
template <class real>
__global__ void k_copy_ghosts(const real *__restrict__ src, real *dst, Dims d) {
    const int n = d.n;
    long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= (long long)NFACE * n * n) return;
    int j = (int)(t % n), i = (int)((t / n) % n), p = (int)(t / ((long long)n * n));
    if (i >= d.i0 && i < d.iend && j >= d.i0 && j < d.iend) return;
    long long o = at(d, p, i, j) + blockIdx.y * d.field;
    dst[o] = src[o];
}

int fused_ghosts_to_current(const Options &o, const Grid &g, int T, FusedState &f, int cur, cudaStream_t st,
                            int first) {
    const Dims d = g.d;
    const size_t ofs = (size_t)first * d.field * (o.precision == 64 ? sizeof(double) : sizeof(float));
    void *src = (char *)f.Qbuf[1 - cur] + ofs, *dst = (char *)f.Qbuf[cur] + ofs;
    if (f.sweep && f.inline_ghosts) {  // the step kernel kept its ghost cells on chip: fill the input's
        const bool pr = o.mf == MF_PR;
        const double *corr = pr ? f.corr[1 - cur] + first : nullptr;
        int rc = o.precision == 64
                     ? launch_halo_dg_tracers<double>((double *)src, T, g, corr, (const double *)f.g_pc, st)
                     : launch_halo_dg_tracers<float>((float *)src, T, g, corr, (const float *)f.g_pc, st);
        if (rc) return rc;
    }
    dim3 grid(ceil_div((long long)NFACE * d.n * d.n, 256), T);
    if (o.precision == 64)
        k_copy_ghosts<double><<<grid, 256, 0, st>>>((const double *)src, (double *)dst, d);
    else
        k_copy_ghosts<float><<<grid, 256, 0, st>>>((const float *)src, (float *)dst, d);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

int fused_alloc(const Options &o, const Grid &g, int T, DeviceArena &mem, FusedState &f, cudaStream_t st) {
    const Dims d = g.d;
    const size_t es = o.precision == 64 ? sizeof(double) : sizeof(float);
    f.on = true;
    // the step kernel evaluates the ET-DG ghost cells of its tiles itself (no ghost-cell launch)
    f.inline_ghosts = true;
    f.Qbuf[1] = mem.alloc<char>((long long)T * d.field * es);
    for (int b = 0; b < 2; ++b) f.corr[b] = mem.alloc<double>(T);
    int maxb = 0;
    for (int c = 0; c < FUSED_NTILE_CFG; ++c) maxb = maxb > fused_blocks(d, c) ? maxb : fused_blocks(d, c);
    for (int c = 0; c < SWEEP_NTILE_CFG; ++c) {
        SweepSolve tmp{};
        tmp.d = d;
        sweep_config(tmp, c);
        maxb = maxb > NFACE * tmp.ntiles ? maxb : NFACE * tmp.ntiles;
    }
    f.partials = mem.alloc<double>((long long)T * maxb);
    f.counter = mem.alloc<unsigned int>(1);
    f.ua = mem.alloc<char>(d.field * es);
    f.va = mem.alloc<char>(d.field * es);
    f.wpitch = d.pitch / 32;
    long long words = (long long)NFACE * (d.n + 1) * f.wpitch;
    f.upos = mem.alloc<uint32_t>(words);
    f.vpos = mem.alloc<uint32_t>(words);
    if (o.precision == 64) {
        f.g_pc = g.g_pc;
        f.g_pu = g.g_pu;
        f.g_pv = g.g_pv;
    } else {
        float *gs[3];
        for (int c = 0; c < 3; ++c) gs[c] = mem.alloc<float>(d.plane);
        if (!mem.ok()) return CSADV_ERR_OOM;
        const double *src[3] = {g.g_pc, g.g_pu, g.g_pv};
        for (int c = 0; c < 3; ++c) k_plane_to_float<<<ceil_div(d.plane, 256), 256, 0, st>>>(src[c], gs[c], d.plane);
        f.g_pc = gs[0];
        f.g_pu = gs[1];
        f.g_pv = gs[2];
    }
    if (!mem.ok()) return CSADV_ERR_OOM;
    // line-marching kernel data: edge records (filled by the wind preparation), cell records
    // {g, 1/g} natural and transposed, the y-edge metric transposed (for the y-edge records)
    // edge records {u, +-g}; FP64: with the flux coefficients in two more vec2 planes behind them
    // (record_coef_offset)
    const size_t rec_bytes = (o.precision == 64 ? 6 : 2) * (size_t)d.field * es;
    f.erx = mem.alloc<char>(rec_bytes);
    f.ery = mem.alloc<char>(rec_bytes);
    f.crx = mem.alloc<char>(2 * d.plane * es);
    f.cry = mem.alloc<char>(2 * d.plane * es);
    void *gpvT = mem.alloc<char>(d.plane * es);
    f.dsolve = mem.alloc<SweepSolve>(2);
    f.dsolve_tr = mem.alloc<SweepSolve>(2 * T);
    if (o.precision == 32 && o.mf == MF_PR) {
        f.mass_target = mem.alloc<double>(T);
        const long long io_blocks = ceil_div((long long)d.n * d.n, IO_B);  // the full layout's upload
        f.anchor_part = mem.alloc<double>(io_blocks > ANCHOR_BLOCKS ? io_blocks : ANCHOR_BLOCKS);
        f.anchor_count = mem.alloc<unsigned int>(1);
    }
    if (!mem.ok()) return CSADV_ERR_OOM;
    {
        const int nb = ceil_div(d.plane, 256);
        const int n = d.n;
        if (o.precision == 64) {
            const double *gpc = (const double *)f.g_pc, *gpv = (const double *)f.g_pv;
            k_cell_records<double><<<nb, 256, 0, st>>>(gpc, (double2 *)f.crx, d, n, 0, 0.0);
            k_cell_records<double><<<nb, 256, 0, st>>>(gpc, (double2 *)f.cry, d, n, 1, 0.0);
            k_plane_xform<double><<<nb, 256, 0, st>>>(gpv, (double *)gpvT, d, n, n + 1, 1, 0);
        } else {
            const float *gpc = (const float *)f.g_pc, *gpv = (const float *)f.g_pv;
            k_cell_records<float><<<nb, 256, 0, st>>>(gpc, (float2 *)f.crx, d, n, 0, 0.f);
            k_cell_records<float><<<nb, 256, 0, st>>>(gpc, (float2 *)f.cry, d, n, 1, 0.f);
            k_plane_xform<float><<<nb, 256, 0, st>>>(gpv, (float *)gpvT, d, n, n + 1, 1, 0);
        }
        CSADV_CUDA(cudaGetLastError());
    }
    f.gpvT = gpvT;
    CSADV_CUDA(cudaMemsetAsync(f.erx, 0, rec_bytes, st));
    CSADV_CUDA(cudaMemsetAsync(f.ery, 0, rec_bytes, st));
    if (f.mass_target) CSADV_CUDA(cudaMemsetAsync(f.mass_target, 0, T * sizeof(double), st));
    if (f.anchor_count) CSADV_CUDA(cudaMemsetAsync(f.anchor_count, 0, sizeof(unsigned int), st));
    CSADV_CUDA(cudaMemsetAsync(f.Qbuf[1], 0, (size_t)T * d.field * es, st));
    for (int b = 0; b < 2; ++b) CSADV_CUDA(cudaMemsetAsync(f.corr[b], 0, T * sizeof(double), st));
    CSADV_CUDA(cudaMemsetAsync(f.counter, 0, sizeof(unsigned int), st));
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

int fused_wind_pipeline(const Options &o, const Grid &g, const Winds &w, DeviceArena &mem, FusedState &f,
                        cudaStream_t st) {
    if (!w.nbasis) return CSADV_OK;
    // the same layout as the first buffer (FP64: the flux coefficients behind the records)
    const size_t bytes = o.precision == 64 ? 6 * (size_t)g.d.field * sizeof(double) : 2 * (size_t)g.d.field * sizeof(float);
    f.erx1 = mem.alloc<char>(bytes);
    f.ery1 = mem.alloc<char>(bytes);
    if (!mem.ok()) return CSADV_ERR_OOM;
    CSADV_CUDA(cudaMemsetAsync(f.erx1, 0, bytes, st));
    CSADV_CUDA(cudaMemsetAsync(f.ery1, 0, bytes, st));
    f.wpipe = true;
    return CSADV_OK;
}

int fused_prep_winds(const Options &o, const Grid &g, const Winds &w, double dt, FusedState &f, int buf,
                     cudaStream_t st, int part, int peek) {
    if (f.sweep && w.nbasis) {  // the records of the x-edges (part 0), the y-edges (1) or both (-1)
        if (o.precision == 64)
            return wind_step<double>(o, g, w, dt, (const double *)f.g_pu, (const double *)f.gpvT,
                                     (double2 *)f.rec_x(buf), (double2 *)f.rec_y(buf), f.crx, f.cry, st, part, peek);
        return wind_step<float>(o, g, w, dt, (const float *)f.g_pu, (const float *)f.gpvT, (float2 *)f.rec_x(buf),
                                (float2 *)f.rec_y(buf), nullptr, nullptr, st, part, peek);
    }
    if (peek) return CSADV_ERR_UNSUPPORTED;  // the other preparations run after the clock's tick
    if (part == 1) return CSADV_OK;          // and whole (part -1 or 0)
    if (w.nbasis) {  // per-edge tile kernel on a basis wind: current and previous winds first
        int rc = wind_sync(o, g, w, st);
        if (rc) return rc;
    }
    if (f.sweep) {
        if (o.precision == 64)
            return wind_avgprep_t<double>(o, g, w, dt, (const double *)f.g_pu, (const double *)f.gpvT,
                                          (double2 *)f.erx, (double2 *)f.ery, f.crx, f.cry, st);
        return wind_avgprep_t<float>(o, g, w, dt, (const float *)f.g_pu, (const float *)f.gpvT, (float2 *)f.erx,
                                     (float2 *)f.ery, nullptr, nullptr, st);
    }
    if (o.precision == 64)
        return wind_avgprep<double>(o, g, w, dt, (double *)f.ua, (double *)f.va, f.upos, f.vpos, f.wpitch, st);
    return wind_avgprep<float>(o, g, w, dt, (float *)f.ua, (float *)f.va, f.upos, f.vpos, f.wpitch, st);
}

int fused_prepare(const Options &o, int tile) {
    if (tile >= FUSED_NTILE_CFG)
        return o.precision == 64 ? sweep_launch<double>(o.recon, o.opsplit, nullptr, nullptr, 0, 0, 0, (cudaStream_t)-1, 0)
                                 : sweep_launch<float>(o.recon, o.opsplit, nullptr, nullptr, 0, 0, 0, (cudaStream_t)-1, 0);
    FusedArgs a{};
    return o.precision == 64 ? fused_launch<double>(a, o.recon, tile, (cudaStream_t)-1)
                             : fused_launch<float>(a, o.recon, tile, (cudaStream_t)-1);
}

int fused_set_tile(const Options &o, const Grid &g, int T, double dt, FusedState &f, int tile, cudaStream_t st) {
    int rc = fused_prepare(o, tile);
    if (rc) return rc;
    const bool was = f.sweep;
    f.tile = tile;
    f.sweep = tile >= FUSED_NTILE_CFG;
    if (!f.sweep) return CSADV_OK;
    f.scfg = tile - FUSED_NTILE_CFG;
    const bool pr = o.mf == MF_PR;
    SweepSolve h[2];
    for (int b = 0; b < 2; ++b) {
        SweepSolve &s = h[b];
        s = SweepSolve{};
        s.d = g.d;
        s.T = T;
        sweep_config(s, f.scfg);
        s.dt = dt;
        s.dx = g.dx;
        s.dtdx = (float)(dt / g.dx);
        s.irdx = (float)(1.0 / g.dx);
        s.a2 = g.a2;
        s.Qin = f.Qbuf[b];
        s.Qout = f.Qbuf[1 - b];
        s.corr_in = pr ? f.corr[b] : nullptr;
        s.corr_out = pr ? f.corr[1 - b] : nullptr;
        s.partials = f.partials;
        s.counter = f.counter;
        s.erx = f.rec_x(b);
        s.ery = f.rec_y(b);
        s.ecofs = o.precision == 64 ? record_coef_offset<double>(g.d) : 0;
        s.crx = f.crx;
        s.cry = f.cry;
        s.gpc = f.g_pc;
        s.split = o.opsplit;
        s.mt = o.mt;
        s.mfpr = pr ? 1 : 0;
        s.mass_target = f.mass_target;
        s.lag_w = f.inline_ghosts ? g.lag_w : nullptr;
        s.lag_k = f.inline_ghosts ? g.lag_k : nullptr;
        s.hlag_w = g.lag_w;
        s.hlag_k = g.lag_k;
        s.gside = g.gside;
        s.gcorner = g.gcorner;
    }
    if (o.precision == 64 && o.opsplit == SP_AVLT) {
        // the FP64 AVLT kernel reads dt/dx (1/g) from the cell records (once, for the final dt)
        const double dtdx = dt / g.dx;
        if (f.crec_dtdx != dtdx) {
            const int nb = ceil_div(g.d.plane, 256);
            k_cell_records<double><<<nb, 256, 0, st>>>((const double *)f.g_pc, (double2 *)f.crx, g.d, g.d.n, 0, dtdx);
            k_cell_records<double><<<nb, 256, 0, st>>>((const double *)f.g_pc, (double2 *)f.cry, g.d, g.d.n, 1, dtdx);
            CSADV_CUDA(cudaGetLastError());
            f.crec_dtdx = dtdx;
        }
    }
    f.nitems = NFACE * h[0].ntiles;
    f.smem = o.precision == 64 ? sweep_smem_bytes<double>(f.scfg) : sweep_smem_bytes<float>(f.scfg);
    // one descriptor per buffer parity and tracer: the tracer's fields, pending corrections,
    // partial sums and mass target (the arrival counter is shared: the launches are ordered)
    std::vector<SweepSolve> ht(2 * (size_t)T);
    const size_t fb = (size_t)g.d.field * (o.precision == 64 ? sizeof(double) : sizeof(float));
    for (int b = 0; b < 2; ++b)
        for (int t = 0; t < T; ++t) {
            SweepSolve s = h[b];
            s.T = 1;
            s.Qin = (const char *)h[b].Qin + t * fb;
            s.Qout = (char *)h[b].Qout + t * fb;
            if (s.corr_in) s.corr_in += t;
            if (s.corr_out) s.corr_out += t;
            s.partials += (long long)t * f.nitems;
            if (s.mass_target) s.mass_target += t;
            ht[(size_t)b * T + t] = s;
        }
    CSADV_CUDA(cudaMemcpyAsync(f.dsolve, h, sizeof(h), cudaMemcpyHostToDevice, st));
    CSADV_CUDA(cudaMemcpyAsync(f.dsolve_tr, ht.data(), ht.size() * sizeof(SweepSolve), cudaMemcpyHostToDevice, st));
    CSADV_CUDA(cudaStreamSynchronize(st));
    (void)was;
    return CSADV_OK;
}

int fused_ghosts(const Options &o, const Grid &g, int T, FusedState &f, int cur, cudaStream_t st) {
    if (f.sweep && f.inline_ghosts) return CSADV_OK;  // the step kernel evaluates them itself
    const bool pr = o.mf == MF_PR;
    if (o.precision == 64)
        return launch_halo_dg_tracers<double>((double *)f.Qbuf[cur], T, g, pr ? f.corr[cur] : nullptr,
                                              (const double *)f.g_pc, st);
    return launch_halo_dg_tracers<float>((float *)f.Qbuf[cur], T, g, pr ? f.corr[cur] : nullptr,
                                         (const float *)f.g_pc, st);
}

int fused_kernel(const Options &o, const Grid &g, double dt, int T, FusedState &f, int &cur, cudaStream_t st,
                 cudaEvent_t ev0, cudaEvent_t ev1) {
    const bool pr = o.mf == MF_PR;
    if (f.sweep) {
        if (ev0) CSADV_CUDA(cudaEventRecord(ev0, st));
        int rc = o.precision == 64
                     ? sweep_launch<double>(o.recon, o.opsplit, f.dsolve + cur, nullptr, f.nitems, f.nitems, f.smem, st, 0)
                     : sweep_launch<float>(o.recon, o.opsplit, f.dsolve + cur, nullptr, f.nitems, f.nitems, f.smem, st,
                                           sweep_tgroup(T));
        if (rc) return rc;
        if (ev1) CSADV_CUDA(cudaEventRecord(ev1, st));
        cur = 1 - cur;
        return CSADV_OK;
    }
    FusedArgs a{};
    a.d = g.d;
    a.T = T;
    a.dt = dt;
    a.dx = g.dx;
    a.a2 = g.a2;
    a.Qin = f.Qbuf[cur];
    a.Qout = f.Qbuf[1 - cur];
    a.corr_in = pr ? f.corr[cur] : nullptr;
    a.corr_out = pr ? f.corr[1 - cur] : nullptr;
    a.partials = f.partials;
    a.counter = f.counter;
    a.ua = f.ua;
    a.va = f.va;
    a.upos = f.upos;
    a.vpos = f.vpos;
    a.g_pc = f.g_pc;
    a.g_pu = f.g_pu;
    a.g_pv = f.g_pv;
    a.split = o.opsplit;
    a.mt = o.mt;
    a.mfpr = pr ? 1 : 0;
    a.wpitch = f.wpitch;
    if (ev0) CSADV_CUDA(cudaEventRecord(ev0, st));
    int rc = o.precision == 64 ? fused_launch<double>(a, o.recon, f.tile, st)
                               : fused_launch<float>(a, o.recon, f.tile, st);
    if (rc) return rc;
    if (ev1) CSADV_CUDA(cudaEventRecord(ev1, st));
    cur = 1 - cur;
    return CSADV_OK;
}

int fused_kernel_tracer(const Options &o, int T, const FusedState &f, int cur, int t, cudaStream_t st) {
    if (!f.sweep || t < 0 || t >= T) return CSADV_ERR_UNSUPPORTED;
    const SweepSolve *s = f.dsolve_tr + (size_t)cur * T + t;
    return o.precision == 64 ? sweep_launch<double>(o.recon, o.opsplit, s, nullptr, f.nitems, f.nitems, f.smem, st, 0)
                             : sweep_launch<float>(o.recon, o.opsplit, s, nullptr, f.nitems, f.nitems, f.smem, st,
                                                   SWEEP_TG_ONE);
}

// sum over the interior of Q g (metric in the state's precision): per-block partials over a
// grid-stride range, then one block sums them in a fixed order -> *out
template <class real>
__global__ void k_anchor_mass(const real *__restrict__ Q, const real *__restrict__ g, Dims d, double *part) {
    __shared__ double red[256];
    const int N = d.N;
    double acc = 0.0;
    for (long long t = blockIdx.x * 256LL + threadIdx.x; t < (long long)NFACE * N * N; t += (long long)gridDim.x * 256) {
        const int j = d.i0 + (int)(t % N), i = d.i0 + (int)((t / N) % N), p = (int)(t / ((long long)N * N));
        acc += (double)Q[at(d, p, i, j)] * (double)g[at2(d, i, j)];
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void k_anchor_sum(const double *__restrict__ part, int np, double *out) {
    __shared__ double red[256];
    double acc = 0.0;
    for (int b = threadIdx.x; b < np; b += 256) acc += part[b];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

int fused_anchor_mass(const Options &o, const Grid &g, FusedState &f, int cur, int t, cudaStream_t st) {
    if (!f.mass_target || o.precision != 32) return CSADV_OK;
    const float *Q = (const float *)f.Qbuf[cur] + (size_t)t * g.d.field;
    const int nb = ceil_div((long long)NFACE * g.d.N * g.d.N, 256) < ANCHOR_BLOCKS
                       ? ceil_div((long long)NFACE * g.d.N * g.d.N, 256)
                       : ANCHOR_BLOCKS;
    k_anchor_mass<float><<<nb, 256, 0, st>>>(Q, (const float *)f.g_pc, g.d, f.anchor_part);
    k_anchor_sum<<<1, 256, 0, st>>>(f.anchor_part, nb, f.mass_target + t);
    CSADV_CUDA(cudaGetLastError());
    return CSADV_OK;
}

int fused_materialize(const Options &o, const Grid &g, int T, FusedState &f, int cur, cudaStream_t st) {
    if (o.mf != MF_PR) return CSADV_OK;
    const Dims d = g.d;
    dim3 grid(ceil_div((long long)NFACE * d.N * d.N, 256), T);
    if (o.precision == 64)
        k_materialize<double><<<grid, 256, 0, st>>>((double *)f.Qbuf[cur], d, (const double *)f.g_pc, f.corr[cur]);
    else
        k_materialize<float><<<grid, 256, 0, st>>>((float *)f.Qbuf[cur], d, (const float *)f.g_pc, f.corr[cur]);
    CSADV_CUDA(cudaGetLastError());
    CSADV_CUDA(cudaMemsetAsync(f.corr[cur], 0, T * sizeof(double), st));
    f.settled = true;
    return CSADV_OK;
}

}  // namespace csadv
