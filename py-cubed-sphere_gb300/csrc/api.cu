// C ABI of csadv (declared in include/csadv.h): plan lifecycle and step orchestration.
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <chrono>
#include <mutex>
#include <new>
#include <vector>

#include "../../include/csadv.h"
#include "cases.cuh"
#include "common.cuh"
#include "internal.h"

namespace csadv {

static thread_local int g_device = -1;

int cuda_fail(cudaError_t e, const char *what, const char *file, int line) {
    if (getenv("CSADV_DEBUG")) fprintf(stderr, "csadv: %s failed: %s (%s:%d)\n", what, cudaGetErrorString(e), file, line);
    (void)cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? CSADV_ERR_OOM : CSADV_ERR_CUDA;
}

int validate_options(const csadv_options *o, Options &out) {
    if (!o) return CSADV_ERR_ARG;
    if (o->recon < 1 || o->recon > 4 || o->dp < 1 || o->dp > 2 || o->opsplit < 1 || o->opsplit > 3 || o->et < 1 ||
        o->et > 3 || o->mt < 1 || o->mt > 2 || o->mf < 1 || o->mf > 3)
        return CSADV_ERR_OPTION;
    if (!((o->vf >= 1 && o->vf <= 4) || o->vf == CSADV_WIND_SOLID || o->vf == CSADV_WIND_DEFORM ||
          o->vf == CSADV_WIND_SOLID_DIV))
        return CSADV_ERR_OPTION;
    if (o->precision != 64 && o->precision != 32) return CSADV_ERR_OPTION;
    if (o->engine < CSADV_ENGINE_AUTO || o->engine > CSADV_ENGINE_FUSED) return CSADV_ERR_OPTION;
    if (o->tile < 0 || o->tile > 8) return CSADV_ERR_OPTION;
    // discrete_operators.py:49-73: SP-AVLT / SP-L04 need MT-0, SP-PL07 needs MT-PL07
    if ((o->opsplit == SP_PL07) != (o->mt == MT_PL07)) return CSADV_ERR_OPTION_PAIR;
    out.recon = o->recon;
    out.dp = o->dp;
    out.opsplit = o->opsplit;
    out.et = o->et;
    out.mt = o->mt;
    out.mf = o->mf;
    out.vf = o->vf;
    out.precision = o->precision;
    out.engine = o->engine;
    out.tile = o->tile;
    for (int c = 0; c < 4; ++c) out.wp[c] = o->wind_param[c];
    return CSADV_OK;
}

bool wind_time_dependent(const Options &o) { return wind_is_time_dependent(o.vf); }

}  // namespace csadv

using namespace csadv;

#include "plan.h"

namespace {

cudaStream_t S(void *stream) { return (cudaStream_t)stream; }

// default tile configuration of the fused engine (zero-based csadv_options.tile code):
// the line-marching kernel, large tiles for large panels
int default_tile(const Options &o, int N, int T) {
    const int t = tuned_tile(N, T, o);
    if (t >= 0) return t;
    return N >= 116 ? 4 : 7;
}

std::mutex g_pool_mu;
cudaMemPool_t g_pools[64] = {};

// grids shared by the plans of one resolution and device
std::mutex g_grid_mu;
std::map<std::pair<int, int>, std::weak_ptr<GridHolder>> g_grids;

}  // namespace

cudaMemPool_t csadv::device_pool() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lock(g_pool_mu);
    if (!g_pools[dev]) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool = nullptr;
        if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
            (void)cudaGetLastError();
            return nullptr;
        }
        unsigned long long keep = ~0ULL;  // freed memory stays in the pool for the next plans
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        g_pools[dev] = pool;
    }
    return g_pools[dev];
}

namespace {

// The grid of resolution N on this device, built by the first plan that asks for it.  The map's
// lock is held only to find or insert the holder: the build itself (host tables, uploads, a wait
// for the stream) runs under the holder's own lock, so plans of other sizes are made and
// released meanwhile.
int acquire_grid(int N, int device, cudaStream_t st, std::shared_ptr<GridHolder> &out) {
    const auto key = std::make_pair(device, N);
    std::shared_ptr<GridHolder> h;
    {
        std::lock_guard<std::mutex> lock(g_grid_mu);
        auto it = g_grids.find(key);
        if (it != g_grids.end()) h = it->second.lock();
        if (!h) {
            h = std::make_shared<GridHolder>();
            g_grids[key] = h;
        }
    }
    std::lock_guard<std::mutex> build(h->build_mu);
    if (!h->built) {
        cudaMemPool_t pool = device_pool();
        int rc = pool ? CSADV_OK : CSADV_ERR_CUDA;
        if (!rc) {
            h->mem.use_pool(pool, st);
            rc = build_grid(N, h->mem, h->grid, st);
        }
        // plans on other streams use it next
        if (cudaStreamSynchronize(st) != cudaSuccess && !rc) rc = CSADV_ERR_CUDA;
        (void)cudaGetLastError();
        if (rc) {
            h->mem.release();
            std::lock_guard<std::mutex> lock(g_grid_mu);
            auto it = g_grids.find(key);
            if (it != g_grids.end() && it->second.lock() == h) g_grids.erase(it);  // the next plan retries
            return rc;
        }
        h->built = true;
    }
    out = h;
    return CSADV_OK;
}

// Drops the plan's reference to its grid.  The last plan to leave frees the grid in the order of
// stream st, after the work that the plans released before it had queued.
void release_grid(csadv_plan *pl, cudaStream_t st) {
    std::lock_guard<std::mutex> lock(g_grid_mu);
    std::shared_ptr<GridHolder> &h = pl->gref;
    if (!h) return;
    if (h.use_count() > 1) {
        auto &left = h->left;
        for (size_t i = 0; i < left.size();) {  // forget the marks whose work has ended
            if (cudaEventQuery(left[i]) == cudaSuccess) {
                cudaEventDestroy(left[i]);
                left[i] = left.back();
                left.pop_back();
            } else {
                ++i;
            }
        }
        (void)cudaGetLastError();
        cudaEvent_t e = nullptr;
        if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess) {
            if (cudaEventRecord(e, st) == cudaSuccess) left.push_back(e);
            else cudaEventDestroy(e);
        }
    } else {
        for (cudaEvent_t e : h->left) {
            cudaStreamWaitEvent(st, e, 0);
            cudaEventDestroy(e);
        }
        h->left.clear();
        h->mem.release_on(st);
    }
    (void)cudaGetLastError();
    h.reset();
}

// the staged engine's per-tracer scratch, allocated on first use
int ensure_scratch(csadv_plan *pl, cudaStream_t st) {
    if (pl->s.Qx) return CSADV_OK;
    pl->mem.set_stream(st);
    const long long F = pl->grid.d.field;
    const size_t es = pl->esize();
    void **sa[] = {&pl->s.Qx, &pl->s.Qy, &pl->s.qLx, &pl->s.qRx, &pl->s.qLy, &pl->s.qRy, &pl->s.fx, &pl->s.fy, &pl->s.div};
    for (void **p : sa) *p = pl->mem.alloc<char>(F * es);
    if (!pl->mem.ok()) return CSADV_ERR_OOM;
    for (void **p : sa) CSADV_CUDA(cudaMemsetAsync(*p, 0, F * es, st));
    return CSADV_OK;
}

template <class real>
int scalar_halo(csadv_plan *pl, real *Q, cudaStream_t st) {
    if (pl->opt.et == ET_DG) return launch_halo_dg<real>(Q, pl->grid, st);
    return launch_halo_adjacent<real>(Q, Q, pl->grid, st);
}

template <class real>
int time_step(csadv_plan *pl, cudaStream_t st, bool update, int only_tracer) {
    int rc = ensure_scratch(pl, st);
    if (rc) return rc;
    for (int t = 0; t < pl->T; ++t) {
        if (only_tracer >= 0 && t != only_tracer) continue;
        rc = scalar_halo<real>(pl, (real *)pl->tracer(t), st);
        if (rc) return rc;
    }
    if (wind_time_dependent(pl->opt)) {
        rc = wind_halo(pl->opt, pl->grid, pl->w, st);
        if (rc) return rc;
        rc = wind_average(pl->opt, pl->grid, pl->w, pl->dt, st);
        if (rc) return rc;
    }
    for (int t = 0; t < pl->T; ++t) {
        if (only_tracer >= 0 && t != only_tracer) continue;
        real *Q = (real *)pl->tracer(t);
        rc = staged_divergence<real>(pl->opt, pl->grid, pl->w, pl->dt, Q, pl->s, pl->partials, pl->npart, st);
        if (rc) return rc;
        rc = staged_update<real>(pl->opt, pl->grid, pl->dt, update ? Q : nullptr, pl->s, pl->partials, pl->npart,
                                 pl->scal, st);
        if (rc) return rc;
    }
    return CSADV_OK;
}

int do_update_winds(csadv_plan *pl, bool tick, long long k, double t, cudaStream_t st);

int ensure_side(csadv_plan *pl) {
    if (!pl->side) {
        // lowest priority: with pipelined winds the step kernel's CTAs go first, the next step's
        // wind records fill the SMs it leaves free
        int least = 0, greatest = 0;
        CSADV_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        CSADV_CUDA(cudaStreamCreateWithPriority(&pl->side, cudaStreamNonBlocking, least));
        for (auto &e : pl->sev) CSADV_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    return CSADV_OK;
}

// One step of the fused engine on two streams:
//   side: tracer ghost cells ............................ | wind update (kind 1)
//   main: wind halo + departure-point winds | fused kernel
// The fused kernel waits for both; the wind update for the next step overlaps it.
int fused_step_work(csadv_plan *pl, int kind, cudaStream_t st) {
    int rc = ensure_side(pl);
    if (rc) return rc;
    cudaStream_t sd = pl->side;
    if (pl->f.wpipe && pl->f.sweep) {
        // Pipelined winds: the step kernel reads the records made during the previous step (or
        // just before this one, run_step), while the side stream ticks the clock (kind 1) and
        // makes the next step's records in the other buffer.
        //   main: step kernel (records cur) ............................ | join
        //   side: [clock tick] wind records for the next step (records 1-cur) |
        CSADV_CUDA(cudaEventRecord(pl->sev[0], st));
        CSADV_CUDA(cudaStreamWaitEvent(sd, pl->sev[0], 0));
        const int cur = pl->cur;
        rc = fused_ghosts(pl->opt, pl->grid, pl->T, pl->f, cur, st);  // none with inline ghost cells
        if (!rc)
            rc = fused_kernel(pl->opt, pl->grid, pl->dt, pl->T, pl->f, pl->cur, st, pl->prof ? pl->pev[0] : nullptr,
                              pl->prof ? pl->pev[1] : nullptr);
        if (!rc && kind == 1) rc = do_update_winds(pl, true, 0, 0.0, sd);
        if (!rc) rc = fused_prep_winds(pl->opt, pl->grid, pl->w, pl->dt, pl->f, 1 - cur, sd);
        if (rc) return rc;
        CSADV_CUDA(cudaEventRecord(pl->sev[3], sd));
        CSADV_CUDA(cudaStreamWaitEvent(st, pl->sev[3], 0));
        return CSADV_OK;
    }
    CSADV_CUDA(cudaEventRecord(pl->sev[0], st));
    CSADV_CUDA(cudaStreamWaitEvent(sd, pl->sev[0], 0));
    rc = fused_ghosts(pl->opt, pl->grid, pl->T, pl->f, pl->cur, sd);
    if (rc) return rc;
    const bool td = wind_time_dependent(pl->opt);
    if (td) {
        if (!pl->w.nbasis) rc = wind_halo(pl->opt, pl->grid, pl->w, st);  // the basis includes the halo
        if (!rc) rc = fused_prep_winds(pl->opt, pl->grid, pl->w, pl->dt, pl->f, pl->cur, st);
        if (rc) return rc;
    }
    CSADV_CUDA(cudaEventRecord(pl->sev[1], sd));
    CSADV_CUDA(cudaStreamWaitEvent(st, pl->sev[1], 0));
    if (kind == 1) {
        CSADV_CUDA(cudaEventRecord(pl->sev[2], st));
        CSADV_CUDA(cudaStreamWaitEvent(sd, pl->sev[2], 0));
        rc = do_update_winds(pl, true, 0, 0.0, sd);
        if (rc) return rc;
    }
    rc = fused_kernel(pl->opt, pl->grid, pl->dt, pl->T, pl->f, pl->cur, st, pl->prof ? pl->pev[0] : nullptr,
                      pl->prof ? pl->pev[1] : nullptr);
    if (rc) return rc;
    CSADV_CUDA(cudaEventRecord(pl->sev[3], sd));
    CSADV_CUDA(cudaStreamWaitEvent(st, pl->sev[3], 0));
    return CSADV_OK;
}

int do_time_step(csadv_plan *pl, cudaStream_t st) {
    if (!pl->f.on) {
        if (pl->prof) CSADV_CUDA(cudaEventRecord(pl->pev[0], st));
        int rc = pl->opt.precision == 64 ? time_step<double>(pl, st, true, -1) : time_step<float>(pl, st, true, -1);
        if (!rc && pl->prof) CSADV_CUDA(cudaEventRecord(pl->pev[1], st));
        return rc;
    }
    return fused_step_work(pl, 0, st);
}

// the stored state equals the true state (no pending MF-PR correction)
int settle(csadv_plan *pl, cudaStream_t st) {
    if (!pl->f.on || pl->f.settled) return CSADV_OK;
    return fused_materialize(pl->opt, pl->grid, pl->T, pl->f, pl->cur, st);
}

// tick: the device clock advances one step (csadv_advance); else it is set to (k, t)
int do_update_winds(csadv_plan *pl, bool tick, long long k, double t, cudaStream_t st) {
    return wind_update(pl->opt, pl->grid, pl->w, tick, k, t, st);
}

// the work of one step: adv_time_step, and for kind 1 also update_adv(k * dt) via the clock
int step_work(csadv_plan *pl, int kind, cudaStream_t st) {
    if (pl->f.on) return fused_step_work(pl, kind, st);
    int rc = do_time_step(pl, st);
    if (!rc && kind == 1) rc = do_update_winds(pl, true, 0, 0.0, st);
    return rc;
}

int count_kernel_nodes(cudaGraph_t g) {
    size_t n = 0;
    if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess) return 0;
    std::vector<cudaGraphNode_t> nodes(n);
    if (cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) return 0;
    int k = 0;
    for (auto nd : nodes) {
        cudaGraphNodeType t;
        if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
    }
    return k;
}

// one step (kind 0: time step; kind 1: time step + wind update), replayed from a graph
int run_step(csadv_plan *pl, int kind, cudaStream_t st) {
    if (pl->f.on && pl->f.sweep && pl->f.wpipe && !pl->f.rec_ready) {  // this step's records first
        int rc = fused_prep_winds(pl->opt, pl->grid, pl->w, pl->dt, pl->f, pl->cur, st);
        if (rc) return rc;
        pl->f.rec_ready = true;
    }
    const int par = pl->cur;
    const bool use_graph = pl->graphs && !pl->prof;  // profiled steps launch directly (events on the stream)
    if (use_graph && !pl->gexec[kind][par]) {
        const auto tb = std::chrono::steady_clock::now();
        if (!pl->cap) CSADV_CUDA(cudaStreamCreateWithFlags(&pl->cap, cudaStreamNonBlocking));
        CSADV_CUDA(cudaStreamBeginCapture(pl->cap, cudaStreamCaptureModeThreadLocal));
        int rc = step_work(pl, kind, pl->cap);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(pl->cap, &g);
        pl->cur = par;  // the captured work has not run yet
        if (rc || e != cudaSuccess || !g) {
            if (g) cudaGraphDestroy(g);
            (void)cudaGetLastError();
            pl->graphs = false;  // fall back to direct launches
        } else {
            pl->gkernels[kind][par] = count_kernel_nodes(g);
            e = cudaGraphInstantiate(&pl->gexec[kind][par], g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                (void)cudaGetLastError();
                pl->gexec[kind][par] = nullptr;
                pl->graphs = false;
            }
        }
        pl->stats.graph_builds += 1;
        pl->stats.graph_build_ms +=
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tb).count();
    }
    if (use_graph && pl->graphs && pl->gexec[kind][par]) {
        CSADV_CUDA(cudaGraphLaunch(pl->gexec[kind][par], st));
        if (pl->f.on) pl->cur = 1 - par;
        pl->stats.kernel_launches += pl->gkernels[kind][par];
        pl->stats.kernels_per_step = pl->gkernels[kind][par];
    } else {
        int rc = step_work(pl, kind, st);
        if (rc) return rc;
    }
    pl->stats.steps += 1;
    if (pl->f.on) pl->f.settled = false;
    if (pl->prof) {
        CSADV_CUDA(cudaEventSynchronize(pl->pev[1]));
        float ms = 0.f;
        CSADV_CUDA(cudaEventElapsedTime(&ms, pl->pev[0], pl->pev[1]));
        pl->stats.main_ms += ms;
        pl->stats.main_launches += 1;
    }
    return CSADV_OK;
}

int select_device(csadv_plan *pl) {
    int cur = -1;
    CSADV_CUDA(cudaGetDevice(&cur));
    if (cur != pl->device) CSADV_CUDA(cudaSetDevice(pl->device));
    return CSADV_OK;
}

int zero(void *p, size_t bytes, cudaStream_t st) {
    CSADV_CUDA(cudaMemsetAsync(p, 0, bytes, st));
    return CSADV_OK;
}

int copy_d2d(void *dst, const void *src, size_t bytes, cudaStream_t st) {
    CSADV_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st));
    return CSADV_OK;
}

IcParams ic_params(const csadv_plan *pl, const double *ic_param) {
    IcParams p{};
    if (ic_param)
        for (int c = 0; c < 4; ++c) p.ic[c] = ic_param[c];
    for (int c = 0; c < 4; ++c) p.wind[c] = pl->opt.wp[c];
    return p;
}

}  // namespace

namespace csadv {

int plan_pre_step(csadv_plan *pl, cudaStream_t st, bool ghosts) {
    int rc = ghosts ? fused_ghosts(pl->opt, pl->grid, pl->T, pl->f, pl->cur, st) : CSADV_OK;
    if (!rc && wind_time_dependent(pl->opt)) {
        if (!pl->w.nbasis) rc = wind_halo(pl->opt, pl->grid, pl->w, st);
        if (!rc) rc = fused_prep_winds(pl->opt, pl->grid, pl->w, pl->dt, pl->f, pl->cur, st);
    }
    return rc;
}

int plan_post_step(csadv_plan *pl, int kind, cudaStream_t st) {
    return kind == 1 ? do_update_winds(pl, true, 0, 0.0, st) : CSADV_OK;
}

int plan_select_device(csadv_plan *pl) { return select_device(pl); }

int plan_settle(csadv_plan *pl, cudaStream_t st) { return settle(pl, st); }

int graph_kernel_nodes(cudaGraph_t g) { return count_kernel_nodes(g); }

}  // namespace csadv

namespace {

// Tracer upload and read-out on the fused engine with MF-PR, without materialising the pending
// correction of the other tracers: the upload clears this tracer's correction (the new field
// replaces the corrected one) and, in FP32, records its mass target in the same pass; the
// read-out forms Q* + g corr as it reads.  Both give the bits of materialise-then-copy.
template <class real>
static int tracer_upload(csadv_plan *pl, int tracer, double *src, int layout, cudaStream_t st) {
    FusedState &f = pl->f;
    IoLazy<real> x;
    if (f.on && pl->opt.mf == MF_PR) {
        x.corr = f.corr[pl->cur] + tracer;
        if (f.mass_target) {
            x.g = (const real *)f.g_pc;
            x.part = f.anchor_part;
            x.count = f.anchor_count;
            x.mass = f.mass_target + tracer;
        }
    }
    return tracer_io<real>(pl->grid, (real *)pl->tracer(tracer), src, layout, true, st, &x);
}
template <class real>
static int tracer_download(csadv_plan *pl, int tracer, double *dst, int layout, cudaStream_t st) {
    FusedState &f = pl->f;
    IoLazy<real> x;
    if (f.on && pl->opt.mf == MF_PR && !f.settled) {
        x.g = (const real *)f.g_pc;
        x.corr = f.corr[pl->cur] + tracer;
    }
    return tracer_io<real>(pl->grid, (real *)pl->tracer(tracer), dst, layout, false, st, &x);
}

// ---------------------------------------------------------------- host-resident state (csadv_advance_host)
int ensure_host_pipeline(csadv_plan *pl, cudaStream_t st) {
    if (!pl->up) {
        CSADV_CUDA(cudaStreamCreateWithFlags(&pl->up, cudaStreamNonBlocking));
        CSADV_CUDA(cudaStreamCreateWithFlags(&pl->down, cudaStreamNonBlocking));
        // the split steps' kernels and the upload conversions at the highest priority: the next
        // step's wind records (side stream) fill the SMs they leave free
        int least = 0, greatest = 0;
        CSADV_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        CSADV_CUDA(cudaStreamCreateWithPriority(&pl->hp, cudaStreamNonBlocking, greatest));
        CSADV_CUDA(cudaStreamCreateWithPriority(&pl->cv, cudaStreamNonBlocking, greatest));
        pl->hev.assign(3 * (size_t)pl->T + 4, nullptr);
        for (auto &e : pl->hev) CSADV_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    if (pl->hstage) return CSADV_OK;
    pl->mem.set_stream(st);
    const long long n = pl->grid.d.n;
    pl->hstage = pl->mem.alloc<double>(2LL * pl->T * NFACE * n * n);
    return pl->mem.ok() ? CSADV_OK : CSADV_ERR_OOM;
}

// tracer t of Qbuf[buf] -> dst (layout), with the tracer's pending MF-PR correction applied
template <class real>
int stage_tracer_out(csadv_plan *pl, int buf, int t, double *dst, int layout, cudaStream_t st) {
    FusedState &f = pl->f;
    IoLazy<real> x;
    if (pl->opt.mf == MF_PR) {
        x.g = (const real *)f.g_pc;
        x.corr = f.corr[buf] + t;
    }
    real *Q = (real *)((char *)f.Qbuf[buf] + (size_t)t * pl->grid.d.field * sizeof(real));
    return tracer_io<real>(pl->grid, Q, dst, layout, false, st, &x);
}

// The side stream's part of a step of the fused engine with pipelined winds, after event
// `after`: the clock tick and the next step's records (part -1: all of them; 0: the x-edges',
// the y-edges' to follow), into the buffer the current step does not read.  The x-edges' records
// come first, computing the next step's time factors themselves, and the tick after them: the
// records start at once.
int side_begin(csadv_plan *pl, cudaEvent_t after, int part) {
    int rc = ensure_side(pl);
    if (rc) return rc;
    cudaStream_t sd = pl->side;
    CSADV_CUDA(cudaStreamWaitEvent(sd, after, 0));
    const bool early = part == 0 && pl->f.wpipe;
    if (early) rc = fused_prep_winds(pl->opt, pl->grid, pl->w, pl->dt, pl->f, 1 - pl->cur, sd, 0, 1);
    if (!rc) rc = do_update_winds(pl, true, 0, 0.0, sd);
    if (!rc && pl->f.wpipe && !early)
        rc = fused_prep_winds(pl->opt, pl->grid, pl->w, pl->dt, pl->f, 1 - pl->cur, sd, part);
    return rc;
}

// One step of the fused engine with the step kernel launched once per tracer.  On `st`, tracer
// t's kernel follows out(t - 1, cur) (t > 0) and in(t); out(T - 1, cur) follows the last kernel
// (cur: the step's input buffer; the results are in 1 - cur).  The side stream ticks the clock and
// makes the next step's records beside the kernels, as in fused_step_work: started here, or
// (side_started) by the caller with side_begin(part 0) when the first tracer arrives by upload:
// the x-edges' records then fill the wait for that upload, and the y-edges' follow the last
// kernel, beside the last read-out (records CTAs cannot be preempted: launched beside a step
// kernel or a conversion they slow it, and one launch of all records would still hold the SMs
// when the first tracer is in place).
template <class In, class Out>
int split_step(csadv_plan *pl, cudaStream_t st, bool side_started, In in, Out out) {
    FusedState &f = pl->f;
    int rc = ensure_side(pl);
    if (rc) return rc;
    if (f.wpipe && !f.rec_ready) {  // this step's records first (before the clock ticks)
        // a caller that starts the side stream itself has made them first (the tick is queued)
        if (side_started) return CSADV_ERR_UNSUPPORTED;
        rc = fused_prep_winds(pl->opt, pl->grid, pl->w, pl->dt, f, pl->cur, st);
        if (rc) return rc;
        f.rec_ready = true;
    }
    const int cur = pl->cur, T = pl->T;
    cudaStream_t sd = pl->side;
    if (!side_started) {
        CSADV_CUDA(cudaEventRecord(pl->sev[0], st));
        rc = side_begin(pl, pl->sev[0], -1);
        if (rc) return rc;
    }
    for (int t = 0; t < T; ++t) {
        if (t > 0) rc = out(t - 1, cur);  // the previous tracer's read-out as early as possible
        if (!rc) rc = in(t);
        if (!rc) rc = fused_kernel_tracer(pl->opt, T, f, cur, t, st);
        if (rc) return rc;
    }
    if (f.wpipe && side_started) {  // the y-edges' records beside the last read-out
        CSADV_CUDA(cudaEventRecord(pl->sev[1], st));
        CSADV_CUDA(cudaStreamWaitEvent(sd, pl->sev[1], 0));
        rc = fused_prep_winds(pl->opt, pl->grid, pl->w, pl->dt, f, 1 - cur, sd, 1);
        if (rc) return rc;
    }
    CSADV_CUDA(cudaEventRecord(pl->sev[3], sd));
    rc = out(T - 1, cur);
    if (rc) return rc;
    CSADV_CUDA(cudaStreamWaitEvent(st, pl->sev[3], 0));
    pl->cur = 1 - cur;
    f.settled = false;
    const int kernels = T + 1 + (f.wpipe ? (side_started ? 2 : 1) : 0);  // step kernels, clock tick, records
    pl->stats.steps += 1;
    pl->stats.kernel_launches += kernels;
    pl->stats.kernels_per_step = kernels;
    return CSADV_OK;
}

}  // namespace

extern "C" {

const char *csadv_version(void) { return "csadv 0.1 (sm_103a)"; }

const char *csadv_status_string(int s) {
    switch (s) {
        case CSADV_OK: return "ok";
        case CSADV_ERR_OPTION: return "invalid option code";
        case CSADV_ERR_OPTION_PAIR: return "unsupported splitting / metric-tensor pair";
        case CSADV_ERR_ARG: return "invalid argument";
        case CSADV_ERR_OOM: return "out of memory";
        case CSADV_ERR_CUDA: return "CUDA error";
        case CSADV_ERR_NONFINITE: return "non-finite value in the state";
        case CSADV_ERR_BLOWUP: return "error norm above 100 (blow-up)";
        case CSADV_ERR_UNSUPPORTED: return "option combination not supported by this engine";
        case CSADV_ERR_TOO_LARGE: return "request exceeds a fixed capacity";
        default: return "unknown status";
    }
}

int csadv_set_device(int device) {
    int n = 0;
    CSADV_CUDA(cudaGetDeviceCount(&n));
    if (device < 0 || device >= n) return CSADV_ERR_ARG;
    CSADV_CUDA(cudaSetDevice(device));
    g_device = device;
    return CSADV_OK;
}

int csadv_plan_create(int N, double dt, int ntracers, const csadv_options *opt, void *stream, csadv_plan **out) {
    if (!out) return CSADV_ERR_ARG;
    *out = nullptr;
    Options o;
    int rc = validate_options(opt, o);
    if (rc) return rc;
    if (N < 8 || N > 16384 || ntracers < 1 || ntracers > 64 || !(dt != 0.0) || dt != dt || dt < -4.0)
        return CSADV_ERR_ARG;
    // dt < 0: -dt is the target CFL number; dt follows from the t = 0 winds below
    const double cfl_target = dt < 0.0 ? -dt : 0.0;
    if (cfl_target > 0.0) dt = 1.0;
    if (o.engine == CSADV_ENGINE_FUSED && !fused_supported(o)) return CSADV_ERR_UNSUPPORTED;
    const bool fused = o.engine == CSADV_ENGINE_FUSED || (o.engine == CSADV_ENGINE_AUTO && fused_supported(o));
    csadv_plan *pl = new (std::nothrow) csadv_plan();
    if (!pl) return CSADV_ERR_OOM;
    pl->opt = o;
    pl->N = N;
    pl->T = ntracers;
    pl->dt = dt;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        delete pl;
        return CSADV_ERR_CUDA;
    }
    pl->device = dev;
    cudaStream_t st = S(stream);
    rc = acquire_grid(N, dev, st, pl->gref);
    if (rc) {
        delete pl;
        return rc;
    }
    pl->grid = pl->gref->grid;
    // failures below: the queued work ends before the memory returns to the pool
    auto fail = [&](int e) {
        cudaStreamSynchronize(st);
        (void)cudaGetLastError();
        release_grid(pl, st);
        delete pl;
        return e;
    };
    const Dims d = pl->grid.d;
    const long long F = d.field;
    const size_t es = pl->esize();
    cudaMemPool_t pool = device_pool();
    if (!pool) return fail(CSADV_ERR_CUDA);
    pl->mem.use_pool(pool, st);
    pl->Q = pl->mem.alloc<char>((long long)ntracers * F * es);
    pl->npart = staged_partial_count(pl->grid);
    pl->partials = pl->mem.alloc<double>(pl->npart);
    pl->scal = pl->mem.alloc<double>(8);
    pl->stage = pl->mem.alloc<double>((long long)NFACE * d.n * d.n);
    pl->tmp = pl->mem.alloc<double>(3LL * diag_partials(pl->grid) + 8);
    if (!pl->mem.ok()) return fail(CSADV_ERR_OOM);
    // the staged engine's scratch (fused plans allocate it on first use: csadv_divergence)
    if (!fused) rc = ensure_scratch(pl, st);
    if (!rc && fused) {
        pl->f.Qbuf[0] = pl->Q;
        rc = fused_alloc(o, pl->grid, ntracers, pl->mem, pl->f, st);
    }
    if (!rc) rc = zero(pl->Q, (size_t)ntracers * F * es, st);
    if (rc) return fail(rc);
    // init_vars_adv (advection_vars.py:19-107): t = 0 winds, wind halo, old <- current,
    // departure-point winds, CFL
    rc = wind_setup(o, pl->grid, pl->w, pl->mem, dt, st);
    if (!rc && fused) rc = wind_basis_setup(o, pl->grid, pl->w, pl->mem, st);
    if (!rc && fused) rc = fused_wind_pipeline(o, pl->grid, pl->w, pl->mem, pl->f, st);  // before the descriptors
    if (!rc) rc = wind_initial(o, pl->grid, pl->w, st);
    if (!rc) rc = wind_halo(o, pl->grid, pl->w, st);
    if (!rc) rc = copy_d2d(pl->w.u_old, pl->w.u_pu, (size_t)F * pl->w.esize, st);
    if (!rc) rc = copy_d2d(pl->w.v_old, pl->w.v_pv, (size_t)F * pl->w.esize, st);
    if (!rc && cfl_target > 0.0) {
        double c1 = 0.0;  // CFL number of dt = 1
        rc = wind_cfl(o, pl->grid, pl->w, 1.0, pl->tmp, c1, st);
        if (!rc && !(c1 > 0.0)) rc = CSADV_ERR_ARG;  // no wind: dt undefined
        if (!rc) {
            dt = cfl_target / c1;
            pl->dt = dt;
            rc = wind_set_dt(pl->w, dt, st);
        }
    }
    if (!rc && fused)
        rc = fused_set_tile(o, pl->grid, ntracers, dt, pl->f, o.tile > 0 ? o.tile - 1 : default_tile(o, N, ntracers), st);
    if (!rc) rc = wind_average(o, pl->grid, pl->w, dt, st);
    if (!rc) rc = wind_cfl(o, pl->grid, pl->w, dt, pl->tmp, pl->cfl, st);
    if (!rc && fused) rc = fused_prep_winds(o, pl->grid, pl->w, dt, pl->f, pl->cur, st);
    pl->f.rec_ready = true;
    if (rc) return fail(rc);
    *out = pl;
    return CSADV_OK;
}

int csadv_get_dt(const csadv_plan *pl, double *dt) {
    if (!pl || !dt) return CSADV_ERR_ARG;
    *dt = pl->dt;
    return CSADV_OK;
}

int csadv_plan_destroy(csadv_plan *plan) {
    if (!plan) return CSADV_ERR_ARG;
    batch_forget(plan);
    select_device(plan);
    cudaDeviceSynchronize();
    release_grid(plan, cudaStreamPerThread);
    delete plan;
    return CSADV_OK;
}

int csadv_plan_release(csadv_plan *plan, void *stream) {
    if (!plan) return CSADV_ERR_ARG;
    batch_forget(plan);
    select_device(plan);
    cudaStream_t st = S(stream);
    plan->mem.release_on(st);
    release_grid(plan, st);
    delete plan;  // its graphs, streams and events are released by CUDA once their work is done
    return CSADV_OK;
}

int csadv_init_tracer(csadv_plan *pl, int tracer, int ic, const double *ic_param, void *stream) {
    if (!pl || tracer < 0 || tracer >= pl->T) return CSADV_ERR_ARG;
    if (!((ic >= 1 && ic <= 4) || (ic >= CSADV_IC_HILL && ic <= CSADV_IC_SMOOTH_BELLS))) return CSADV_ERR_OPTION;
    if (ic == CSADV_IC_HILL && !ic_param) return CSADV_ERR_ARG;
    IcParams p = ic_params(pl, ic_param);
    cudaStream_t st = S(stream);
    int rc = settle(pl, st);  // a pending correction belongs to the old field
    if (rc) return rc;
    rc = pl->opt.precision == 64 ? init_tracer<double>(pl->grid, ic, pl->opt.vf, p, (double *)pl->tracer(tracer), st)
                                 : init_tracer<float>(pl->grid, ic, pl->opt.vf, p, (float *)pl->tracer(tracer), st);
    if (!rc && pl->f.on) rc = fused_anchor_mass(pl->opt, pl->grid, pl->f, pl->cur, tracer, st);
    return rc;
}

// Page-locked host memory (cudaMallocHost, csadv_host_alloc, cudaHostRegister) is mapped into the
// device's address space: the layout conversion then reads or writes the caller's array directly
// (one pass over the interconnect, no staging copy).  Returns the device-side address of `host`, or
// null for pageable memory, which goes through a copy into the plan's staging buffer.
static double *mapped_host(const void *host) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? (double *)a.devicePointer : nullptr;
}

int csadv_set_tracer(csadv_plan *pl, int tracer, const double *host, int layout, void *stream) {
    if (!pl || !host || tracer < 0 || tracer >= pl->T) return CSADV_ERR_ARG;
    if (layout != CSADV_LAYOUT_FULL && layout != CSADV_LAYOUT_INTERIOR) return CSADV_ERR_ARG;
    const Dims d = pl->grid.d;
    const int m = layout == CSADV_LAYOUT_FULL ? d.n : d.N;
    cudaStream_t st = S(stream);
    double *src = mapped_host(host);
    if (!src) {
        CSADV_CUDA(cudaMemcpyAsync(pl->stage, host, (size_t)NFACE * m * m * sizeof(double), cudaMemcpyHostToDevice, st));
        src = pl->stage;
    }
    return pl->opt.precision == 64 ? tracer_upload<double>(pl, tracer, src, layout, st)
                                   : tracer_upload<float>(pl, tracer, src, layout, st);
}

int csadv_get_tracer(csadv_plan *pl, int tracer, double *host, int layout, void *stream) {
    if (!pl || !host || tracer < 0 || tracer >= pl->T) return CSADV_ERR_ARG;
    if (layout != CSADV_LAYOUT_FULL && layout != CSADV_LAYOUT_INTERIOR) return CSADV_ERR_ARG;
    const Dims d = pl->grid.d;
    const int m = layout == CSADV_LAYOUT_FULL ? d.n : d.N;
    cudaStream_t st = S(stream);
    // the full array carries the ghost cells filled at the start of the last step, as the
    // reference's Q does; the fused engine keeps them in its other buffer
    if (layout == CSADV_LAYOUT_FULL && pl->f.on && pl->k > 0) {
        int rc = fused_ghosts_to_current(pl->opt, pl->grid, pl->T, pl->f, pl->cur, st);
        if (rc) return rc;
    }
    double *dst = mapped_host(host);
    int rc = pl->opt.precision == 64 ? tracer_download<double>(pl, tracer, dst ? dst : pl->stage, layout, st)
                                     : tracer_download<float>(pl, tracer, dst ? dst : pl->stage, layout, st);
    if (rc) return rc;
    if (!dst)
        CSADV_CUDA(cudaMemcpyAsync(host, pl->stage, (size_t)NFACE * m * m * sizeof(double), cudaMemcpyDeviceToHost, st));
    CSADV_CUDA(cudaStreamSynchronize(st));
    return CSADV_OK;
}

int csadv_advance_host(csadv_plan *pl, int nsteps, const double *const *in, int in_layout, double *const *out,
                       int out_layout, void *stream) {
    if (!pl || nsteps < 0) return CSADV_ERR_ARG;
    const int T = pl->T;
    for (int t = 0; t < T; ++t)
        if ((in && !in[t]) || (out && !out[t])) return CSADV_ERR_ARG;
    auto bad = [](int l) { return l != CSADV_LAYOUT_FULL && l != CSADV_LAYOUT_INTERIOR; };
    if ((in && bad(in_layout)) || (out && bad(out_layout))) return CSADV_ERR_ARG;
    cudaStream_t st = S(stream);
    FusedState &f = pl->f;
    const bool overlap = f.on && f.sweep && f.inline_ghosts && !pl->prof && nsteps >= 1 &&
                         (f.wpipe || !wind_time_dependent(pl->opt));
    int rc = CSADV_OK;
    if (!overlap) {  // the same calls one after another
        for (int t = 0; in && !rc && t < T; ++t) rc = csadv_set_tracer(pl, t, in[t], in_layout, stream);
        if (!rc) rc = csadv_advance(pl, nsteps, stream);
        for (int t = 0; out && !rc && t < T; ++t) rc = csadv_get_tracer(pl, t, out[t], out_layout, stream);
        if (!rc) CSADV_CUDA(cudaStreamSynchronize(st));
        return rc;
    }
    rc = ensure_host_pipeline(pl, st);
    if (!rc) rc = ensure_side(pl);
    if (rc) return rc;
    const Dims d = pl->grid.d;
    const size_t slot = (size_t)NFACE * d.n * d.n;  // doubles per staging array (full layout)
    auto cells = [&](int l) { return (size_t)NFACE * (l == CSADV_LAYOUT_FULL ? (size_t)d.n * d.n : (size_t)d.N * d.N); };
    double *sin = pl->hstage, *sout = pl->hstage + (size_t)T * slot;
    cudaEvent_t *uploaded = pl->hev.data(), *converted = pl->hev.data() + T, *arrived = pl->hev.data() + 2 * T;
    cudaEvent_t fork = pl->hev[3 * T], downloaded = pl->hev[3 * T + 1], to_hp = pl->hev[3 * T + 2],
                from_hp = pl->hev[3 * T + 3];
    const bool f64 = pl->opt.precision == 64;
    cudaStream_t hp = pl->hp, cv = pl->cv;
    if (f.wpipe && !f.rec_ready) {  // this step's records, while the clock holds its time
        rc = fused_prep_winds(pl->opt, pl->grid, pl->w, pl->dt, f, pl->cur, st);
        if (rc) return rc;
        f.rec_ready = true;
    }
    CSADV_CUDA(cudaEventRecord(fork, st));
    // with an upload, the first step's side-stream work is queued first: the clock tick and the
    // next step's x-edge records run while the first tracer is copied
    if (in) rc = side_begin(pl, fork, 0);
    if (rc) return rc;
    if (in) {  // copies on the copy engine (host -> staging), all tracers in order
        CSADV_CUDA(cudaStreamWaitEvent(pl->up, fork, 0));
        for (int t = 0; t < T; ++t) {
            CSADV_CUDA(cudaMemcpyAsync(sin + t * slot, in[t], cells(in_layout) * sizeof(double), cudaMemcpyHostToDevice,
                                       pl->up));
            CSADV_CUDA(cudaEventRecord(uploaded[t], pl->up));
        }
    }
    auto convert_in = [&](int t, cudaStream_t s) -> int {  // staging -> the tracer's field
        CSADV_CUDA(cudaStreamWaitEvent(s, uploaded[t], 0));
        const int r = f64 ? tracer_upload<double>(pl, t, sin + t * slot, in_layout, s)
                          : tracer_upload<float>(pl, t, sin + t * slot, in_layout, s);
        if (r) return r;
        CSADV_CUDA(cudaEventRecord(arrived[t], s));
        return CSADV_OK;
    };
    // tracer t in place before its kernel: tracer 0 converted on the kernels' stream itself, the
    // others on the conversion stream as their copies land (beside tracer 0's kernel), one after
    // another (the FP32 form's mass sums share their partials)
    auto wait_in = [&](int t) -> int {
        if (!in) return CSADV_OK;
        if (t == 0) {
            int r = convert_in(0, hp);
            if (r) return r;
            CSADV_CUDA(cudaStreamWaitEvent(cv, arrived[0], 0));
            for (int u = 1; u < T && !r; ++u) r = convert_in(u, cv);
            return r;
        }
        CSADV_CUDA(cudaStreamWaitEvent(hp, arrived[t], 0));
        return CSADV_OK;
    };
    auto convert_out = [&](int t, int cur) -> int {  // the step's result -> staging -> host
        if (!out) return CSADV_OK;
        const int nb = 1 - cur;
        int r = out_layout == CSADV_LAYOUT_FULL ? fused_ghosts_to_current(pl->opt, pl->grid, 1, f, nb, hp, t) : 0;
        if (!r) r = f64 ? stage_tracer_out<double>(pl, nb, t, sout + t * slot, out_layout, hp)
                        : stage_tracer_out<float>(pl, nb, t, sout + t * slot, out_layout, hp);
        if (r) return r;
        CSADV_CUDA(cudaEventRecord(converted[t], hp));
        CSADV_CUDA(cudaStreamWaitEvent(pl->down, converted[t], 0));
        CSADV_CUDA(cudaMemcpyAsync(out[t], sout + t * slot, cells(out_layout) * sizeof(double), cudaMemcpyDeviceToHost,
                                   pl->down));
        return CSADV_OK;
    };
    auto none_in = [](int) { return CSADV_OK; };
    auto none_out = [](int, int) { return CSADV_OK; };
    // the first and the last step on the high-priority stream, forked from and joined to `st`
    auto on_hp = [&](bool side_started, auto in_fn, auto out_fn) -> int {
        CSADV_CUDA(cudaEventRecord(to_hp, st));
        CSADV_CUDA(cudaStreamWaitEvent(hp, to_hp, 0));
        const int r = split_step(pl, hp, side_started, in_fn, out_fn);
        CSADV_CUDA(cudaEventRecord(from_hp, hp));
        CSADV_CUDA(cudaStreamWaitEvent(st, from_hp, 0));
        return r;
    };
    for (int s = 0; s < nsteps && !rc; ++s) {
        const bool first = s == 0, last = s == nsteps - 1;
        if (first && last) rc = on_hp(in != nullptr, wait_in, convert_out);
        else if (first) rc = on_hp(in != nullptr, wait_in, none_out);
        else if (last) rc = on_hp(false, none_in, convert_out);
        else rc = run_step(pl, 1, st);
        if (!rc) pl->k += 1;
    }
    if (rc) return rc;
    if (out) {
        CSADV_CUDA(cudaEventRecord(downloaded, pl->down));
        CSADV_CUDA(cudaStreamWaitEvent(st, downloaded, 0));
    }
    CSADV_CUDA(cudaStreamSynchronize(st));
    return CSADV_OK;
}

int csadv_time_step(csadv_plan *pl, int k, void *stream) {
    if (!pl) return CSADV_ERR_ARG;
    int rc = run_step(pl, 0, S(stream));
    if (rc) return rc;
    pl->k = k;
    return CSADV_OK;
}

int csadv_update_winds(csadv_plan *pl, double t, void *stream) {
    if (!pl) return CSADV_ERR_ARG;
    pl->f.rec_ready = false;  // pipelined winds: the next step's records follow the new clock
    return do_update_winds(pl, false, pl->k, t, S(stream));
}

int csadv_advance(csadv_plan *pl, int nsteps, void *stream) {
    if (!pl || nsteps < 0) return CSADV_ERR_ARG;
    cudaStream_t st = S(stream);
    for (int s = 0; s < nsteps; ++s) {
        int rc = run_step(pl, 1, st);
        if (rc) return rc;
        pl->k += 1;
    }
    return CSADV_OK;
}

int csadv_mass(csadv_plan *pl, int tracer, double *mass, void *stream) {
    if (!pl || !mass || tracer < 0 || tracer >= pl->T) return CSADV_ERR_ARG;
    int rc = settle(pl, S(stream));
    if (rc) return rc;
    if (pl->opt.precision == 64) return diag_mass<double>(pl->grid, (const double *)pl->tracer(tracer), pl->tmp, *mass, S(stream));
    return diag_mass<float>(pl->grid, (const float *)pl->tracer(tracer), pl->tmp, *mass, S(stream));
}

int csadv_errors(csadv_plan *pl, int tracer, int ic, const double *ic_param, double t, double out[3], void *stream) {
    if (!pl || !out || tracer < 0 || tracer >= pl->T) return CSADV_ERR_ARG;
    if (!((ic >= 1 && ic <= 4) || (ic >= CSADV_IC_HILL && ic <= CSADV_IC_SMOOTH_BELLS))) return CSADV_ERR_OPTION;
    if (ic == CSADV_IC_HILL && !ic_param) return CSADV_ERR_ARG;
    IcParams p = ic_params(pl, ic_param);
    int rc = settle(pl, S(stream));
    if (rc) return rc;
    rc = pl->opt.precision == 64
                 ? diag_errors<double>(pl->grid, (const double *)pl->tracer(tracer), ic, pl->opt.vf, p, t, pl->tmp, out, S(stream))
                 : diag_errors<float>(pl->grid, (const float *)pl->tracer(tracer), ic, pl->opt.vf, p, t, pl->tmp, out, S(stream));
    if (rc) return rc;
    if (!(out[0] == out[0])) return CSADV_ERR_NONFINITE;
    if (out[0] > 100.0) return CSADV_ERR_BLOWUP;
    return CSADV_OK;
}

int csadv_get_cfl(const csadv_plan *pl, double *cfl) {
    if (!pl || !cfl) return CSADV_ERR_ARG;
    *cfl = pl->cfl;
    return CSADV_OK;
}

int csadv_get_step(const csadv_plan *pl, int *k) {
    if (!pl || !k) return CSADV_ERR_ARG;
    *k = pl->k;
    return CSADV_OK;
}

int csadv_divergence(csadv_plan *pl, int tracer, double *host_div, void *stream) {
    if (!pl || !host_div || tracer < 0 || tracer >= pl->T) return CSADV_ERR_ARG;
    cudaStream_t st = S(stream);
    int rc = settle(pl, st);
    if (!rc) rc = wind_sync(pl->opt, pl->grid, pl->w, st);  // the staged operators read u_pu, u_old
    if (rc) return rc;
    rc = pl->opt.precision == 64 ? time_step<double>(pl, st, false, tracer) : time_step<float>(pl, st, false, tracer);
    if (rc) return rc;
    rc = pl->opt.precision == 64 ? tracer_io<double>(pl->grid, (double *)pl->s.div, pl->stage, CSADV_LAYOUT_INTERIOR, false, st)
                                 : tracer_io<float>(pl->grid, (float *)pl->s.div, pl->stage, CSADV_LAYOUT_INTERIOR, false, st);
    if (rc) return rc;
    const Dims d = pl->grid.d;
    CSADV_CUDA(cudaMemcpyAsync(host_div, pl->stage, (size_t)NFACE * d.N * d.N * sizeof(double), cudaMemcpyDeviceToHost, st));
    CSADV_CUDA(cudaStreamSynchronize(st));
    return CSADV_OK;
}

int csadv_set_graphs(csadv_plan *pl, int enable) {
    if (!pl) return CSADV_ERR_ARG;
    pl->drop_graphs();
    pl->graphs = enable != 0;
    return CSADV_OK;
}

int csadv_set_inline_ghosts(csadv_plan *pl, int enable) {
    if (!pl) return CSADV_ERR_ARG;
    if (!pl->f.on || !pl->f.sweep) return CSADV_ERR_UNSUPPORTED;
    if (pl->f.inline_ghosts == (enable != 0)) return CSADV_OK;
    cudaStream_t st = (cudaStream_t)0;
    int rc = settle(pl, st);
    if (rc) return rc;
    pl->f.inline_ghosts = enable != 0;
    rc = fused_set_tile(pl->opt, pl->grid, pl->T, pl->dt, pl->f, pl->f.tile, st);
    if (rc) return rc;
    pl->drop_graphs();
    batch_touch(pl);
    return CSADV_OK;
}

int csadv_set_profiling(csadv_plan *pl, int enable) {
    if (!pl) return CSADV_ERR_ARG;
    if (enable && !pl->pev[0]) {
        CSADV_CUDA(cudaEventCreate(&pl->pev[0]));
        CSADV_CUDA(cudaEventCreate(&pl->pev[1]));
    }
    pl->prof = enable != 0;
    return CSADV_OK;
}

int csadv_get_stats(csadv_plan *pl, csadv_stats *out) {
    if (!pl || !out) return CSADV_ERR_ARG;
    *out = pl->stats;
    out->engine = pl->f.on ? CSADV_ENGINE_FUSED : CSADV_ENGINE_STAGED;
    out->tile = pl->f.on ? pl->f.tile + 1 : 0;
    out->device_bytes = pl->mem.bytes() + (pl->gref ? pl->gref->mem.bytes() : 0);
    return CSADV_OK;
}

int csadv_set_step(csadv_plan *pl, int k, void *stream) {
    if (!pl || k < 0) return CSADV_ERR_ARG;
    cudaStream_t st = S(stream);
    int rc = select_device(pl);
    // the clock (and, for per-edge winds, the current and previous winds) at (k-1) dt, then at
    // k dt: what k steps of csadv_advance leave
    pl->k = k > 0 ? k - 1 : 0;
    if (!rc) rc = do_update_winds(pl, false, pl->k, pl->k * pl->dt, st);
    pl->k = k;
    if (!rc) rc = do_update_winds(pl, false, pl->k, pl->k * pl->dt, st);
    pl->f.rec_ready = false;
    if (!rc) CSADV_CUDA(cudaStreamSynchronize(st));
    return rc;
}

int csadv_mass_target(csadv_plan *pl, int tracer, double *get, const double *set, void *stream) {
    if (!pl || tracer < 0 || tracer >= pl->T) return CSADV_ERR_ARG;
    if (!pl->f.on || !pl->f.mass_target) return CSADV_ERR_UNSUPPORTED;
    cudaStream_t st = S(stream);
    if (get) {
        CSADV_CUDA(cudaMemcpyAsync(get, pl->f.mass_target + tracer, sizeof(double), cudaMemcpyDeviceToHost, st));
        CSADV_CUDA(cudaStreamSynchronize(st));
    }
    if (set) {
        CSADV_CUDA(cudaMemcpyAsync(pl->f.mass_target + tracer, set, sizeof(double), cudaMemcpyHostToDevice, st));
        CSADV_CUDA(cudaStreamSynchronize(st));
    }
    return CSADV_OK;
}

int csadv_reset_stats(csadv_plan *pl) {
    if (!pl) return CSADV_ERR_ARG;
    pl->stats = csadv_stats{};
    return CSADV_OK;
}

int csadv_host_alloc(void **ptr, size_t bytes) {
    if (!ptr) return CSADV_ERR_ARG;
    if (cudaMallocHost(ptr, bytes) != cudaSuccess) {
        (void)cudaGetLastError();
        *ptr = nullptr;
        return CSADV_ERR_OOM;
    }
    return CSADV_OK;
}

int csadv_host_free(void *ptr) {
    if (!ptr) return CSADV_ERR_ARG;
    CSADV_CUDA(cudaFreeHost(ptr));
    return CSADV_OK;
}

}  // extern "C"
