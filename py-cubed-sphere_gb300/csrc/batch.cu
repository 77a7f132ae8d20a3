// Batches of solves (csadv_batch_*) and the tile autotuner (csadv_tune).
//
// A batch advances every attached plan by one step per step with ONE launch of the
// line-marching step kernel for all of them: each plan contributes its own descriptor
// (two, one per buffer parity) and its tiles to a work table, so solves of different N,
// tracer counts, winds and tile shapes share the launch.  The ghost cells of all solves are
// filled by one launch too (a second work table over the same descriptors); only the wind
// work of time-dependent winds (one wind pass and the next clock tick) is launched per plan.  A step is captured as a CUDA
// graph per parity and replayed while the membership does not change.
//
// Results: the kernel's MF-PR sums run in a fixed order per solve (its tiles, then its
// items in index order), so a plan gives the same bits alone and in any batch, provided its
// tile configuration is the same.
#include <algorithm>
#include <map>
#include <chrono>
#include <mutex>
#include <new>
#include <tuple>
#include <vector>

#include "plan.h"
#include "tiles.h"

struct csadv_batch {
    int capacity = 0;
    int device = 0;
    std::vector<csadv_plan *> plans;
    std::vector<int> base_cur;       // each plan's buffer parity when the tables were built
    csadv::DeviceArena mem;
    SweepSolve *dsolves = nullptr;   // [capacity][2]
    int2 *dwork[2] = {nullptr, nullptr};   // step-kernel work tables (per phase)
    int2 *dhwork[2] = {nullptr, nullptr};  // ghost-cell work tables (per phase)
    void *work_mem = nullptr;        // all four tables, grown on demand
    int work_cap = 0;                // entries per table
    int nwork = 0, nhwork = 0;
    size_t smem = 0;
    int precision = 0, recon = 0, split = 0;
    int tgroup = 0;                  // tracer grouping of the FP32 step kernel (SWEEP_TG_*)
    int phase = 0;                   // steps since the tables were built, mod 2
    bool dirty = true;
    bool graphs = true;
    cudaStream_t cap = nullptr;
    cudaGraphExec_t gexec[2] = {nullptr, nullptr};
    int gkernels[2] = {0, 0};
    bool prof = false;               // time the step kernel (direct launches)
    cudaEvent_t pev[2] = {nullptr, nullptr};
    // csadv_batch_set_queue_depth: the ends of the last `qdepth` advance calls
    int qdepth = 0;
    long long qn = 0;
    std::vector<cudaEvent_t> qev;
    csadv_stats stats{};
    void drop_graphs() {
        for (auto &e : gexec)
            if (e) {
                cudaGraphExecDestroy(e);
                e = nullptr;
            }
    }
    ~csadv_batch() {
        drop_graphs();
        for (csadv_plan *p : plans) p->batch = nullptr;
        if (work_mem) cudaFree(work_mem);
        if (cap) cudaStreamDestroy(cap);
        for (auto &e : pev)
            if (e) cudaEventDestroy(e);
        for (auto &e : qev) cudaEventDestroy(e);
    }
};

namespace csadv {
namespace {

bool batch_compatible(const csadv_batch *b, const csadv_plan *pl) {
    if (!pl->f.on || !pl->f.sweep) return false;
    if (b->plans.empty()) return true;
    const csadv_plan *r = b->plans.front();
    return pl->opt.precision == r->opt.precision && pl->opt.recon == r->opt.recon &&
           pl->opt.opsplit == r->opt.opsplit && pl->device == b->device;
}

// descriptors and work tables from the current membership and buffer parities
int batch_rebuild(csadv_batch *b, cudaStream_t st) {
    b->drop_graphs();
    b->phase = 0;
    b->base_cur.clear();
    b->nwork = 0;
    b->smem = 0;
    if (b->plans.empty()) {
        b->dirty = false;
        return CSADV_OK;
    }
    const int M = (int)b->plans.size();
    std::vector<int> order(M);
    for (int m = 0; m < M; ++m) order[m] = m;
    std::stable_sort(order.begin(), order.end(),
                     [&](int x, int y) { return b->plans[x]->f.nitems > b->plans[y]->f.nitems; });
    int total = 0, htotal = 0;
    for (int m = 0; m < M; ++m) {
        csadv_plan *pl = b->plans[m];
        CSADV_CUDA(cudaMemcpyAsync(b->dsolves + 2 * m, pl->f.dsolve, 2 * sizeof(SweepSolve), cudaMemcpyDeviceToDevice,
                                   st));
        b->base_cur.push_back(pl->cur);
        total += pl->f.nitems;
        if (!pl->f.inline_ghosts) htotal += pl->T * halo_blocks(pl->grid.d);
        b->smem = b->smem > pl->f.smem ? b->smem : pl->f.smem;
    }
    const int need = total > htotal ? total : htotal;
    if (need > b->work_cap) {
        if (b->work_mem) {
            CSADV_CUDA(cudaStreamSynchronize(st));
            CSADV_CUDA(cudaFree(b->work_mem));
            b->work_mem = nullptr;
        }
        int cap = need + need / 2 + 64;
        CSADV_CUDA(cudaMalloc(&b->work_mem, 4 * (size_t)cap * sizeof(int2)));
        b->work_cap = cap;
        b->dwork[0] = (int2 *)b->work_mem;
        b->dwork[1] = b->dwork[0] + cap;
        b->dhwork[0] = b->dwork[1] + cap;
        b->dhwork[1] = b->dhwork[0] + cap;
    }
    // step kernel: the tiles of each solve, largest solves first; ghost cells: per solve and
    // tracer the blocks of its ghost-cell strip
    std::vector<int2> h(2 * (size_t)total), hh(2 * (size_t)htotal);
    int e = 0, eh = 0;
    for (int m : order) {
        const csadv_plan *pl = b->plans[m];
        for (int it = 0; it < pl->f.nitems; ++it, ++e) {
            h[e] = make_int2(2 * m + pl->cur, it);
            h[total + e] = make_int2(2 * m + (1 - pl->cur), it);
        }
        const int hb = pl->f.inline_ghosts ? 0 : pl->T * halo_blocks(pl->grid.d);
        for (int it = 0; it < hb; ++it, ++eh) {
            hh[eh] = make_int2(2 * m + pl->cur, it);
            hh[htotal + eh] = make_int2(2 * m + (1 - pl->cur), it);
        }
    }
    CSADV_CUDA(cudaMemcpyAsync(b->dwork[0], h.data(), (size_t)total * sizeof(int2), cudaMemcpyHostToDevice, st));
    CSADV_CUDA(cudaMemcpyAsync(b->dwork[1], h.data() + total, (size_t)total * sizeof(int2), cudaMemcpyHostToDevice, st));
    CSADV_CUDA(cudaMemcpyAsync(b->dhwork[0], hh.data(), (size_t)htotal * sizeof(int2), cudaMemcpyHostToDevice, st));
    CSADV_CUDA(cudaMemcpyAsync(b->dhwork[1], hh.data() + htotal, (size_t)htotal * sizeof(int2), cudaMemcpyHostToDevice,
                               st));
    CSADV_CUDA(cudaStreamSynchronize(st));  // h, hh go out of scope
    b->nwork = total;
    b->nhwork = htotal;
    b->precision = b->plans.front()->opt.precision;
    b->recon = b->plans.front()->opt.recon;
    b->split = b->plans.front()->opt.opsplit;
    b->tgroup = sweep_tgroup(b->plans.front()->T);
    for (csadv_plan *pl : b->plans)
        if (sweep_tgroup(pl->T) != b->tgroup) b->tgroup = SWEEP_TG_ANY;
    b->dirty = false;
    return CSADV_OK;
}

// membership or a plan's parity changed outside the batch -> rebuild
bool batch_stale(const csadv_batch *b) {
    if (b->dirty) return true;
    for (size_t m = 0; m < b->plans.size(); ++m)
        if (b->plans[m]->cur != (b->base_cur[m] ^ b->phase)) return true;
    return false;
}

int batch_step_work(csadv_batch *b, int kind, cudaStream_t st) {
    // ghost cells of every solve in one launch, then each plan's wind work (time-dependent winds)
    // (solves whose step kernel evaluates their ghost cells itself have no items in it)
    int rc0 = b->precision == 64 ? launch_halo_batch<double>(b->dsolves, b->dhwork[b->phase], b->nhwork, st)
                                 : launch_halo_batch<float>(b->dsolves, b->dhwork[b->phase], b->nhwork, st);
    if (rc0) return rc0;
    for (csadv_plan *pl : b->plans) {
        int rc = plan_pre_step(pl, st, false);
        if (rc) return rc;
    }
    if (b->prof) CSADV_CUDA(cudaEventRecord(b->pev[0], st));
    int rc = b->precision == 64
                 ? sweep_launch<double>(b->recon, b->split, b->dsolves, b->dwork[b->phase], b->nwork, b->nwork, b->smem, st,
                                        b->tgroup)
                 : sweep_launch<float>(b->recon, b->split, b->dsolves, b->dwork[b->phase], b->nwork, b->nwork, b->smem, st,
                                       b->tgroup);
    if (rc) return rc;
    if (b->prof) CSADV_CUDA(cudaEventRecord(b->pev[1], st));
    for (csadv_plan *pl : b->plans) {
        rc = plan_post_step(pl, kind, st);
        if (rc) return rc;
    }
    return CSADV_OK;
}

int batch_run_step(csadv_batch *b, int kind, cudaStream_t st) {
    const int ph = b->phase;
    const bool use_graph = b->graphs && !b->prof;
    if (use_graph && !b->gexec[ph]) {
        const auto tb = std::chrono::steady_clock::now();
        if (!b->cap) CSADV_CUDA(cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking));
        CSADV_CUDA(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
        int rc = batch_step_work(b, kind, b->cap);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(b->cap, &g);
        if (rc || e != cudaSuccess || !g) {
            if (g) cudaGraphDestroy(g);
            (void)cudaGetLastError();
            b->graphs = false;
        } else {
            b->gkernels[ph] = graph_kernel_nodes(g);
            e = cudaGraphInstantiate(&b->gexec[ph], g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                (void)cudaGetLastError();
                b->gexec[ph] = nullptr;
                b->graphs = false;
            }
        }
        b->stats.graph_builds += 1;
        b->stats.graph_build_ms +=
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - tb).count();
    }
    if (use_graph && b->graphs && b->gexec[ph]) {
        CSADV_CUDA(cudaGraphLaunch(b->gexec[ph], st));
        b->stats.kernel_launches += b->gkernels[ph];
        b->stats.kernels_per_step = b->gkernels[ph];
    } else {
        int rc = batch_step_work(b, kind, st);
        if (rc) return rc;
    }
    for (csadv_plan *pl : b->plans) {
        pl->cur = 1 - pl->cur;
        pl->k += 1;
        pl->f.settled = false;
        pl->f.rec_ready = false;  // a batch step makes no records for the plan's next step
        pl->stats.steps += 1;
    }
    b->phase ^= 1;
    b->stats.steps += 1;
    if (b->prof) {
        CSADV_CUDA(cudaEventSynchronize(b->pev[1]));
        float ms = 0.f;
        CSADV_CUDA(cudaEventElapsedTime(&ms, b->pev[0], b->pev[1]));
        b->stats.main_ms += ms;
        b->stats.main_launches += 1;
    }
    return CSADV_OK;
}

// ---------------------------------------------------------------- autotuner cache
using TuneKey = std::tuple<int, int, int, int, int, int, int>;  // N, T, precision, recon, opsplit, mt, mf
std::mutex g_tune_mu;
std::map<TuneKey, int> g_tune;

TuneKey tune_key(const csadv_plan *pl) {
    const Options &o = pl->opt;
    return TuneKey(pl->N, pl->T, o.precision, o.recon, o.opsplit, o.mt, o.mf);
}

}  // namespace

// tile chosen earlier by csadv_tune for plans of this shape, or -1
int tuned_tile(int N, int T, const Options &o) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    auto it = g_tune.find(TuneKey(N, T, o.precision, o.recon, o.opsplit, o.mt, o.mf));
    return it == g_tune.end() ? -1 : it->second;
}

void batch_forget(csadv_plan *pl) {
    csadv_batch *b = pl->batch;
    if (!b) return;
    auto it = std::find(b->plans.begin(), b->plans.end(), pl);
    if (it != b->plans.end()) b->plans.erase(it);
    b->dirty = true;
    b->drop_graphs();
    pl->batch = nullptr;
}

void batch_touch(csadv_plan *pl) {
    if (pl->batch) {
        pl->batch->dirty = true;
        pl->batch->drop_graphs();
    }
}

}  // namespace csadv

extern "C" {

int csadv_batch_create(int capacity, csadv_batch **out) {
    if (!out || capacity < 1 || capacity > (1 << 20)) return CSADV_ERR_ARG;
    *out = nullptr;
    csadv_batch *b = new (std::nothrow) csadv_batch();
    if (!b) return CSADV_ERR_OOM;
    if (cudaGetDevice(&b->device) != cudaSuccess) {
        delete b;
        return CSADV_ERR_CUDA;
    }
    b->capacity = capacity;
    b->dsolves = b->mem.alloc<SweepSolve>(2LL * capacity);
    if (!b->mem.ok()) {
        delete b;
        return CSADV_ERR_OOM;
    }
    *out = b;
    return CSADV_OK;
}

int csadv_batch_destroy(csadv_batch *b) {
    if (!b) return CSADV_ERR_ARG;
    delete b;
    return CSADV_OK;
}

int csadv_batch_add(csadv_batch *b, csadv_plan *pl) {
    if (!b || !pl) return CSADV_ERR_ARG;
    if (pl->batch) return pl->batch == b ? CSADV_OK : CSADV_ERR_ARG;
    if ((int)b->plans.size() >= b->capacity) return CSADV_ERR_TOO_LARGE;
    if (!batch_compatible(b, pl)) return CSADV_ERR_UNSUPPORTED;
    b->plans.push_back(pl);
    pl->batch = b;
    b->dirty = true;
    b->drop_graphs();
    return CSADV_OK;
}

int csadv_batch_remove(csadv_batch *b, csadv_plan *pl) {
    if (!b || !pl || pl->batch != b) return CSADV_ERR_ARG;
    batch_forget(pl);
    return CSADV_OK;
}

int csadv_batch_size(const csadv_batch *b, int *n) {
    if (!b || !n) return CSADV_ERR_ARG;
    *n = (int)b->plans.size();
    return CSADV_OK;
}

int csadv_batch_advance(csadv_batch *b, int nsteps, void *stream) {
    if (!b || nsteps < 0) return CSADV_ERR_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (b->plans.empty()) return CSADV_OK;
    cudaEvent_t qe = nullptr;
    if (b->qdepth > 0) {  // the advance `qdepth` calls back has finished before this one is queued
        qe = b->qev[b->qn % b->qdepth];
        if (b->qn >= b->qdepth) CSADV_CUDA(cudaEventSynchronize(qe));
    }
    for (int s = 0; s < nsteps; ++s) {
        if (batch_stale(b)) {
            int rc = batch_rebuild(b, st);
            if (rc) return rc;
        }
        int rc = batch_run_step(b, 1, st);
        if (rc) return rc;
    }
    if (qe) {
        CSADV_CUDA(cudaEventRecord(qe, st));
        b->qn += 1;
    }
    return CSADV_OK;
}

int csadv_batch_set_queue_depth(csadv_batch *b, int depth) {
    if (!b || depth < 0 || depth > 64) return CSADV_ERR_ARG;
    for (auto &e : b->qev) cudaEventDestroy(e);  // (a pending record completes on its own)
    b->qev.clear();
    b->qdepth = 0;
    b->qn = 0;
    for (int k = 0; k < depth; ++k) {
        cudaEvent_t e = nullptr;
        CSADV_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming | cudaEventBlockingSync));
        b->qev.push_back(e);
    }
    b->qdepth = depth;
    return CSADV_OK;
}

int csadv_batch_set_graphs(csadv_batch *b, int enable) {
    if (!b) return CSADV_ERR_ARG;
    b->drop_graphs();
    b->graphs = enable != 0;
    return CSADV_OK;
}

int csadv_batch_set_profiling(csadv_batch *b, int enable) {
    if (!b) return CSADV_ERR_ARG;
    if (enable && !b->pev[0]) {
        CSADV_CUDA(cudaEventCreate(&b->pev[0]));
        CSADV_CUDA(cudaEventCreate(&b->pev[1]));
    }
    b->prof = enable != 0;
    return CSADV_OK;
}

int csadv_batch_reset_stats(csadv_batch *b) {
    if (!b) return CSADV_ERR_ARG;
    b->stats = csadv_stats{};
    return CSADV_OK;
}

int csadv_batch_get_stats(const csadv_batch *b, csadv_stats *out) {
    if (!b || !out) return CSADV_ERR_ARG;
    *out = b->stats;
    out->engine = CSADV_ENGINE_FUSED;
    out->tile = 0;
    size_t bytes = 0;
    for (const csadv_plan *pl : b->plans) bytes += pl->mem.bytes() + (pl->gref ? pl->gref->mem.bytes() : 0);
    out->device_bytes = bytes;
    return CSADV_OK;
}

int csadv_tune(csadv_plan *pl, int reps, void *stream, int *tile_out) {
    if (!pl || reps < 1) return CSADV_ERR_ARG;
    if (!pl->f.on) return CSADV_ERR_UNSUPPORTED;
    cudaStream_t st = (cudaStream_t)stream;
    const TuneKey key = tune_key(pl);
    int best = -1;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tune.find(key);
        if (it != g_tune.end()) best = it->second;
    }
    if (best < 0) {
        cudaEvent_t e0, e1;
        CSADV_CUDA(cudaEventCreate(&e0));
        CSADV_CUDA(cudaEventCreate(&e1));
        float best_ms = 1e30f;
        int rc = CSADV_OK;
        for (int c = 0; c < SWEEP_NTILE_CFG && !rc; ++c) {
            const int tile = FUSED_NTILE_CFG + c;
            rc = fused_set_tile(pl->opt, pl->grid, pl->T, pl->dt, pl->f, tile, st);
            if (!rc) rc = fused_prep_winds(pl->opt, pl->grid, pl->w, pl->dt, pl->f, pl->cur, st);
            // the kernel reads Qbuf[cur] and writes the other buffer: the state does not change
            for (int r = 0; r < reps + 1 && !rc; ++r) {
                if (r == 1) {
                    if (cudaEventRecord(e0, st) != cudaSuccess) rc = CSADV_ERR_CUDA;
                }
                int cur = pl->cur;
                if (!rc) rc = fused_kernel(pl->opt, pl->grid, pl->dt, pl->T, pl->f, cur, st);
            }
            if (!rc && cudaEventRecord(e1, st) == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess) {
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (ms < best_ms) {
                    best_ms = ms;
                    best = tile;
                }
            } else if (!rc) {
                rc = CSADV_ERR_CUDA;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (rc) return rc;
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune[key] = best;
    }
    int rc = fused_set_tile(pl->opt, pl->grid, pl->T, pl->dt, pl->f, best, st);
    if (!rc) rc = fused_prep_winds(pl->opt, pl->grid, pl->w, pl->dt, pl->f, pl->cur, st);
    if (rc) return rc;
    pl->f.rec_ready = true;
    pl->drop_graphs();
    batch_touch(pl);
    if (tile_out) *tile_out = best + 1;
    return CSADV_OK;
}

}  // extern "C"
