// The plan object behind the C ABI's csadv_plan handle, shared by the plan and batch
// entry points (internal; not part of the ABI).
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <mutex>
#include <vector>

#include "../../include/csadv.h"
#include "common.cuh"
#include "internal.h"

using namespace csadv;

struct csadv_batch;

namespace csadv {
// The FP64 grid of one resolution on one device, shared by every plan of that N (built by
// the first, freed with the last).
struct GridHolder {
    DeviceArena mem;
    Grid grid;
    std::mutex build_mu;  // held while the first plan builds the grid
    bool built = false;
    // events recorded where the work of plans released while others still used the grid ends;
    // the last plan's stream waits for them before the grid is freed
    std::vector<cudaEvent_t> left;
    ~GridHolder() {
        for (cudaEvent_t e : left) cudaEventDestroy(e);
    }
};
}  // namespace csadv

struct csadv_plan {
    Options opt;
    csadv_batch *batch = nullptr;  // the batch the plan is attached to, if any
    int N = 0, T = 0;
    double dt = 0.0;
    DeviceArena mem;
    std::shared_ptr<GridHolder> gref;  // shared grid; `grid` is a copy of its descriptor
    Grid grid;
    Winds w;
    void *Q = nullptr;  // T fields of `real`
    Scratch s{};
    double *partials = nullptr;
    int npart = 0;
    double *scal = nullptr;
    double *stage = nullptr;
    double *tmp = nullptr;
    int k = 0;
    double cfl = 0.0;
    int device = 0;
    FusedState f;  // fused engine (f.on) : Q double-buffered in f.Qbuf[cur]
    int cur = 0;
    // execution: CUDA graphs of one step, keyed by [kind: 0 time step, 1 time step + wind update][parity]
    bool graphs = true;
    cudaStream_t cap = nullptr;
    cudaGraphExec_t gexec[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
    int gkernels[2][2] = {{0, 0}, {0, 0}};
    // second stream and fork/join events of the fused step
    cudaStream_t side = nullptr;
    cudaEvent_t sev[4] = {nullptr, nullptr, nullptr, nullptr};
    // csadv_advance_host: copy streams, the high-priority streams of the split steps and of the
    // upload conversions, events (uploaded[t], converted[t], arrived[t], fork, downloaded, to /
    // from the high-priority stream) and the device staging arrays (full layout, one per tracer
    // and direction)
    cudaStream_t up = nullptr, down = nullptr, hp = nullptr, cv = nullptr;
    std::vector<cudaEvent_t> hev;
    double *hstage = nullptr;
    // profiling of the main kernel
    bool prof = false;
    cudaEvent_t pev[2] = {nullptr, nullptr};
    csadv_stats stats{};
    void drop_graphs() {
        for (auto &row : gexec)
            for (auto &e : row)
                if (e) {
                    cudaGraphExecDestroy(e);
                    e = nullptr;
                }
    }
    ~csadv_plan() {
        drop_graphs();
        if (cap) cudaStreamDestroy(cap);
        if (side) cudaStreamDestroy(side);
        if (up) cudaStreamDestroy(up);
        if (down) cudaStreamDestroy(down);
        if (hp) cudaStreamDestroy(hp);
        if (cv) cudaStreamDestroy(cv);
        for (auto &e : hev)
            if (e) cudaEventDestroy(e);
        for (auto &e : sev)
            if (e) cudaEventDestroy(e);
        for (auto &e : pev)
            if (e) cudaEventDestroy(e);
    }
    size_t esize() const { return opt.precision == 64 ? sizeof(double) : sizeof(float); }
    void *state() const { return f.on ? f.Qbuf[cur] : Q; }
    void *tracer(int t) const { return (char *)state() + (size_t)t * grid.d.field * esize(); }
};

namespace csadv {
// the plan's fused-step work split for batches: per-plan work before the step kernel (ghost
// cells; for time-dependent winds the wind halo and departure-point winds) and after it
// (kind 1: the wind update of the next step); single stream
int plan_pre_step(csadv_plan *pl, cudaStream_t st, bool ghosts = true);
int plan_post_step(csadv_plan *pl, int kind, cudaStream_t st);
int plan_select_device(csadv_plan *pl);
// apply a pending MF-PR correction: the stored state becomes the true state
int plan_settle(csadv_plan *pl, cudaStream_t st);
int graph_kernel_nodes(cudaGraph_t g);
// batch.cu: tile chosen by csadv_tune for plans of this shape (-1: none); detach a plan from
// its batch; mark the plan's batch for a rebuild (its descriptors changed)
int tuned_tile(int N, int T, const Options &o);
void batch_forget(csadv_plan *pl);
void batch_touch(csadv_plan *pl);
}  // namespace csadv
