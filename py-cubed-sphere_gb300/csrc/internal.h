// Internal (non-ABI) declarations shared by the csadv translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdio>
#include <vector>

#include "../../include/csadv.h"
#include "common.cuh"

namespace csadv {

// Record the first CUDA error and turn it into CSADV_ERR_CUDA.
int cuda_fail(cudaError_t e, const char *what, const char *file, int line);
#define CSADV_CUDA(call)                                                          \
    do {                                                                          \
        cudaError_t _e = (call);                                                  \
        if (_e != cudaSuccess) return ::csadv::cuda_fail(_e, #call, __FILE__, __LINE__); \
    } while (0)

// The library's stream-ordered memory pool of the current device (created on first use; memory
// freed into it stays reserved for the library's next allocations).  Plans and grids allocate
// from it, so that csadv_plan_release can free a plan in the order of a stream instead of
// waiting for the whole device.
cudaMemPool_t device_pool();

// Owner of a plan's device allocations (one allocation per array, freed together): cudaMalloc,
// or, after use_pool(), the library's pool in the order of a stream.
class DeviceArena {
   public:
    void use_pool(cudaMemPool_t pool, cudaStream_t st) {
        pool_ = pool;
        st_ = st;
    }
    // the stream of the next allocations (pool mode)
    void set_stream(cudaStream_t st) { st_ = st; }
    template <class T>
    T *alloc(long long count) {
        if (failed_) return nullptr;
        void *p = nullptr;
        size_t bytes = (size_t)(count > 0 ? count : 1) * sizeof(T);
        const cudaError_t e = pool_ ? cudaMallocFromPoolAsync(&p, bytes, pool_, st_) : cudaMalloc(&p, bytes);
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            failed_ = true;
            return nullptr;
        }
        ptrs_.push_back(p);
        bytes_ += bytes;
        return static_cast<T *>(p);
    }
    bool ok() const { return !failed_; }
    size_t bytes() const { return bytes_; }
    // free in the order of stream s (pool allocations; others with cudaFree)
    void release_on(cudaStream_t s) {
        for (void *p : ptrs_) {
            if (pool_) cudaFreeAsync(p, s);
            else cudaFree(p);
        }
        ptrs_.clear();
        bytes_ = 0;
        failed_ = false;
    }
    // free now: the caller has made sure no work that uses the memory is pending
    void release() { release_on(cudaStreamPerThread); }
    ~DeviceArena() { release(); }

   private:
    std::vector<void *> ptrs_;
    size_t bytes_ = 0;
    bool failed_ = false;
    cudaMemPool_t pool_ = nullptr;
    cudaStream_t st_ = nullptr;
};

struct Options {
    int recon, dp, opsplit, et, mt, mf, vf, precision, engine, tile;
    double wp[4];
};

enum { ET_S72 = 1, ET_PL07 = 2, ET_DG = 3 };
enum { MF_0 = 1, MF_AF = 2, MF_PR = 3 };
enum { SP_AVLT = 1, SP_L04 = 2, SP_PL07 = 3 };
enum { MT_0 = 1, MT_PL07 = 2 };
enum { REC_PPM0 = 1, REC_CW84 = 2, REC_PL07 = 3, REC_L04 = 4 };

// IC parameters (meaning per IC code) and the wind parameters the exact solution needs
struct IcParams {
    double ic[4];
    double wind[4];
};

int validate_options(const csadv_options *o, Options &out);
bool wind_time_dependent(const Options &o);

// grid.cu
int build_grid(int N, DeviceArena &mem, Grid &grid, cudaStream_t st);
std::vector<double> linspace(double start, double stop, int num);

struct SweepSolve;

// Per-tracer scratch of the staged engine (type-erased; element type = real)
struct Scratch {
    void *Qx, *Qy, *qLx, *qRx, *qLy, *qRy, *fx, *fy, *div;
};

// Launch wrappers (defined in the .cu files)
template <class real> int launch_halo_dg(real *F, const Grid &g, cudaStream_t st);
template <class real> int launch_halo_adjacent(real *Qx, real *Qy, const Grid &g, cudaStream_t st);
template <class real>
int launch_halo_dg_tracers(real *F, int T, const Grid &g, const double *corr, const real *greal, cudaStream_t st);
// ghost cells of the input buffers of many solves (work items: solve descriptor, block)
template <class real>
int launch_halo_batch(const SweepSolve *dsolves, const int2 *work, int nwork, cudaStream_t st);
template <class real>
int staged_divergence(const Options &o, const Grid &g, const Winds &w, double dt, real *Q, const Scratch &s,
                      double *partials, int npart, cudaStream_t st);
template <class real>
int staged_update(const Options &o, const Grid &g, double dt, real *Q, const Scratch &s, double *partials,
                  int npart, double *scal, cudaStream_t st);
int staged_partial_count(const Grid &g);

int wind_setup(const Options &o, const Grid &g, Winds &w, DeviceArena &mem, double dt, cudaStream_t st);
// the time step of the device clock (set before the first step)
int wind_set_dt(Winds &w, double dt, cudaStream_t st);
// time-dependent wind of a fused plan as coefficient fields of a time basis, ghost edges
// included (uses u_pu / v_pv as scratch: call before wind_initial)
int wind_basis_setup(const Options &o, const Grid &g, Winds &w, DeviceArena &mem, cudaStream_t st);
// departure-point winds + upwind flags of the step from the basis (line-marching layouts); FP64:
// with the edges' flux coefficients, from the cell records crx / cry
// (part -1: every edge; 0: the x-edges only; 1: the y-edges only; peek: for the clock's next step,
// before the clock ticks)
template <class real, class V>
int wind_step(const Options &o, const Grid &g, const Winds &w, double dt, const real *gpu, const real *gpvT, V *erx,
              V *ery, const void *crx, const void *cry, cudaStream_t st, int part = -1, int peek = 0);
// u_pu, v_pv, u_old, v_old <- the basis at the clock's times (before staged operators run)
int wind_sync(const Options &o, const Grid &g, const Winds &w, cudaStream_t st);
int wind_initial(const Options &o, const Grid &g, Winds &w, cudaStream_t st);
int wind_update(const Options &o, const Grid &g, Winds &w, bool tick, long long k, double t, cudaStream_t st);
int wind_halo(const Options &o, const Grid &g, Winds &w, cudaStream_t st);
int wind_average(const Options &o, const Grid &g, Winds &w, double dt, cudaStream_t st);
// departure-point winds in the state's precision + upwind bits (fused engine), one pass
template <class real>
int wind_avgprep(const Options &o, const Grid &g, const Winds &w, double dt, real *ua, real *va, uint32_t *ub,
                 uint32_t *vb, int wpitch, cudaStream_t st);
int wind_cfl(const Options &o, const Grid &g, const Winds &w, double dt, double *dev_tmp, double &cfl, cudaStream_t st);

// ---------------------------------------------------------------- fused engine state
struct FusedState {
    bool on = false;
    bool settled = true;        // host record: no MF-PR correction is pending in Qbuf[cur]
    int tile = 1;               // 0-3: k_fused (FUSED_TILES), 4-7: k_sweep (SWEEP_TILES[tile - 4])
    void *Qbuf[2] = {nullptr, nullptr};
    double *corr[2] = {nullptr, nullptr};  // [T] pending MF-PR correction of Qbuf[b]
    double *partials = nullptr; // [T][max blocks]
    unsigned int *counter = nullptr;
    void *ua = nullptr, *va = nullptr;     // departure-point winds in the state's precision
    uint32_t *upos = nullptr, *vpos = nullptr;  // upwind flags (1 bit per edge)
    int wpitch = 0;             // 32-bit words per row of the flag arrays
    const void *g_pc = nullptr, *g_pu = nullptr, *g_pv = nullptr;  // metric in the state's precision
    // line-marching kernel (k_sweep): y-edge winds/flags and metric planes transposed,
    // 1/g, and one launch descriptor per buffer parity (device memory)
    bool sweep = false;
    int scfg = 0;               // SWEEP_TILES index
    void *erx = nullptr, *ery = nullptr;  // edge records {wind, +-g} (x natural, y transposed)
    // Pipelined winds (FP32 step kernel with a time-dependent wind): a second record buffer; the
    // step that reads Qbuf[b] reads records b, and while it runs the records of the next step are
    // computed into the other buffer on a second stream.  rec_ready: the records of the step that
    // reads Qbuf[cur] are in place (host record; false after a clock change or a batch step).
    void *erx1 = nullptr, *ery1 = nullptr;
    bool wpipe = false;
    bool rec_ready = false;
    void *rec_x(int b) const { return wpipe && b == 1 ? erx1 : erx; }
    void *rec_y(int b) const { return wpipe && b == 1 ? ery1 : ery; }
    void *crx = nullptr, *cry = nullptr;  // cell records {g, 1/g} (natural, transposed)
    double crec_dtdx = 0.0;  // FP64 AVLT: the cell records hold {g, dtdx / g} for this dt/dx
    const void *gpvT = nullptr;           // y-edge metric transposed
    SweepSolve *dsolve = nullptr;  // [2]
    SweepSolve *dsolve_tr = nullptr;  // [2][T]: the same launches restricted to one tracer each
    int nitems = 0;             // work items of one sweep launch (6 x tiles)
    bool inline_ghosts = false; // k_sweep evaluates the ET-DG ghost cells of its tiles (no ghost kernel)
    double *mass_target = nullptr;  // [T] FP32 + MF-PR: sum(Q g) of each tracer when it was set
    double *anchor_part = nullptr;  // block partials of that sum (k_anchor_mass or the tracer upload)
    unsigned int *anchor_count = nullptr;  // blocks of the tracer upload that have written theirs
    size_t smem = 0;
};

int fused_supported(const Options &o);
int fused_alloc(const Options &o, const Grid &g, int T, DeviceArena &mem, FusedState &f, cudaStream_t st);
// departure-point winds of the step that reads Qbuf[buf] (edge records buffer buf when pipelined)
int fused_prep_winds(const Options &o, const Grid &g, const Winds &w, double dt, FusedState &f, int buf,
                     cudaStream_t st, int part = -1, int peek = 0);
// step kernel with a time-dependent (basis) wind: allocate the second record buffer (the next
// step's records are made while the step kernel runs)
int fused_wind_pipeline(const Options &o, const Grid &g, const Winds &w, DeviceArena &mem, FusedState &f,
                        cudaStream_t st);
// ghost cells of every tracer of Qbuf[cur] (with the pending correction applied)
int fused_ghosts(const Options &o, const Grid &g, int T, FusedState &f, int cur, cudaStream_t st);
// the fused kernel Qbuf[cur] -> Qbuf[1-cur]; cur flips
int fused_kernel(const Options &o, const Grid &g, double dt, int T, FusedState &f, int &cur, cudaStream_t st,
                 cudaEvent_t ev0 = nullptr, cudaEvent_t ev1 = nullptr);
// the line-marching step kernel on tracer t alone, Qbuf[cur] -> Qbuf[1-cur] (cur does not flip):
// the tracers of one step in separate launches, so that the copies of one tracer overlap the
// step of another
int fused_kernel_tracer(const Options &o, int T, const FusedState &f, int cur, int t, cudaStream_t st);
// set the dynamic shared-memory limit of the kernel a plan will launch (outside capture)
int fused_prepare(const Options &o, int tile);
// select the tile configuration of the fused engine (tile code as in csadv_options.tile,
// zero-based); rewrites the sweep descriptors.  Outside stream capture.
int fused_set_tile(const Options &o, const Grid &g, int T, double dt, FusedState &f, int tile, cudaStream_t st);
// the line-marching step kernel over `nwork` items (stream -1: prepare the kernels' shared-memory
// limits only); tgroup (SWEEP_TG_*) is how the FP32 form groups the tracers of the solves
template <class real>
int sweep_launch(int recon, int split, const SweepSolve *dsolves, const int2 *work, int nwork, int grid, size_t smem,
                 cudaStream_t st, int tgroup);
// the FP32 form runs the paired-tracer kernel (sweep2.cuh)
template <>
int sweep_launch<float>(int recon, int split, const SweepSolve *dsolves, const int2 *work, int nwork, int grid,
                        size_t smem, cudaStream_t st, int tgroup);
// edge records of the line-marching kernel from the reference-layout winds (static winds: once)
template <class real, class V>
int wind_avgprep_t(const Options &o, const Grid &g, const Winds &w, double dt, const real *gpu, const real *gpvT,
                   V *erx, V *ery, const void *crx, const void *cry, cudaStream_t st);
// ghost cells of Qbuf[cur] <- those of Qbuf[1-cur] (the halo the last step used), tracers
// first .. first + T - 1
int fused_ghosts_to_current(const Options &o, const Grid &g, int T, FusedState &f, int cur, cudaStream_t st,
                            int first = 0);
// FP32 form with MF-PR: record sum(Q g) of tracer t of Qbuf[cur] (no pending correction) as the
// mass the step's correction restores
int fused_anchor_mass(const Options &o, const Grid &g, FusedState &f, int cur, int t, cudaStream_t st);
// apply and clear the pending MF-PR correction of Qbuf[cur]
int fused_materialize(const Options &o, const Grid &g, int T, FusedState &f, int cur, cudaStream_t st);
template <class real> int fused_launch(const struct FusedArgs &a, int recon, int tile, cudaStream_t st);

int diag_partials(const Grid &g);
template <class real>
int init_tracer(const Grid &g, int ic, int vf, const IcParams &prm, real *Q, cudaStream_t st);
// Optional work of the layout conversion on the fused engine's state (null pointers: none).
//  to the device -- *corr = 0: the tracer's pending MF-PR correction belongs to the field the
//                   upload replaces; with `mass`, sum(Q g) over the interior of the uploaded field
//                   (FP64 products of the stored values), one partial per block in `part`, summed
//                   in block order by the block that finishes last (`count` back to 0)
//  to the host   -- with `corr`, each interior value read out is the true state Q* + g corr
constexpr int IO_B = 128;  // cells per block of the layout conversion
template <class real>
struct IoLazy {
    const real *g = nullptr;  // metric plane in the state's precision
    double *corr = nullptr;   // this tracer's pending correction
    double *part = nullptr;   // [blocks of the conversion]
    unsigned int *count = nullptr;
    double *mass = nullptr;
};
template <class real>
int tracer_io(const Grid &g, real *Q, double *dev_stage, int layout, bool to_native, cudaStream_t st,
              const IoLazy<real> *lazy = nullptr);
template <class real>
int diag_mass(const Grid &g, const real *Q, double *dev_tmp, double &mass, cudaStream_t st);
template <class real>
int diag_errors(const Grid &g, const real *Q, int ic, int vf, const IcParams &prm, double t, double *dev_tmp,
                double out[3], cudaStream_t st);

// device address of a host array: page-locked memory in place, else a stream-ordered copy
struct DevArray {
    void *dev = nullptr;
    bool owned = false;
};
inline int dev_in(const void *host, size_t bytes, cudaStream_t st, DevArray &a) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, host) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer) {
        a.dev = at.devicePointer;
        return CSADV_OK;
    }
    (void)cudaGetLastError();
    CSADV_CUDA(cudaMallocAsync(&a.dev, bytes, st));
    a.owned = true;
    CSADV_CUDA(cudaMemcpyAsync(a.dev, host, bytes, cudaMemcpyHostToDevice, st));
    return CSADV_OK;
}
inline int dev_out(void *host, size_t bytes, cudaStream_t st, DevArray &a) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, host) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer) {
        a.dev = at.devicePointer;
        return CSADV_OK;
    }
    (void)cudaGetLastError();
    CSADV_CUDA(cudaMallocAsync(&a.dev, bytes, st));
    a.owned = true;
    return CSADV_OK;
}
inline int dev_back(void *host, size_t bytes, cudaStream_t st, DevArray &a) {
    if (a.owned) CSADV_CUDA(cudaMemcpyAsync(host, a.dev, bytes, cudaMemcpyDeviceToHost, st));
    return CSADV_OK;
}
inline void dev_free(DevArray &a, cudaStream_t st) {
    if (a.owned && a.dev) cudaFreeAsync(a.dev, st);
    a.dev = nullptr;
}

}  // namespace csadv
