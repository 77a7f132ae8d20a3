/*
 * csadv -- cubed-sphere tracer advection on NVIDIA GB300 (sm_103a).
 *
 * C ABI of the GPU implementation of the advection time step of luanfs/py-cubed-sphere.
 * The reference is pure Python and has no FFI; its seam is a set of Python calls
 * (advection_sphere.py, advection_timestep.py, advection_vars.py, diagnostics.py,
 * errors.py).  Each entry point below names the reference call it replaces.  The Python
 * shim in py-cubed-sphere_gb300/csadv binds these with ctypes and re-exposes the
 * reference's function names and signatures.
 *
 * Conventions
 *  - Every function returns an int status (CSADV_OK == 0, negative on error) and never
 *    exits the process (the reference prints and calls exit(); the Python shim maps the
 *    codes back to the reference's behaviour).
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).  Work is
 *    enqueued on it; functions that return host values synchronise it.
 *  - Host arrays are float64 in the reference layout A[i][j][p] (p fastest), either the
 *    full array with 4 ghost cells per side, shape (N+8, N+8, 6)  (CSADV_LAYOUT_FULL),
 *    or the interior only, shape (N, N, 6)                      (CSADV_LAYOUT_INTERIOR).
 *  - A plan is not thread-safe; use one plan per host thread/stream.
 */
#ifndef CSADV_H
#define CSADV_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status codes */
#define CSADV_OK 0
#define CSADV_ERR_OPTION (-1)      /* unknown option code; reference: print + exit(), advection_ic.py:61-166 */
#define CSADV_ERR_OPTION_PAIR (-2) /* split/metric pair the reference cannot run (UnboundLocalError,
                                      discrete_operators.py:49-73): AVLT/L04 need MT-0, PL07 needs MT-PL07 */
#define CSADV_ERR_ARG (-3)         /* bad argument (NULL, size, tracer index, N < 8 ...) */
#define CSADV_ERR_OOM (-4)         /* device or pinned-host allocation failed */
#define CSADV_ERR_CUDA (-5)        /* a CUDA runtime call failed */
#define CSADV_ERR_NONFINITE (-6)   /* NaN/Inf found in the state */
#define CSADV_ERR_BLOWUP (-7)      /* Linf error > 100; reference: print + exit(), output.py:44-47 */
#define CSADV_ERR_UNSUPPORTED (-8) /* option combination not implemented by the requested engine */
#define CSADV_ERR_TOO_LARGE (-9)   /* request exceeds a fixed capacity */

#define CSADV_LAYOUT_FULL 0
#define CSADV_LAYOUT_INTERIOR 1

/* engines */
#define CSADV_ENGINE_AUTO 0   /* fused when the scheme allows it, else staged */
#define CSADV_ENGINE_STAGED 1 /* one kernel per reference stage; every option combination */
#define CSADV_ENGINE_FUSED 2  /* one tile kernel per step (ET-DG, MF-0/MF-PR) */

/* wind codes: 1-4 are the reference's vf (advection_ic.py:287-313); the others are the
   parameterised benchmark winds (wind_param meaning in brackets) */
#define CSADV_WIND_SOLID 101     /* solid-body rotation [alpha, u0]               (static)  */
#define CSADV_WIND_DEFORM 102    /* Nair-Lauritzen 2010 case 4 [k, T]             (time-dependent) */
#define CSADV_WIND_SOLID_DIV 103 /* solid body + eps*u0 divergent part [alpha, u0, eps] (static) */

/* initial-condition codes: 1-4 are the reference's ic (advection_ic.py:215-281, exact
   solution depends on the wind code exactly as in the reference); the others: */
#define CSADV_IC_HILL 101         /* exp(-b0 |x - xc|^2) [lon_c, lat_c, b0] */
#define CSADV_IC_BELLS 102        /* 0.1 + 0.9 * two cosine bells of radius 1/2 at lon 5pi/6, 7pi/6 */
#define CSADV_IC_SMOOTH_BELLS 103 /* 0.95 + 0.05 * the same bells */

typedef struct csadv_options {
    int recon;     /* advection.par "Reconstruction": 1 PPM-0, 2 PPM-CW84, 3 PPM-PL07, 4 PPM-L04 */
    int dp;        /* "Departure point scheme": 1 RK1, 2 RK2 */
    int opsplit;   /* "Operator splitting": 1 SP-AVLT, 2 SP-L04, 3 SP-PL07 */
    int et;        /* "Edge treatment": 1 ET-S72, 2 ET-PL07, 3 ET-DG */
    int mt;        /* "Metric tensor treatment": 1 MT-0, 2 MT-PL07 */
    int mf;        /* "Mass fixer": 1 MF-0, 2 MF-AF, 3 MF-PR */
    int vf;        /* wind code (see above) */
    int precision; /* 64: state in float64 ("plain form"); 32: state/PPM/fluxes in float32 */
    int engine;    /* CSADV_ENGINE_* */
    int tile;      /* fused engine tile (rows x columns of cells).  Per-edge tile kernel: 1 = 16x58,
                      2 = 32x58, 3 = 16x26, 4 = 32x26.  Line-marching kernel (largest tiles; the N
                      cells of each direction are split into nearly equal tiles no larger):
                      5 = 55x55, 6 = 55x26, 7 = 26x55, 8 = 26x26.  0 = default: the tile csadv_tune
                      chose for this shape, else 5 for N >= 116 and 8 below */
    double wind_param[4];
} csadv_options;

typedef struct csadv_plan csadv_plan;

/* ---------------------------------------------------------------- library */
const char *csadv_version(void);
const char *csadv_status_string(int status);
/* Select the CUDA device used by plans created afterwards on this host thread. */
int csadv_set_device(int device);

/* ---------------------------------------------------------------- plan (one solve) */
/* Replaces cubed_sphere(N, "gnomonic_equiangular", ...) (cs_datastruct.py:25-541),
 * adv_simulation_par(...) (advection_ic.py:21-203) and init_vars_adv (advection_vars.py:19-107):
 * builds the FP64 grid and Lagrange tables on the device, allocates the tracer state and
 * scratch, and computes the t = 0 winds, wind halo and departure-point winds.
 * Tracers start at zero; set them with csadv_init_tracer / csadv_set_tracer.
 * dt > 0 is the time step; dt < 0 asks for the time step whose CFL number (as
 * advection_vars.py:89-98 defines it, from the t = 0 winds) is -dt (csadv_get_dt reads it).
 * Errors: CSADV_ERR_OPTION, CSADV_ERR_OPTION_PAIR, CSADV_ERR_ARG, CSADV_ERR_OOM. */
int csadv_plan_create(int N, double dt, int ntracers, const csadv_options *opt, void *stream,
                      csadv_plan **out);
/* Frees the plan after waiting for all work on its device. */
int csadv_plan_destroy(csadv_plan *plan);
/* Frees the plan without waiting (no reference counterpart: the reference's simulation objects
 * are garbage-collected Python objects; this serves many short-lived plans).  `stream` is the
 * stream of the plan's last work, or one ordered after it: the plan's device memory, and its
 * grid if no other plan shares it, return to the library's memory pool in that stream's order
 * and are reused by later plans.  Detaches the plan from its batch first. */
int csadv_plan_release(csadv_plan *plan, void *stream);
int csadv_get_dt(const csadv_plan *plan, double *dt);

/* q0_adv (advection_ic.py:208-210) evaluated on the device at the interior cell centres
 * (the reference's Q0 is a point value, advection_vars.py:105). */
int csadv_init_tracer(csadv_plan *plan, int tracer, int ic, const double *ic_param, void *stream);
/* simulation.Q = host array  /  host array = simulation.Q
 * The host array is FP64 in the reference's layout.  Page-locked host memory (csadv_host_alloc,
 * cudaMallocHost, cudaHostRegister) is read or written by the device directly, in one pass over
 * the interconnect; pageable memory is staged through a device buffer.  csadv_set_tracer is
 * ordered on the stream: the array must stay unchanged until the stream has passed the call.
 * csadv_get_tracer returns when the array holds the field.  With the fused engine and MF-PR the
 * read-out applies the tracer's pending mass-fixer correction as it reads, and the upload
 * replaces it (and, in FP32, records the uploaded field's sum(Q g) as the mass the fixer keeps);
 * neither touches the other tracers' pending corrections. */
int csadv_set_tracer(csadv_plan *plan, int tracer, const double *host, int layout, void *stream);
int csadv_get_tracer(csadv_plan *plan, int tracer, double *host, int layout, void *stream);

/* adv_time_step(cs_grid, simulation, k, t) (advection_timestep.py:19-43) for every tracer. */
int csadv_time_step(csadv_plan *plan, int k, void *stream);
/* update_adv(cs_grid, simulation, t) (advection_timestep.py:48-75). */
int csadv_update_winds(csadv_plan *plan, double t, void *stream);
/* nsteps iterations of the time loop of adv_sphere (advection_sphere.py:45-57):
 * time step k then update_adv(k*dt), k = current_step+1 ... current_step+nsteps. */
int csadv_advance(csadv_plan *plan, int nsteps, void *stream);
/* The same time loop on a state held in host memory, as the reference keeps it (the numpy
 * arrays that adv_sphere's loop updates, advection_sphere.py:45-57): every tracer t is read from
 * in[t] (layout in_layout, as csadv_set_tracer), nsteps iterations run as csadv_advance runs them,
 * and every tracer is written to out[t] (out_layout, as csadv_get_tracer).  Returns when out[]
 * holds the fields; in or out may be NULL (no upload, no read-out), and in[t] may equal out[t].
 * With the line-marching fused engine the copies run on the copy engines beside the steps: the
 * step kernel is launched once per tracer in the first and the last step, tracer t+1's upload
 * overlaps tracer t's first step and tracer t's read-out overlaps tracer t+1's last step.  The
 * results equal those of csadv_set_tracer, csadv_advance and csadv_get_tracer bit for bit.  The
 * overlap needs page-locked host arrays (csadv_host_alloc, cudaHostRegister); with pageable ones
 * the copies wait for each other.  Other engines run those three calls in turn. */
int csadv_advance_host(csadv_plan *plan, int nsteps, const double *const *in, int in_layout,
                       double *const *out, int out_layout, void *stream);

/* mass_computation (diagnostics.py:14-26): sum over the interior of Q*sqrt(g)*dx*dy, FP64. */
int csadv_mass(csadv_plan *plan, int tracer, double *mass, void *stream);
/* compute_errors(Q, qexact_adv(lon, lat, t)) (errors.py:99-113, advection_ic.py:215-281):
 * out = {Linf, L1, L2}, FP64 reductions.  Returns CSADV_ERR_BLOWUP when Linf > 100
 * (output.py:44-47) after writing out. */
int csadv_errors(csadv_plan *plan, int tracer, int ic, const double *ic_param, double t,
                 double out[3], void *stream);
/* simulation.CFL (advection_vars.py:89-98). */
int csadv_get_cfl(const csadv_plan *plan, double *cfl);
/* number of completed steps */
int csadv_get_step(const csadv_plan *plan, int *k);
/* divergence(cs_grid, simulation) (discrete_operators.py:18-101) of one tracer at the
 * current state, written as an interior (N, N, 6) array; the state is not advanced. */
int csadv_divergence(csadv_plan *plan, int tracer, double *host_div, void *stream);

/* ---------------------------------------------------------------- checkpoint / resume (no counterpart
 * in the reference, which keeps no state between runs) */
/* Sets the step counter to k and the wind clock to time k dt with previous time (k-1) dt (the
 * current and previous winds of per-edge winds likewise): the state k steps of csadv_advance
 * leave.  With the tracers restored by csadv_set_tracer, a saved run continues with the same bits. */
int csadv_set_step(csadv_plan *plan, int k, void *stream);
/* The FP32 form's mass-fixer target of a tracer (the sum of Q g that its MF-PR correction
 * restores, recorded when the tracer was set): read into *get and/or replaced by *set (either
 * may be NULL).  CSADV_ERR_UNSUPPORTED for plans without one (FP64, or no MF-PR). */
int csadv_mass_target(csadv_plan *plan, int tracer, double *get, const double *set, void *stream);

/* ---------------------------------------------------------------- grid file */
/* The arrays of the reference's grid file (save_grid_netcdf4, plot.py:522-660; read back by
 * cubed_sphere, cs_datastruct.py:45-195) for the equiangular grid of N cells per panel edge and
 * 4 ghost layers, computed on the device: kind 0 po (cell corners, (N+9) x (N+9)), 1 pc (centres,
 * (N+8) x (N+8)), 2 pu (x-edges, (N+9) x (N+8)), 3 pv (y-edges, (N+8) x (N+9)).  P[i][j][panel][5]
 * = X, Y, Z, lon, lat (cs_datastruct.py:238-330 with cs_transform.py:41-96); EX, EY the tangent
 * vectors in the same layout (cs_transform.py:245-397: X, Y, Z, then lon = lat = 0 as the
 * reference leaves them).  Any of P, EX, EY may be NULL; host arrays, page-locked ones used in
 * place.  Returns when the outputs are written. */
int csadv_grid_points(int N, int kind, double *P, double *EX, double *EY, void *stream);

/* ---------------------------------------------------------------- lat-lon output (headless plots) */
/* ll2cs (interpolation.py:38-140), equiangular grid of N cells per panel edge: for n points
 * (X, Y, Z) on the unit sphere (a lat-lon grid's sph2cart coordinates, sphgeo.py:18-22), the
 * panel (Lauritzen et al. 2015: the largest |coordinate|, later panels winning ties as the
 * reference's masks do) and the interior cell indices (i, j) in [0, N) of the cell holding each
 * point (inverse gnomonic map, cs_transform.py:101-126, binned as floor((x + pi/4) / dx)).
 * Host arrays; page-locked ones are used in place.  Returns when the outputs are written. */
int csadv_ll2cs(int N, const double *X, const double *Y, const double *Z, long long n, uint32_t *i, uint32_t *j,
                uint32_t *panel, void *stream);
/* nearest_neighbour (interpolation.py:145-150): out[t] = Q[i0 + i[t], j0 + j[t], panel[t]] of one tracer
 * of the plan (its current state, float64).  CSADV_ERR_ARG if an index is out of range (those
 * outputs are NaN).  Returns when out is written. */
int csadv_nearest_neighbour(csadv_plan *plan, int tracer, const uint32_t *i, const uint32_t *j,
                            const uint32_t *panel, long long n, double *out, void *stream);

/* ---------------------------------------------------------------- execution control and statistics */
/* Steps run as CUDA graphs by default: one graph per step kind and buffer parity is
 * captured on first use and replayed on the caller's stream.  enable = 0 launches the
 * kernels directly. */
int csadv_set_graphs(csadv_plan *plan, int enable);
/* Record CUDA events around every launch of the plan's main step kernel (the fused
 * kernel; the whole step for the staged engine) and accumulate their durations in
 * csadv_stats.main_ms.  Profiled steps launch directly (no graph) and synchronise. */
int csadv_set_profiling(csadv_plan *plan, int enable);
/* Where the ET-DG ghost cells of a fused plan come from (interpolation.py:154-314): enable = 1
 * (the default) has the step kernel evaluate the ghost cells of its tiles from the neighbouring
 * panels itself; enable = 0 fills them with a separate ghost-cell launch before each step.  Both
 * give the same bits.  CSADV_ERR_UNSUPPORTED for a plan that does not run the line-marching step
 * kernel.  Outside stream capture. */
int csadv_set_inline_ghosts(csadv_plan *plan, int enable);
typedef struct csadv_stats {
    long long steps;            /* steps advanced */
    long long kernel_launches;  /* kernels launched by steps (graph kernel nodes count once per replay) */
    long long main_launches;    /* timed launches of the main kernel */
    double main_ms;             /* their total device time */
    int kernels_per_step;       /* kernel launches of one step (from the captured graph; 0 if none yet) */
    int engine;                 /* CSADV_ENGINE_STAGED or CSADV_ENGINE_FUSED */
    int tile;                   /* fused tile configuration in use (1..8, as csadv_options.tile), 0 for staged */
    int reserved;
    size_t device_bytes;        /* device memory held by the plan (with its grid, which plans of one N share) */
    long long graph_builds;     /* step graphs captured and instantiated (a batch: one per membership change
                                   and buffer parity) */
    double graph_build_ms;      /* host time spent capturing and instantiating them */
} csadv_stats;
int csadv_get_stats(csadv_plan *plan, csadv_stats *out);
int csadv_reset_stats(csadv_plan *plan);

/* ---------------------------------------------------------------- batches of solves */
/* Replaces the reference's one-solve-at-a-time loop (advection_sphere.py:45-58) when many
 * independent solves run together; no single reference function corresponds.  A batch
 * advances every attached plan by one step per step (adv_time_step + update_adv,
 * advection_timestep.py:19-75) with ONE launch of the step kernel over the tiles of all of
 * them; each plan's ghost-cell and wind work is launched per plan on the same stream, and a
 * step is replayed as a CUDA graph while the membership is unchanged.  Plans must use the
 * fused engine's line-marching kernel (tile 5..8 or the default), one precision and one
 * reconstruction; N, tracer count, wind, dt and tile may differ (CSADV_ERR_UNSUPPORTED
 * otherwise).  A plan keeps its own state, step counter and diagnostics; it gives the same
 * result in a batch as alone.  Destroying an attached plan detaches it. */
typedef struct csadv_batch csadv_batch;
int csadv_batch_create(int capacity, csadv_batch **out);
int csadv_batch_destroy(csadv_batch *batch);
int csadv_batch_add(csadv_batch *batch, csadv_plan *plan);       /* CSADV_ERR_TOO_LARGE when full */
int csadv_batch_remove(csadv_batch *batch, csadv_plan *plan);
int csadv_batch_size(const csadv_batch *batch, int *n);
int csadv_batch_advance(csadv_batch *batch, int nsteps, void *stream);
/* depth > 0: csadv_batch_advance first waits until the call `depth` calls before it has finished
 * on the device, so the host runs at most `depth` calls ahead of the GPU (a serving loop then sees
 * finished solves, and frees their memory, within that many calls); 0 (the default): no wait.
 * CSADV_ERR_ARG outside 0..64. */
int csadv_batch_set_queue_depth(csadv_batch *batch, int depth);
int csadv_batch_set_graphs(csadv_batch *batch, int enable);
/* profiling: steps launch directly and the step kernel is timed (csadv_stats.main_ms) */
int csadv_batch_set_profiling(csadv_batch *batch, int enable);
int csadv_batch_get_stats(const csadv_batch *batch, csadv_stats *out);
int csadv_batch_reset_stats(csadv_batch *batch);

/* Tile autotuner (no reference counterpart): times the step kernel of `plan` with each
 * line-marching tile configuration (`reps` launches each, on `stream`, without changing the
 * plan's state), selects the fastest and remembers it for plans of the same N, tracer count,
 * precision and scheme created later in the process with tile = 0.  *tile_out (optional)
 * receives the chosen csadv_options.tile code. */
int csadv_tune(csadv_plan *plan, int reps, void *stream, int *tile_out);

/* ---------------------------------------------------------------- allocation-free mass fixer */
/* No counterpart in the reference.  The divergence-projection mass fixer (the MF-PR step of
 * divergence, div -= g * sum(div g) / sum(g g) over the interior) applied to caller-owned
 * DEVICE arrays in the reference layout (N+8, N+8, 6) float64: div_in (a divergence),
 * metric (sqrt(g) at the cell centres, cs_grid.metric_tensor_pc), div_out (may equal
 * div_in; non-interior cells are copied).  For callers that cannot call cudaMalloc (a
 * service whose device memory is fully committed, or memory owned by another runtime's
 * pool): it needs no plan and allocates nothing; its reduction scratch is a fixed 98 KB
 * device array inside the library, held by every GPU that loads it until exit.
 * Limit: N <= 2048 (CSADV_ERR_TOO_LARGE beyond).  The first call on a device looks up the
 * scratch's device address; make it before any stream capture.  That address is remembered
 * for the life of the process: it does not survive cudaDeviceReset (or any other teardown
 * of the device's primary context), after which this entry point must not be called again
 * in the process.  Calls that overlap on the GPU share the scratch and race; order them on
 * one stream. */
int csadv_mass_fixer_noalloc(const double *div_in, const double *metric, double *div_out, int N, void *stream);

/* ---------------------------------------------------------------- measurement */
/* No counterpart in the reference.  The FP64 fused multiply-add rate of the current device in
 * flop/s (2 per DFMA): independent dependency chains on every SM, `iters` DFMA per chain, best
 * of three CUDA-event-timed launches on `stream`.  The FP64 step kernel is bound by this pipe
 * on GB300, so its roofline is stated against it.  Synchronises the stream. */
int csadv_fp64_rate(int iters, double *flops_per_s, void *stream);

/* ---------------------------------------------------------------- pinned host memory */
int csadv_host_alloc(void **ptr, size_t bytes);
int csadv_host_free(void *ptr);

#ifdef __cplusplus
}
#endif
#endif /* CSADV_H */
