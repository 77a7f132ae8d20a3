"""Benchmark of the cubed-sphere advection time step on one GB300 (or N replicas).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl csadv|reference]

Workload (the reference's scheme on the deformational-flow configuration):
  gnomonic equiangular cubed sphere N = 384 (6 x 384^2 cells), two tracers (cosine bells
  0.1 + 0.9 h, and 0.95 + 0.05 h), Nair-Lauritzen case-4 deformational wind (k = 0.48,
  T = 5 in the reference's units: k = 2.4 R / T), PPM-CW84 monotone reconstruction,
  RK2 departure points, AVLT splitting, ET-DG Lagrange ghost cells, MT-0, MF-PR mass
  fixer, dt from CFL 0.5.  One step = both tracers advanced one time step (plus the
  wind update).  Metric: tracer cell-steps per second (6 N^2 x tracers per step).

The headline (`value`, `e2e`, `roofline`) is the FP64 ("plain") form, the reference's own
arithmetic, so that it compares like for like with the reference arm.  The FP32 form
(tracer state, PPM and fluxes in float32; geometry, winds, Lagrange weights, mass and error
sums in float64) is the `fp32` sub-object, with its own end-to-end rate and HBM roofline.
Timed steps run as CUDA graphs; L2 is flushed (256 MB write) before every timed step and each
step is timed alone with CUDA events on the launching stream.  `e2e` is the same step through
the C ABI with page-locked host arrays: one `csadv_advance_host` call per step (upload both
tracers, step, read both out, the copies beside the step), and `e2e.separate_calls` the same
work as separate set / advance / get calls.  N > 1 (torchrun): every rank
runs an independent replica (the solve does not shard; "replicas only"), max time over ranks.

Further sub-objects, in the one-GPU job only: `accuracy` (one revolution at N = 48 and the
deformational flow at N = 384 to t = T, FP64 and FP32, error norms against the exact solution),
`batched` (256 solves, 200 steps), `large` (N = 1536, 8 tracers, 500 steps), `serving` (the
Poisson request stream, 10^4 requests: several minutes) and `cpu_baseline` (the oracle on one
host core).

--impl reference times the reference algorithm on the host cores: the CPU oracle (a numpy
restatement of the reference, test infrastructure) advancing one independent replica of the
same workload per core, the same warm-up and timed step counts as the GPU arm, the aggregate
taken over the replicas' common wall-clock window.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "py-cubed-sphere_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

N_CELLS = 384
NTRACERS = 2
SCHEME = dict(recon=2, dp=2, opsplit=1, et=3, mt=1, mf=3)
WIND = 102           # deformational (Nair-Lauritzen 2010 case 4)
WIND_PARAM = (0.48, 5.0, 0.0, 0.0)   # k = 2.4 R / T with R = 1, T = 5
ICS = (102, 103)     # cosine bells; smooth bells
CFL = 0.5
E2E_CALL = ("csadv_advance_host per step (page-locked host arrays: upload both tracers, step, read both out; "
            "separate_calls: csadv_set_tracer x2, csadv_advance, csadv_get_tracer x2)")
METRIC = "tracer cell-steps/s"


def workload_config():
    """The workload only (identical in both arms); how each arm runs it is reported beside."""
    return {"workload": "deformational flow, N=384 (6x384^2 cells), 2 tracers, PPM-CW84 RK2 AVLT ET-DG MT-0 MF-PR, CFL 0.5",
            "N": N_CELLS, "tracers": NTRACERS, "cells_per_tracer": 6 * N_CELLS * N_CELLS,
            "wind": "deformational, k=0.48, T=5 (k = 2.4 R/T)", "ics": "cosine bells; smooth bells"}


def dt_for_cfl(make_plan):
    pl = make_plan(1e-3)
    c = pl.cfl
    pl.close()
    return 1e-3 * CFL / c


PROFILES = {32: os.path.join(ROOT, "profiles", "k_sweep2_N384_T2.md"),
            64: os.path.join(ROOT, "profiles", "k_sweep_f64_N384_T2.md"),
            "rec64": os.path.join(ROOT, "profiles", "k_wind_rec_f64_N384.md")}
# the sources each kernel is compiled from: a committed ncu summary states their digest, and its
# figures are used only while those sources are unchanged
KERNEL_SOURCES = {32: ("sweep2.cuh", "fused.cuh", "halo.cuh", "common.cuh", "tiles.h", "sweep_f32_pairs.cu"),
                  64: ("sweep.cuh", "fused.cuh", "halo.cuh", "common.cuh", "tiles.h", "sweep_f64.cu"),
                  "rec64": ("wind.cu", "common.cuh", "internal.h")}


def kernel_digest(precision):
    import hashlib
    h = hashlib.sha256()
    for name in KERNEL_SOURCES[precision]:
        with open(os.path.join(ROOT, "py-cubed-sphere_gb300", "csrc", name), "rb") as f:
            h.update(name.encode() + b"\0" + f.read())
    return h.hexdigest()[:16]


def profiled(precision, key):
    """A figure of one launch of a step kernel on this workload from the committed ncu summary
    (its `key = value` line, commas allowed).  None when absent, or when the summary was taken
    from other kernel sources than the ones built (its `source_digest` line differs)."""
    vals = {}
    try:
        for ln in open(PROFILES[precision]):
            if "=" in ln:
                k, v = ln.split("=", 1)
                vals[k.strip()] = v.split()[0].replace(",", "") if v.split() else ""
    except OSError:
        return None
    if vals.get("source_digest") != kernel_digest(precision) or key not in vals:
        return None
    try:
        return float(vals[key])
    except ValueError:
        return None


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while active."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sms, mx, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sms.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sms:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sms.sort()
        return {"sm_mhz": sms[len(sms) // 2], "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sms)}


# ----------------------------------------------------------------------------- replicas (N > 1)
def replica_barrier(world, device=None):
    """Barrier across the replicas (N > 1) and a device synchronisation: brackets every timed
    region, so every rank starts and ends its timed steps together."""
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    if device == "cuda":
        import torch
        torch.cuda.synchronize()


def max_over_ranks(values, world, device="cuda"):
    """Each value maximised over the ranks (the job ends with its slowest replica); unchanged
    on one rank.  device: where the collective's tensor lives ("cuda" for NCCL, "cpu" for gloo)."""
    if world <= 1:
        return [float(v) for v in values]
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def job_rate(units_per_step, world, ms_per_step):
    """Whole-job rate: the units all ranks processed per step over the slowest rank's step time."""
    return world * units_per_step / (ms_per_step * 1e-3)


# ----------------------------------------------------------------------------- GPU arm
def run_form(torch, precision, steps, warmup, flush, stream, world=1):
    """Throughput loop (graphs, no host syncs), then a kernel-timing loop (events around the
    main kernel, recorded inside the graph) over the same number of steps."""
    from csadv import Plan

    def make(dt):
        return Plan(N_CELLS, dt, vf=WIND, ntracers=NTRACERS, precision=precision, wind_param=WIND_PARAM,
                    stream=stream, **SCHEME)

    dt = dt_for_cfl(make)
    pl = make(dt)
    for t, ic in enumerate(ICS):
        pl.init_tracer(ic, tracer=t)
    pl.advance(warmup)
    pl.reset_stats()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    replica_barrier(world, "cuda")
    for k in range(steps):
        flush.fill_(k)
        ev[k][0].record(stream)
        pl.advance(1)
        ev[k][1].record(stream)
    replica_barrier(world, "cuda")
    ms = [a.elapsed_time(b) for a, b in ev]
    st = pl.stats()
    pl.set_profiling(True)
    pl.advance(1)  # captures the profiled graph
    pl.reset_stats()
    for k in range(steps):
        flush.fill_(k)
        pl.advance(1)
    torch.cuda.synchronize()
    pst = pl.stats()
    pl.set_profiling(False)
    res = {"dt": dt, "ms_per_step": sum(ms) / steps, "ms_min": min(ms), "stats": st,
           "kernel_ms": pst["main_ms"] / max(pst["main_launches"], 1)}
    pl.close()
    return res


def run_e2e(torch, precision, steps, stream, world=1, one_call=True):
    """Through the C ABI with host buffers: per step, upload both tracers from pinned host
    memory (reference layout, full arrays), advance, download both tracers.  one_call: the
    drop-in call for a host-resident state, csadv_advance_host (the copies on the copy engines
    beside per-tracer step kernels); else csadv_set_tracer, csadv_advance and csadv_get_tracer."""
    import ctypes
    import numpy as np
    from csadv import Plan, _lib

    def make(dt):
        return Plan(N_CELLS, dt, vf=WIND, ntracers=NTRACERS, precision=precision, wind_param=WIND_PARAM,
                    stream=stream, **SCHEME)

    dt = dt_for_cfl(make)
    pl = make(dt)
    n = N_CELLS + 8
    nb_in, nb_out = n * n * 6 * 8, N_CELLS * N_CELLS * 6 * 8
    bufs = []
    for _ in range(NTRACERS):
        pin, pout = ctypes.c_void_p(), ctypes.c_void_p()
        _lib.check(_lib.lib().csadv_host_alloc(ctypes.byref(pin), nb_in))
        _lib.check(_lib.lib().csadv_host_alloc(ctypes.byref(pout), nb_out))
        bufs.append((pin, pout))
    for t, ic in enumerate(ICS):
        pl.init_tracer(ic, tracer=t)
        arr = np.ctypeslib.as_array(ctypes.cast(bufs[t][0], ctypes.POINTER(ctypes.c_double)), shape=(n, n, 6))
        arr[...] = pl.get_tracer(t, full=True)
    L = _lib.lib()
    sh = pl.stream

    ins = (ctypes.c_void_p * NTRACERS)(*[b[0].value for b in bufs])
    outs = (ctypes.c_void_p * NTRACERS)(*[b[1].value for b in bufs])

    def one_step():
        if one_call:
            _lib.check(L.csadv_advance_host(pl._h, 1, ins, _lib.LAYOUT_FULL, outs, _lib.LAYOUT_INTERIOR, sh))
            return
        for t in range(NTRACERS):
            _lib.check(L.csadv_set_tracer(pl._h, t, bufs[t][0], _lib.LAYOUT_FULL, sh))
        _lib.check(L.csadv_advance(pl._h, 1, sh))
        for t in range(NTRACERS):
            _lib.check(L.csadv_get_tracer(pl._h, t, bufs[t][1], _lib.LAYOUT_INTERIOR, sh))

    for _ in range(3):
        one_step()
    replica_barrier(world, "cuda")
    t0 = time.perf_counter()
    for _ in range(steps):
        one_step()
    replica_barrier(world, "cuda")
    sec = (time.perf_counter() - t0) / steps
    for pin, pout in bufs:
        L.csadv_host_free(pin)
        L.csadv_host_free(pout)
    pl.close()
    return sec, NTRACERS * nb_in, NTRACERS * nb_out


# ----------------------------------------------------------------------------- accuracy runs
def steps_to(Plan, N, vf, wp, tf, stream):
    """(nsteps, dt): the fewest whole steps that end exactly at tf with CFL <= 0.5 (the
    reference's CFL definition, advection_vars.py:89-98)."""
    import math
    with Plan(N, -CFL, vf=vf, wind_param=wp, stream=stream, **SCHEME) as pl:
        n = int(math.ceil(tf / pl.dt - 1e-9))
    return n, tf / n


def run_to_end(Plan, N, dt, nsteps, vf, wp, ics, precision, stream):
    """Error norms against the exact solution at the end time (advection_sphere.py:45-61,
    errors.py:99-113), relative mass change and final fields of each tracer."""
    with Plan(N, dt, vf=vf, wind_param=wp, ntracers=len(ics), precision=precision, stream=stream, **SCHEME) as pl:
        for t, (ic, ip) in enumerate(ics):
            pl.init_tracer(ic, ic_param=ip, tracer=t)
        m0 = [pl.mass(t) for t in range(len(ics))]
        t0 = time.perf_counter()
        pl.advance(nsteps)
        q = [pl.get_tracer(t) for t in range(len(ics))]
        wall = time.perf_counter() - t0
        errs = [pl.errors(ic, nsteps * dt, ic_param=ip, tracer=t) for t, (ic, ip) in enumerate(ics)]
        dm = [abs(pl.mass(t) - m0[t]) / abs(m0[t]) for t in range(len(ics))]
    return q, errs, dm, wall


def run_accuracy(stream):
    """Configurations 1 and 2 run to their end times in FP64 and FP32: one revolution of a
    Gaussian hill (b0 = 5 at (0, 0)) in the solid-body wind at alpha = pi/4, N = 48; the cosine
    bells and smooth bells in the deformational wind at N = 384 to t = T, where the exact
    solution is the initial field.  FP32 is also compared with FP64 cell by cell."""
    import math
    import numpy as np
    from csadv import Plan

    def rel(a, b):
        return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))

    out = {}
    cases = (("revolution_N48", 48, 101, (math.pi / 4, 2 * math.pi / 5, 0.0, 0.0), [(101, (0.0, 0.0, 5.0, 0.0))],
              "N=48, Gaussian hill b0=5 at (0,0), solid-body wind alpha=pi/4 u0=2pi/5, one revolution (t=T=5)"),
             ("deformational_N384", N_CELLS, WIND, WIND_PARAM, [(ic, None) for ic in ICS],
              "N=384, cosine bells and smooth bells, deformational wind k=0.48, to t=T=5 (exact = initial field)"))
    for name, N, vf, wp, ics, desc in cases:
        nsteps, dt = steps_to(Plan, N, vf, wp, 5.0, stream)
        r = {}
        for prec in (64, 32):
            r[prec] = run_to_end(Plan, N, dt, nsteps, vf, wp, ics, prec, stream)
        fmt = lambda v: [float("%.6e" % x) for x in v]  # noqa: E731
        out[name] = {
            "config": desc + ", PPM-CW84 RK2 AVLT ET-DG MT-0 MF-PR", "steps": nsteps, "dt": dt,
            "fp64": {"linf_l1_l2": [fmt(e) for e in r[64][1]], "mass_change": [float("%.3e" % d) for d in r[64][2]],
                     "wall_s": round(r[64][3], 3)},
            "fp32": {"linf_l1_l2": [fmt(e) for e in r[32][1]], "mass_change": [float("%.3e" % d) for d in r[32][2]],
                     "wall_s": round(r[32][3], 3),
                     "max_diff_vs_fp64": [float("%.3e" % rel(a, b)) for a, b in zip(r[32][0], r[64][0])],
                     "l2_vs_fp64_l2": [round(a[2] / b[2], 5) for a, b in zip(r[32][1], r[64][1])]},
        }
    return out


# ----------------------------------------------------------------------------- batched and serving legs
BATCH_SOLVES = 256
BATCH_NS = (48, 96, 192, 384, 768)
BATCH_STEPS = 200


def batched_requests(n=BATCH_SOLVES, seed=0, steps=BATCH_STEPS):
    """256 independent FP32 solves: N uniform in {48, 96, 192, 384, 768}, 1-3 tracers of
    Gaussian hills (centres uniform on the sphere, width parameter uniform in [2, 10]),
    solid-body rotation at an angle uniform in [0, pi/2], CFL 0.5, 200 steps."""
    import math
    import numpy as np
    from csadv import serve
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        N = int(rng.choice(BATCH_NS))
        T = int(rng.integers(1, 4))
        hills = tuple((float(rng.uniform(-math.pi, math.pi)), float(math.asin(rng.uniform(-1.0, 1.0))),
                       float(rng.uniform(2.0, 10.0))) for _ in range(T))
        out.append(serve.Request(rid=i, N=N, steps=steps, tracers=T, wind="solid",
                                 alpha=float(rng.uniform(0.0, math.pi / 2)), hills=hills))
    return out


def run_batched(torch, warmup, stream, hbm):
    """All 256 solves in one batch for their 200 steps: one step-kernel launch per step for all
    of them, tile shapes from the autotuner (one probe plan per distinct N and tracer count).
    The first `warmup` steps are untimed, the rest timed as one region.  The resident state
    (~10 GB) is far larger than L2, so no flush is needed between steps.  At the end, each
    solve's error norms against the exact rotated hills and its mass change."""
    import numpy as np
    from csadv import Batch, serve, tune
    reqs = batched_requests()
    tiles = {}
    for key in sorted({(r.N, r.tracers) for r in reqs}):
        probe = next(r for r in reqs if (r.N, r.tracers) == key)
        with serve.make_plan(probe, 32, 0.5, stream) as pl:
            tiles["%dx%d" % key] = tune(pl, reps=3, stream=stream)
    t0 = time.perf_counter()
    plans = [serve.make_plan(r, 32, 0.5, stream) for r in reqs]
    torch.cuda.synchronize()
    create_s = time.perf_counter() - t0
    mass0 = [[pl.mass(t) for t in range(r.tracers)] for pl, r in zip(plans, reqs)]
    b = Batch(len(plans))
    for pl in plans:
        b.add(pl)
    b.advance(warmup, stream)
    torch.cuda.synchronize()
    b.reset_stats()
    timed = BATCH_STEPS - warmup
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    b.advance(timed, stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / timed
    st = b.stats()
    l2, dm = [], []
    for pl, r, m0 in zip(plans, reqs, mass0):
        errs, d = serve.finish(pl, r, m0)
        l2 += [e[2] for e in errs]
        dm += d
    b.set_profiling(True)  # after the 200 steps: these extra steps only time the step kernel
    b.reset_stats()
    b.advance(3, stream)
    pst = b.stats()
    b.set_profiling(False)
    kms = pst["main_ms"] / max(1, pst["main_launches"])
    cells = sum(6 * r.N * r.N * r.tracers for r in reqs)
    alg = sum(6 * r.N * r.N * (r.tracers * 2 * 4 + 3 * 4) for r in reqs)
    b.close()
    for pl in plans:
        pl.close()
    achieved = alg / (kms * 1e-3) / 1e9
    return {"value": round(cells / (ms * 1e-3), 1), "unit": "tracer cell-steps/s", "solves": len(reqs),
            "ms_per_step": round(ms, 4), "timed_steps": timed, "kernels_per_step": st["kernels_per_step"],
            "gpu_launches": st["kernel_launches"], "step_kernel_ms": round(kms, 4),
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                         "frac": round(achieved / hbm, 4), "alg_bytes_per_launch": alg},
            "plan_create_s": round(create_s, 2), "tiles": tiles,
            "l2_error_median_max": [float("%.4e" % np.median(l2)), float("%.4e" % max(l2))],
            "max_mass_change": float("%.3e" % max(dm)),
            "config": "256 solves, N in {48,96,192,384,768}, 1-3 tracers, solid-body wind at random angles, "
                      "Gaussian hills, CFL 0.5, FP32, 200 steps (%d warm-up, %d timed); L2 errors against the "
                      "exact rotated hills at the end" % (warmup, timed)}


LARGE_STEPS = 500


def run_large(torch, warmup, stream, hbm, total=LARGE_STEPS):
    """N = 1536 (6 x 1536^2 = 14.2 M cells per tracer), 8 FP32 tracers sharing one divergent
    wind (solid body at alpha = pi/4 plus the 0.3 u0 divergent perturbation), CFL 0.7, the
    whole 500-step run: `warmup` steps untimed, the rest timed.  State ~3.6 GB, far above L2.
    The divergent wind has no exact solution; mass (MF-PR) and the fields' range are reported."""
    import math
    import numpy as np
    from csadv import Plan, tune
    N, T = 1536, 8
    kw = dict(vf=103, wind_param=(math.pi / 4, 2 * math.pi / 5, 0.3, 0.0), ntracers=T, precision=32,
              stream=stream, **SCHEME)
    pl = Plan(N, -0.7, **kw)
    tile = tune(pl, reps=2, stream=stream)
    for t in range(T):
        lon = -math.pi + 2 * math.pi * t / T
        pl.init_tracer(101, ic_param=(lon, 0.3 * math.sin(3 * t), 5.0, 0.0), tracer=t)
    m0 = [pl.mass(t) for t in range(T)]
    hi0 = max(float(np.max(pl.get_tracer(t))) for t in range(T))
    pl.advance(warmup)
    torch.cuda.synchronize()
    timed = total - warmup
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    pl.advance(timed)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / timed
    dm = max(abs(pl.mass(t) - m0[t]) / abs(m0[t]) for t in range(T))
    q = [pl.get_tracer(t) for t in range(T)]
    pl.set_profiling(True)  # after the 500 steps
    pl.reset_stats()
    pl.advance(3)
    pst = pl.stats()
    pl.set_profiling(False)
    kms = pst["main_ms"] / max(1, pst["main_launches"])
    cells = T * 6 * N * N
    alg = 6 * N * N * (T * 2 * 4 + 3 * 4)
    achieved = alg / (kms * 1e-3) / 1e9
    res = {"value": round(cells / (ms * 1e-3), 1), "unit": "tracer cell-steps/s", "ms_per_step": round(ms, 4),
           "timed_steps": timed, "step_kernel_ms": round(kms, 4), "tile": tile, "cfl": round(pl.cfl, 4),
           "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                        "frac": round(achieved / hbm, 4), "alg_bytes_per_launch": alg},
           "max_mass_change": float("%.3e" % dm),
           "min_max_at_end": [float("%.4e" % min(float(np.min(x)) for x in q)),
                              float("%.4e" % max(float(np.max(x)) for x in q))],
           "max_at_start": float("%.4e" % hi0),
           "config": "N=1536, 8 FP32 tracers, solid body + 0.3 u0 divergent wind, CFL 0.7, %d steps "
                     "(%d warm-up, %d timed)" % (total, warmup, timed)}
    pl.close()
    return res


def run_serving(torch, nreq, stream, budget_gb=120.0):
    """The request loop on a seeded Poisson stream (200 req/s; N log-uniform in [32, 1024],
    steps uniform in [50, 2000], 1-4 tracers, solid-body or deformational wind 50/50, FP32,
    120 GB budget), its first `nreq` requests (the configuration's 10^4 by default)."""
    import numpy as np
    from csadv import serve
    reqs = serve.poisson_requests(nreq, rate=200.0, seed=0)
    # the loop on its own non-blocking streams: plans are built and read out beside the step loop
    srv = serve.Server(budget_bytes=budget_gb * 1e9, precision=32, stream=torch.cuda.Stream(),
                       build_stream=torch.cuda.Stream(), device=torch.cuda.current_device())
    res, summ = srv.run(reqs, realtime=True)
    offered = sum(6 * r.N * r.N * r.tracers * r.steps for r in reqs) / max(reqs[-1].arrival, 1e-9)
    served = [r for r in res if r.error is None]
    wait = np.array([r.admitted - r.arrival for r in served]) if served else np.zeros(1)
    run = np.array([r.finished - r.admitted for r in served]) if served else np.zeros(1)
    out = {"requests": summ["requests"], "failed": summ["failed"], "p50_latency_s": round(summ["p50_latency_s"], 3),
           "p99_latency_s": round(summ["p99_latency_s"], 3),
           "admission_wait_p50_p99_s": [round(float(np.percentile(wait, 50)), 3),
                                        round(float(np.percentile(wait, 99)), 3)],
           "on_gpu_p50_p99_s": [round(float(np.percentile(run, 50)), 3), round(float(np.percentile(run, 99)), 3)],
           "value": round(summ["throughput"], 1), "unit": "tracer cell-steps/s", "wall_s": round(summ["wall_s"], 2),
           "offered_load": round(offered, 1), "peak_resident_gb": round(summ["peak_bytes"] / 1e9, 2),
           "budget_gb": budget_gb, "max_mass_change": float("%.3e" % summ["max_mass_change"]),
           "batch_steps": summ["batch_steps"],
           "config": "Poisson 200 req/s, N log-uniform [32,1024], steps U[50,2000], 1-4 tracers, "
                     "solid/deformational 50/50, FP32, 120 GB budget, %d requests of the seeded stream" % nreq}
    for k in ("membership_changes", "graph_builds", "graph_build_ms", "plan_build_s", "release_s", "advance_s"):
        if k in summ:
            out[k] = summ[k]
    cap = serving_capacity(torch, srv, reqs, budget_gb)
    out["mix_capacity"] = cap
    out["vs_mix_capacity"] = round(summ["throughput"] / cap["value"], 4) if cap["value"] else None
    return out


def serving_capacity(torch, srv, reqs, budget_gb, steps=20, warmup=3):
    """The GPU's throughput on the serving mix with no arrivals or departures: the stream's
    requests in arrival order, admitted by the loop's own estimate up to the budget and its
    resident limit, stepped as one static batch (graph per step; CUDA events on the batch's
    stream).  The served throughput over this is the loop's efficiency."""
    from csadv import Batch, serve
    st = torch.cuda.Stream()
    used, plans = 0, []
    try:
        for r in reqs:
            need = srv.estimate(r)
            if used + need > budget_gb * 1e9 or len(plans) >= srv.max_active:
                break
            plans.append((serve.make_plan(r, 32, srv.cfl, st), r))
            used += need
        cells = sum(6 * r.N * r.N * r.tracers for _, r in plans)
        with Batch(len(plans)) as b:
            for pl, _ in plans:
                b.add(pl)
            b.advance(warmup, st)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            st.synchronize()
            e0.record(st)
            b.advance(steps, st)
            e1.record(st)
            e1.synchronize()
            ms = e0.elapsed_time(e1) / steps
            for pl, _ in plans:
                b.remove(pl)
    finally:
        for pl, _ in plans:
            pl.release(st)
        st.synchronize()
    return {"value": round(cells / (ms * 1e-3), 1), "unit": "tracer cell-steps/s", "solves": len(plans),
            "resident_gb": round(used / 1e9, 2), "ms_per_step": round(ms, 4), "timed_steps": steps,
            "solid_fraction": round(sum(r.wind == "solid" for _, r in plans) / max(len(plans), 1), 3)}


def oracle_replica():
    """The oracle (numpy restatement of the reference) on the bench workload: both tracers'
    simulations on one grid, dt from CFL 0.5 as the GPU arm chooses it."""
    from oracle import cases, solver
    from oracle.grid import CubedSphere
    g = CubedSphere(N_CELLS)
    wind = cases.WindSpec("deform", k=WIND_PARAM[0], T=WIND_PARAM[1])
    it = g.interior
    probe = solver.Simulation(g, 1e-3, 5.0, 2, 2, *SCHEME.values(), wind=wind, q0=0.0)
    dt = 1e-3 * CFL / probe.CFL
    sims = []
    for ic in ("bells", "smooth_bells"):
        spec = cases.ICSpec(ic)
        q0 = spec(g.pc.lon[it], g.pc.lat[it])
        sims.append(solver.Simulation(g, dt, 5.0, 2, 2, *SCHEME.values(), ic_spec=spec, wind=wind, q0=q0))
    return sims


def oracle_steps(sims, nsteps, k0=1):
    from oracle import solver
    for s in sims:
        solver.run_steps(s, nsteps, k0)


def cpu_sample(nsteps):
    """The oracle on this host, one core: tracer cell-steps/s over `nsteps` steps."""
    sims = oracle_replica()
    t0 = time.perf_counter()
    oracle_steps(sims, nsteps)
    sec = time.perf_counter() - t0
    return NTRACERS * 6 * N_CELLS * N_CELLS * nsteps / sec


def peaks_file():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def fp64_roofline(step_ms, kms, fp64_flops, hbm):
    """The FP64 step against the FP64 pipe.  Its two FP64 kernels, the step kernel and the next
    step's edge records (on a second stream, beside it), are both bound by the FP64 pipe, so the
    step is the unit: the FP64 arithmetic instructions (DFMA + DADD + DMUL, each one issue of the
    pipe) that the two execute per step, from the committed ncu summaries of these kernels on this
    workload (used only while their sources are unchanged), over the CUDA-event step time, against
    this GPU's DFMA issue rate measured here (csadv_fp64_rate / 2).  `kernel_ms` is the step
    kernel's own CUDA-event time, with the records running beside it."""
    alg = 6 * N_CELLS * N_CELLS * (NTRACERS * 2 * 8 + 3 * 8)
    inst_s, inst_r = profiled(64, "fp64_inst_per_launch"), profiled("rec64", "fp64_inst_per_launch")
    inst = inst_s + inst_r if inst_s and inst_r else None
    hbm_gbs = alg / (step_ms * 1e-3) / 1e9
    peak = fp64_flops / 2.0
    roof = {"bound": "fp64", "kernel": "k_sweep<double, PPM-CW84, AVLT> + k_wind_rec<double> (the FP64 step)",
            "unit": "T FP64 inst/s", "peak": round(peak / 1e12, 4),
            "peak_source": "csadv_fp64_rate (DFMA chains on every SM, measured here) / 2 flop per DFMA",
            "achieved": None, "frac": None, "step_ms": round(step_ms, 5), "kernel_ms": round(kms, 5),
            "fp64_inst_per_step": inst, "fp64_inst_step_kernel": inst_s, "fp64_inst_records": inst_r,
            "traffic": None, "alg_bytes_per_step": alg, "hbm_gbs": round(hbm_gbs, 1),
            "hbm_frac": round(hbm_gbs / hbm, 4)}
    tr_s, tr_r = profiled(64, "dram_bytes_per_launch"), profiled("rec64", "dram_bytes_per_launch")
    roof["traffic"] = int(tr_s + tr_r) if tr_s and tr_r else None
    if inst and peak:
        roof["achieved"] = round(inst / (step_ms * 1e-3) / 1e12, 4)
        roof["frac"] = round(inst / (step_ms * 1e-3) / peak, 4)
    else:
        roof["note"] = "no ncu summary for the current kernel sources: executed FP64 instructions unknown"
    return roof


def fp32_roofline(kms, hbm, peaks, mhz):
    """The FP32 step kernel against HBM (algorithmic bytes over its CUDA-event launch time) and,
    since it is bound by instruction issue, its warp instructions per launch (committed ncu
    summary, current sources only) against 4 per SM per cycle at the sampled clock."""
    alg = 6 * N_CELLS * N_CELLS * (NTRACERS * 2 * 4 + 3 * 4)
    achieved = alg / (kms * 1e-3) / 1e9
    roof = {"bound": "hbm", "kernel": "k_sweep2<PPM-CW84, AVLT> (paired-tracer FP32 step kernel)",
            "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s", "frac": round(achieved / hbm, 4),
            "traffic": None, "kernel_ms": round(kms, 5), "alg_bytes_per_launch": alg,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback"}
    tr = profiled(32, "dram_bytes_per_launch")
    roof["traffic"] = int(tr) if tr else None
    inst = profiled(32, "smsp__inst_executed.sum")
    issue = None
    if inst:
        peak_issue = 152 * 4 * mhz * 1e6
        issue = {"bound": "issue", "achieved": round(inst / (kms * 1e-3) / 1e12, 4),
                 "peak": round(peak_issue / 1e12, 4), "unit": "T warp-inst/s",
                 "frac": round(inst / (kms * 1e-3) / peak_issue, 4), "inst_per_launch": int(inst),
                 "thread_inst_per_tracer_cell_step": profiled(32, "thread_inst_per_tracer_cell_step"),
                 "source": "profiles/k_sweep2_N384_T2.md"}
    return roof, issue


def bench_gpu(args):
    import ctypes
    import torch
    import __graft_entry__
    __graft_entry__.build()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from csadv import _lib
    _lib.check(_lib.lib().csadv_set_device(local))
    stream = torch.cuda.current_stream()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2 (129 MB)
    if args.large_only:  # profiling aid: the N=1536 leg alone, `--large-steps` steps
        peaks = peaks_file()
        print(json.dumps({"large": run_large(torch, args.warmup, stream, peaks.get("hbm_gbs", 6800.0),
                                             args.large_steps)}))
        return

    with ClockSampler(local) as clk:
        f64 = run_form(torch, 64, args.steps, args.warmup, flush, stream, world)
        f32 = run_form(torch, 32, args.steps, args.warmup, flush, stream, world)
    e64_sec, h2d64, d2h64 = run_e2e(torch, 64, max(3, args.steps // 2), stream, world)
    e32_sec, h2d32, d2h32 = run_e2e(torch, 32, max(3, args.steps // 2), stream, world)
    s64_sec = run_e2e(torch, 64, max(3, args.steps // 2), stream, world, one_call=False)[0]
    s32_sec = run_e2e(torch, 32, max(3, args.steps // 2), stream, world, one_call=False)[0]
    rate = ctypes.c_double()
    _lib.check(_lib.lib().csadv_fp64_rate(512, ctypes.byref(rate), _lib.stream_handle(stream)), "csadv_fp64_rate")

    ms64, ms32, e64_sec, e32_sec, s64_sec, s32_sec = max_over_ranks(
        [f64["ms_per_step"], f32["ms_per_step"], e64_sec, e32_sec, s64_sec, s32_sec], world)
    cells = NTRACERS * 6 * N_CELLS * N_CELLS
    if rank != 0:
        return
    peaks = peaks_file()
    hbm = peaks.get("hbm_gbs", 6800.0)
    clk_s = clk.summary()
    mhz = clk_s.get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    roof64 = fp64_roofline(ms64, f64["kernel_ms"], rate.value, hbm)
    roof32, issue32 = fp32_roofline(f32["kernel_ms"], hbm, peaks, mhz)
    v64, v32 = job_rate(cells, world, ms64), job_rate(cells, world, ms32)
    line = {
        "metric": METRIC, "value": round(v64, 1), "unit": "tracer cell-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms64, 5), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (analytic ICs and winds)",
        "config": workload_config(),
        "timing": {"l2": "flushed (256 MB write) before every timed step", "execution": "CUDA graph per step",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": round(job_rate(cells, world, e64_sec * 1e3), 1), "unit": "tracer cell-steps/s",
                "h2d_bytes_per_step": h2d64, "d2h_bytes_per_step": d2h64, "call": E2E_CALL,
                "separate_calls": round(job_rate(cells, world, s64_sec * 1e3), 1)},
        "gpu_launches": int(f64["stats"]["kernel_launches"]),
        "kernels_per_step": int(f64["stats"]["kernels_per_step"]),
        "roofline": roof64,
        "clocks": clk_s,
        "fp32": {"value": round(v32, 1), "unit": "tracer cell-steps/s", "dtype": "f32", "ms_per_step": round(ms32, 5),
                 "kernel_ms": round(f32["kernel_ms"], 5), "vs_fp64": round(ms64 / ms32, 2),
                 "gpu_launches": int(f32["stats"]["kernel_launches"]),
                 "kernels_per_step": int(f32["stats"]["kernels_per_step"]),
                 "e2e": {"value": round(job_rate(cells, world, e32_sec * 1e3), 1), "unit": "tracer cell-steps/s",
                         "h2d_bytes_per_step": h2d32, "d2h_bytes_per_step": d2h32, "call": E2E_CALL,
                         "separate_calls": round(job_rate(cells, world, s32_sec * 1e3), 1)},
                 "roofline": roof32, "issue_roofline": issue32},
    }
    # the single-GPU legs (accuracy runs, batch, N=1536, serving) run in the one-GPU job only: under
    # torchrun the other ranks have finished, and their GPUs would wait for rank 0
    single = world == 1
    if single and not args.no_accuracy:
        line["accuracy"] = run_accuracy(stream)
    if single and not args.no_batched:
        line["batched"] = run_batched(torch, args.warmup, stream, hbm)
        line["batched"]["vs_fp64_single"] = round(line["batched"]["value"] / v64, 2)
    if single and not args.no_large:
        line["large"] = run_large(torch, args.warmup, stream, hbm, args.large_steps)
    if single and args.serve_requests > 0:
        line["serving"] = run_serving(torch, args.serve_requests, stream)
    if world == 1 and not args.no_cpu:
        k = 2
        line["cpu_baseline"] = {"value": round(cpu_sample(k), 1), "unit": "tracer cell-steps/s", "cores": 1,
                                "kind": "port", "sample": "oracle (numpy restatement of the reference, FP64), "
                                                          "N=384, 2 tracers, %d steps on one core" % k}
    print(json.dumps(line))


# ----------------------------------------------------------------------------- reference arm
def _ref_replica(warmup, steps, barrier, results):
    """One replica on one core: build, `warmup` steps, then the `steps` timed steps between two
    barriers shared by all replicas; reports its window on the system-wide monotonic clock."""
    sims = oracle_replica()
    oracle_steps(sims, warmup)
    barrier.wait()
    t0 = time.monotonic()
    oracle_steps(sims, steps, warmup + 1)
    t1 = time.monotonic()
    barrier.wait()
    results.put((t0, t1))


def bench_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(cores)
    results = ctx.Queue()
    t_start = time.perf_counter()
    procs = [ctx.Process(target=_ref_replica, args=(args.warmup, args.steps, barrier, results)) for _ in range(cores)]
    for p in procs:
        p.start()
    windows = [results.get() for _ in procs]
    for p in procs:
        p.join()
    window = max(w[1] for w in windows) - min(w[0] for w in windows)
    cells = NTRACERS * 6 * N_CELLS * N_CELLS
    value = cores * cells * args.steps / window
    line = {"metric": METRIC, "value": round(value, 1), "unit": "tracer cell-steps/s", "impl": "reference",
            "n_gpus": 0, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(window / args.steps * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (analytic ICs and winds)", "config": workload_config(),
            "timing": {"execution": "oracle (numpy restatement of the reference), one independent replica per host "
                                    "core, all replicas' timed steps inside one common wall-clock window"},
            "cpu_baseline": {"value": round(value, 1), "unit": "tracer cell-steps/s", "cores": cores, "kind": "port",
                             "sample": "oracle (numpy restatement of the reference, FP64), N=384, 2 tracers; %d "
                                       "replicas (one per core), %d warm-up + %d timed steps each; cells of all "
                                       "replicas over the window from the first start to the last end"
                                       % (cores, args.warmup, args.steps)},
            "e2e": {"value": round(value, 1), "unit": "tracer cell-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "wall_s": round(time.perf_counter() - t_start, 1)}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="csadv", choices=("csadv", "reference"))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the runs to the end times")
    ap.add_argument("--no-batched", action="store_true", help="skip the 256-solve batched leg")
    ap.add_argument("--no-large", action="store_true", help="skip the N=1536, 8-tracer leg")
    ap.add_argument("--large-only", action="store_true", help="run only the N=1536 leg (profiling aid)")
    ap.add_argument("--large-steps", type=int, default=LARGE_STEPS, help="steps of the N=1536 run")
    ap.add_argument("--serve-requests", type=int, default=10000,
                    help="run the serving leg on the first N requests of the seeded stream (0: skip)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        bench_reference(args)
    else:
        bench_gpu(args)


if __name__ == "__main__":
    main()
