"""Benchmark of the cubed-sphere advection time step on one GB300 (or N replicas).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl csadv|reference]

Workload (the reference's scheme on the deformational-flow configuration):
  gnomonic equiangular cubed sphere N = 384 (6 x 384^2 cells), two tracers (cosine bells
  0.1 + 0.9 h, and 0.95 + 0.05 h), Nair-Lauritzen case-4 deformational wind (k = 0.48,
  T = 5 in the reference's units: k = 2.4 R / T), PPM-CW84 monotone reconstruction,
  RK2 departure points, AVLT splitting, ET-DG Lagrange ghost cells, MT-0, MF-PR mass
  fixer, dt from CFL 0.5.  One step = both tracers advanced one time step (plus the
  wind update).  Metric: tracer cell-steps per second (6 N^2 x tracers per step).

The headline line is the FP32 form (tracer state, PPM and fluxes in float32; geometry,
winds, Lagrange weights, mass and error sums in float64); the FP64 ("plain") form of the
same workload is reported in the same line.  Timed steps run as CUDA graphs; L2 is
flushed (256 MB write) before every timed step and each step is timed alone with CUDA
events on the launching stream.  N > 1 (torchrun): every rank runs an independent replica
(the solve does not shard; "replicas only"), max time over ranks.

--impl reference times the reference algorithm on the host cores: the CPU oracle (a
numpy restatement of the reference, test infrastructure) advancing independent replicas of
the same workload, one process per core, on a bounded number of steps.
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
METRIC = "tracer cell-steps/s"


def workload_config():
    return {"workload": "deformational flow, N=384 (6x384^2 cells), 2 tracers, PPM-CW84 RK2 AVLT ET-DG MT-0 MF-PR, CFL 0.5",
            "N": N_CELLS, "tracers": NTRACERS, "cells_per_tracer": 6 * N_CELLS * N_CELLS,
            "l2": "flushed (256 MB write) before every timed step", "execution": "CUDA graph per step"}


def dt_for_cfl(make_plan):
    pl = make_plan(1e-3)
    c = pl.cfl
    pl.close()
    return 1e-3 * CFL / c


PROFILE = os.path.join(ROOT, "profiles", "k_sweep2_N384_T2.md")


def profiled(key):
    """A figure of one launch of the step kernel on this workload from the committed ncu summary
    (its `key = value` line, commas allowed); None when absent."""
    try:
        for ln in open(PROFILE):
            if ln.strip().startswith(key + " ="):
                return float(ln.split("=")[1].split()[0].replace(",", ""))
    except (OSError, ValueError):
        pass
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
    res["errors_linf_l1_l2"] = pl.errors(ICS[0], pl.step * dt, tracer=0)
    pl.close()
    return res


def run_e2e(torch, precision, steps, stream, world=1):
    """Through the C ABI with host buffers: per step, upload both tracers from pinned host
    memory (reference layout, full arrays), advance, download both tracers."""
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

    def one_step():
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


# ----------------------------------------------------------------------------- batched and serving legs
BATCH_SOLVES = 256
BATCH_NS = (48, 96, 192, 384, 768)


def batched_requests(n=BATCH_SOLVES, seed=0, steps=200):
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


def run_batched(torch, steps, warmup, stream, hbm):
    """All 256 solves in one batch: one step-kernel launch per step for all of them, tile
    shapes from the autotuner (one probe plan per distinct N and tracer count).  The resident
    state (~10 GB) is far larger than L2, so no flush is needed between steps."""
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
    b = Batch(len(plans))
    for pl in plans:
        b.add(pl)
    b.advance(warmup, stream)
    torch.cuda.synchronize()
    b.reset_stats()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    b.advance(steps, stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / steps
    st = b.stats()
    b.set_profiling(True)
    b.reset_stats()
    b.advance(max(3, steps // 4), stream)
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
            "ms_per_step": round(ms, 4), "kernels_per_step": st["kernels_per_step"],
            "gpu_launches": st["kernel_launches"], "step_kernel_ms": round(kms, 4),
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                         "frac": round(achieved / hbm, 4), "alg_bytes_per_launch": alg},
            "plan_create_s": round(create_s, 2), "tiles": tiles,
            "config": "256 solves, N in {48,96,192,384,768}, 1-3 tracers, solid-body wind at random angles, "
                      "Gaussian hills, CFL 0.5, FP32 (timed: %d of the 200 steps)" % steps}


def run_large(torch, steps, warmup, stream, hbm):
    """N = 1536 (6 x 1536^2 = 14.2 M cells per tracer), 8 FP32 tracers sharing one divergent
    wind (solid body at alpha = pi/4 plus the 0.3 u0 divergent perturbation), CFL 0.7; the
    timed steps are a sample of the 500-step run.  State ~3.6 GB, far above L2."""
    import math
    from csadv import Plan, tune
    N, T = 1536, 8
    kw = dict(vf=103, wind_param=(math.pi / 4, 2 * math.pi / 5, 0.3, 0.0), ntracers=T, precision=32,
              stream=stream, **SCHEME)
    pl = Plan(N, -0.7, **kw)
    for t in range(T):
        lon = -math.pi + 2 * math.pi * t / T
        pl.init_tracer(101, ic_param=(lon, 0.3 * math.sin(3 * t), 5.0, 0.0), tracer=t)
    tile = tune(pl, reps=2, stream=stream)
    m0 = [pl.mass(t) for t in range(T)]
    pl.advance(warmup)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    pl.advance(steps)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / steps
    pl.set_profiling(True)
    pl.reset_stats()
    pl.advance(3)
    pst = pl.stats()
    pl.set_profiling(False)
    kms = pst["main_ms"] / max(1, pst["main_launches"])
    cells = T * 6 * N * N
    alg = 6 * N * N * (T * 2 * 4 + 3 * 4)
    achieved = alg / (kms * 1e-3) / 1e9
    dm = max(abs(pl.mass(t) - m0[t]) / abs(m0[t]) for t in range(T))
    res = {"value": round(cells / (ms * 1e-3), 1), "unit": "tracer cell-steps/s", "ms_per_step": round(ms, 4),
           "step_kernel_ms": round(kms, 4), "tile": tile, "cfl": round(pl.cfl, 4),
           "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                        "frac": round(achieved / hbm, 4), "alg_bytes_per_launch": alg},
           "max_mass_change": float("%.3e" % dm),
           "config": "N=1536, 8 FP32 tracers, solid body + 0.3 u0 divergent wind, CFL 0.7 (timed: %d of the "
                     "500 steps)" % steps}
    pl.close()
    return res


def run_serving(torch, nreq, stream, budget_gb=120.0):
    """The request loop on a seeded Poisson stream (200 req/s; N log-uniform in [32, 1024],
    steps uniform in [50, 2000], 1-4 tracers, solid-body or deformational wind 50/50, FP32,
    120 GB budget), truncated to the first `nreq` requests."""
    from csadv import serve
    reqs = serve.poisson_requests(nreq, rate=200.0, seed=0)
    srv = serve.Server(budget_bytes=budget_gb * 1e9, precision=32, stream=stream)
    _, summ = srv.run(reqs, realtime=True)
    offered = sum(6 * r.N * r.N * r.tracers * r.steps for r in reqs) / max(reqs[-1].arrival, 1e-9)
    return {"requests": summ["requests"], "failed": summ["failed"], "p50_latency_s": round(summ["p50_latency_s"], 3),
            "p99_latency_s": round(summ["p99_latency_s"], 3), "value": round(summ["throughput"], 1),
            "unit": "tracer cell-steps/s", "wall_s": round(summ["wall_s"], 2),
            "offered_load": round(offered, 1), "peak_resident_gb": round(summ["peak_bytes"] / 1e9, 2),
            "budget_gb": budget_gb, "max_mass_change": float("%.3e" % summ["max_mass_change"]),
            "config": "Poisson 200 req/s, N log-uniform [32,1024], steps U[50,2000], 1-4 tracers, "
                      "solid/deformational 50/50, FP32, first %d requests of the seeded stream" % nreq}


def cpu_sample(nsteps):
    """The oracle (numpy restatement of the reference) on this host, one core."""
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
    t0 = time.perf_counter()
    for s in sims:
        solver.run_steps(s, nsteps)
    sec = time.perf_counter() - t0
    return NTRACERS * 6 * N_CELLS * N_CELLS * nsteps / sec


def bench_gpu(args):
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

    with ClockSampler(local) as clk:
        f32 = run_form(torch, 32, args.steps, args.warmup, flush, stream, world)
    f64 = run_form(torch, 64, max(3, args.steps // 5), args.warmup, flush, stream, world)
    e2e_sec, h2d, d2h = run_e2e(torch, 32, max(3, args.steps // 2), stream, world)

    ms, ms64, e2e_sec = max_over_ranks([f32["ms_per_step"], f64["ms_per_step"], e2e_sec], world)
    cells = NTRACERS * 6 * N_CELLS * N_CELLS
    value = job_rate(cells, world, ms)
    if rank != 0:
        return
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    # algorithmic bytes of one fused-kernel launch: per cell T*(read + write Q) + (u_avg, v_avg, g) once
    s_q = 4
    alg = 6 * N_CELLS * N_CELLS * (NTRACERS * 2 * s_q + 3 * 4)
    kms = f32["kernel_ms"]
    achieved = alg / (kms * 1e-3) / 1e9
    roof = {"bound": "hbm", "kernel": "k_sweep2<PPM-CW84, AVLT> (paired-tracer FP32 step kernel)",
            "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s", "frac": round(achieved / hbm, 4),
            "traffic": None, "kernel_ms": round(kms, 5), "alg_bytes_per_launch": alg,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback"}
    tr = profiled("dram_bytes_per_launch")
    roof["traffic"] = int(tr) if tr else None
    # The kernel is bound by instruction issue (DRAM a few percent busy): its warp instructions per
    # launch (ncu, committed summary) over the launch time, against 4 per SM per cycle at the
    # clock sampled during the timed steps.
    inst = profiled("smsp__inst_executed.sum")
    clk_s = clk.summary()
    mhz = clk_s.get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    if inst:
        peak_issue = 152 * 4 * mhz * 1e6
        issue = {"bound": "issue", "achieved": round(inst / (kms * 1e-3) / 1e12, 4), "peak": round(peak_issue / 1e12, 4),
                 "unit": "T warp-inst/s", "frac": round(inst / (kms * 1e-3) / peak_issue, 4),
                 "inst_per_launch": int(inst), "source": "profiles/k_sweep2_N384_T2.md"}
    else:
        issue = None
    line = {
        "metric": METRIC, "value": round(value, 1), "unit": "tracer cell-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 5), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (analytic ICs and winds)",
        "config": dict(workload_config(), parallelism="replicas" if world > 1 else "single GPU"),
        "fp64": {"value": round(job_rate(cells, world, ms64), 1), "ms_per_step": round(ms64, 5),
                 "kernel_ms": round(f64["kernel_ms"], 5), "dtype": "f64"},
        "fp32_over_fp64": round(ms64 / ms, 2),
        "e2e": {"value": round(job_rate(cells, world, e2e_sec * 1e3), 1), "unit": "tracer cell-steps/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(f32["stats"]["kernel_launches"]),
        "kernels_per_step": int(f32["stats"]["kernels_per_step"]),
        "roofline": roof,
        "issue_roofline": issue,
        "clocks": clk_s,
        "errors_fp32_linf_l1_l2_vs_exact": [float("%.4e" % e) for e in f32["errors_linf_l1_l2"]],
    }
    if not args.no_batched:
        line["batched"] = run_batched(torch, args.batched_steps, args.warmup, stream, hbm)
        line["batched"]["vs_fp64_single"] = round(line["batched"]["value"] / line["fp64"]["value"], 2)
    if not args.no_large:
        line["large"] = run_large(torch, args.large_steps, args.warmup, stream, hbm)
    if args.serve_requests > 0:
        line["serving"] = run_serving(torch, args.serve_requests, stream)
    if world == 1 and not args.no_cpu:
        k = 2
        line["cpu_baseline"] = {"value": round(cpu_sample(k), 1), "unit": "tracer cell-steps/s", "cores": 1,
                                "kind": "port", "sample": "oracle, N=384, 2 tracers, %d steps" % k}
    print(json.dumps(line))


# ----------------------------------------------------------------------------- reference arm
def _ref_worker(args):
    nsteps, = args
    return cpu_sample(nsteps)


def bench_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    nsteps = 1
    timed = max(1, min(args.steps, 3))
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        pool.map(_ref_worker, [(1,)] * cores)  # warm-up: imports, grid, first step
        t1 = time.perf_counter()
        rates = []
        for _ in range(timed):
            rates.append(sum(pool.map(_ref_worker, [(nsteps,)] * cores)))
    value = sorted(rates)[len(rates) // 2]
    cells = NTRACERS * 6 * N_CELLS * N_CELLS
    line = {"metric": METRIC, "value": round(value, 1), "unit": "tracer cell-steps/s", "impl": "reference",
            "n_gpus": 0, "steps": timed, "warmup": 1, "ms_per_step": round(cores * cells / value * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (analytic ICs and winds)", "config": workload_config(),
            "cpu_baseline": {"value": round(value, 1), "unit": "tracer cell-steps/s", "cores": cores, "kind": "port",
                             "sample": "oracle (numpy restatement of the reference), N=384, 2 tracers; one independent "
                                       "replica per core, %d step(s) each, median of %d" % (nsteps, timed)},
            "e2e": {"value": round(value, 1), "unit": "tracer cell-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "wall_s": round(time.perf_counter() - t0, 1)}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="csadv", choices=("csadv", "reference"))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-batched", action="store_true", help="skip the 256-solve batched leg")
    ap.add_argument("--batched-steps", type=int, default=20, help="timed steps of the batched leg")
    ap.add_argument("--no-large", action="store_true", help="skip the N=1536, 8-tracer leg")
    ap.add_argument("--large-steps", type=int, default=20, help="timed steps of the N=1536 leg")
    ap.add_argument("--serve-requests", type=int, default=100,
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
