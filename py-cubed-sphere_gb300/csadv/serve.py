"""Continuous-batching request loop: many advection solves resident on one GPU.

Requests (N, tracer count, step count, wind, Gaussian-hill initial conditions) arrive over
time.  The loop admits them in arrival order while their device memory fits a budget,
attaches each admitted solve to one ``Batch`` (one step-kernel launch per step for all
resident solves, whatever their sizes), advances the batch, and retires a solve as soon as
it has taken its steps: its error norms against the exact solution and its mass change are
read, its memory is released, and the next queued request can take its place.  Requests
that arrive while others are on the GPU join at the next step boundary, so their work
overlaps on the device.

Everything a solve computes depends only on that solve (the step kernel's reductions have
a fixed order per solve), so each result is the same alone and in the mix; the tests check
this bit for bit.

The reference has no counterpart (it runs one solve per process: advection_sphere.py:13-61).
"""
import collections
import dataclasses
import math
import sys
import time

import numpy as np

from . import _lib as L
from .batch import Batch
from .plan import Plan

# the scheme of the serving and batched workloads: monotone PPM (CW84), RK2 departure points,
# AVLT splitting, Lagrange ghost cells, MT-0, divergence-projection mass fixer
SCHEME = dict(recon=2, dp=2, opsplit=1, et=3, mt=1, mf=3)
U0 = 2.0 * math.pi / 5.0   # solid-body speed: one revolution in T = 5 (unit sphere)
DEFORM = (0.48, 5.0, 0.0, 0.0)  # deformational wind: k = 2.4 R / T, period T = 5


@dataclasses.dataclass
class Request:
    rid: int
    N: int
    steps: int
    tracers: int
    wind: str                  # "solid" or "deform"
    arrival: float = 0.0       # seconds after the start of the run
    alpha: float = 0.0         # solid-body rotation angle
    hills: tuple = ()          # per tracer: (lon, lat, width)
    deadline: float = None     # most seconds it may wait for admission (None: no limit)


@dataclasses.dataclass
class Result:
    rid: int
    N: int
    tracers: int
    steps: int
    arrival: float
    admitted: float
    finished: float
    errors: list               # per tracer (Linf, L1, L2) against the exact solution
    mass_change: list          # per tracer, relative
    cell_steps: int
    state: list = None         # per tracer final interior field (keep_state=True)
    error: str = None          # why the request failed (not admitted, or a failed solve); None if served

    @property
    def latency(self):
        return self.finished - self.arrival


def poisson_requests(n, rate, seed=0, n_range=(32, 1024), steps_range=(50, 2000), tracers=(1, 4),
                     width_range=(2.0, 10.0)):
    """A seeded request stream: Poisson arrivals at `rate` per second, N log-uniform in
    n_range, steps uniform in steps_range, tracer count uniform in tracers (inclusive),
    wind solid-body or deformational 50/50, hill centres uniform on the sphere."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n))
    out = []
    lo, hi = math.log(n_range[0]), math.log(n_range[1])
    for i in range(n):
        N = int(round(math.exp(rng.uniform(lo, hi))))
        T = int(rng.integers(tracers[0], tracers[1] + 1))
        hills = []
        for _ in range(T):
            lon = rng.uniform(-math.pi, math.pi)
            lat = math.asin(rng.uniform(-1.0, 1.0))
            hills.append((lon, lat, rng.uniform(*width_range)))
        out.append(Request(rid=i, N=N, steps=int(rng.integers(steps_range[0], steps_range[1] + 1)), tracers=T,
                           wind="solid" if rng.random() < 0.5 else "deform", arrival=float(t[i]),
                           alpha=float(rng.uniform(0.0, math.pi / 2)), hills=tuple(hills)))
    return out


def make_plan(req, precision=32, cfl=0.5, stream=None):
    """The plan of one request, initial conditions set, dt from the CFL number."""
    if req.wind == "solid":
        vf, wp = L.WIND_SOLID, (req.alpha, U0, 0.0, 0.0)
    else:
        vf, wp = L.WIND_DEFORM, DEFORM
    kw = dict(vf=vf, wind_param=wp, ntracers=req.tracers, precision=precision, stream=stream, **SCHEME)
    pl = Plan(req.N, -cfl, **kw)  # dt from the CFL number of the t = 0 wind
    for t, (lon, lat, w) in enumerate(req.hills):
        pl.init_tracer(L.IC_HILL, ic_param=(lon, lat, w, 0.0), tracer=t)
    return pl


def finish(pl, req, mass0):
    """Error norms (vs the exact solution at the final time) and relative mass change."""
    errs, dm = [], []
    t_end = pl.step * pl.dt
    for t, (lon, lat, w) in enumerate(req.hills):
        errs.append(pl.errors(L.IC_HILL, t_end, ic_param=(lon, lat, w, 0.0), tracer=t) if req.wind == "solid"
                    else (float("nan"),) * 3)
        m = pl.mass(t)
        if not (math.isfinite(m) and math.isfinite(mass0[t])):  # whatever the wind: no error norms for
            raise L.CsadvError(L.ERR_NONFINITE, "mass")          # the deformational one
        dm.append(abs(m - mass0[t]) / abs(mass0[t]) if mass0[t] != 0 else abs(m))
    return errs, dm


def plane_elems(N):
    n = N + 8
    return 6 * (n + 1) * ((n + 1 + 31) // 32 * 32)


class Server:
    """The request loop.  budget_bytes bounds the device memory of resident solves.

    With `stream` and `build_stream` given (two non-blocking CUDA streams; `threads` True by
    default then), plans are made and read off the step loop: `builders` threads create the plans
    of admitted requests (grid, winds, initial conditions, on `build_stream`) while the batch
    steps, and a retirement thread reads a finished solve's error norms and mass on `stream`, after
    its last step.  A plan joins the batch at the first step boundary after it is ready; when
    nothing is resident, the requests admitted together are awaited and start together.  A plan
    that has been read out is freed by the loop at once, in the order of `stream`
    (csadv_plan_release: nothing waits for the device), and its memory is reused by the next
    plans from the library's pool.  The loop runs at most `queue_depth` ticks ahead of the GPU
    (csadv_batch_set_queue_depth), so a solve's end is seen, and its memory reused, within that
    many ticks of its last step on the device instead of a full launch queue later.  Without the
    two streams everything runs inline on `stream`.

    Failures stay with their request: a request whose plan cannot be made (bad size, no
    memory), whose state turns non-finite, or that waits past its deadline gets a Result with
    `error` set and no cell-steps; the loop carries on with the others.  Deadlines are checked
    for every queued request at every step boundary, not only for the head of the queue."""

    def __init__(self, budget_bytes, precision=32, cfl=0.5, max_active=512, stream=None, clock=time.perf_counter,
                 keep_state=False, max_steps_per_tick=8, threads=None, build_stream=None, device=None, builders=2,
                 queue_depth=2):
        self.budget = int(budget_bytes)
        self.precision = precision
        self.cfl = cfl
        self.max_active = max_active
        self.stream = stream
        self.build_stream = build_stream
        self.device = device
        self.clock = clock
        self.keep_state = keep_state
        self.max_steps_per_tick = max_steps_per_tick
        self.threads = (stream is not None and build_stream is not None) if threads is None else bool(threads)
        self.builders = builders
        self.queue_depth = queue_depth
        self._coef = {}

    # device bytes of a plan ~ plane elements x (a + b T), per wind kind; measured once
    def estimate(self, req):
        key = req.wind
        if key not in self._coef:
            sizes = []
            for T in (1, 2):
                probe = Request(rid=-1, N=32, steps=1, tracers=T, wind=req.wind, hills=((0.0, 0.0, 5.0),) * T)
                with make_plan(probe, self.precision, self.cfl, self.stream) as pl:
                    sizes.append(pl.stats()["device_bytes"] / plane_elems(32))
            self._coef[key] = (2 * sizes[0] - sizes[1], sizes[1] - sizes[0])
        a, b = self._coef[key]
        return int(plane_elems(req.N) * (a + b * req.tracers) * 1.02) + (1 << 20)

    def _thread_init(self):
        if self.device is not None:
            L.check(L.lib().csadv_set_device(int(self.device)), "csadv_set_device")

    def _build(self, req):
        """The plan of one request with its initial conditions in place (its mass read back, which
        waits for the build stream); its later work runs on the loop's stream."""
        t0 = time.perf_counter()
        stream = self.build_stream if self.threads else self.stream
        pl = make_plan(req, self.precision, self.cfl, stream)
        try:
            mass0 = [pl.mass(t) for t in range(req.tracers)]
            nbytes = pl.stats()["device_bytes"]
        except Exception:
            pl.release()
            raise
        pl.stream = L.stream_handle(self.stream)
        return pl, mass0, nbytes, time.perf_counter() - t0

    def _retire(self, pl, req, admitted, mass0, t0, realtime):
        """Result of a finished solve (error norms, mass change, optionally its fields), read on
        the loop's stream after the solve's last step; then the plan is freed in that stream's
        order (it has left the batch, and every step that used it was queued before)."""
        try:
            errs, dm = finish(pl, req, mass0)  # synchronises the plan's stream
            failed = None
        except L.CsadvError as e:  # e.g. a non-finite state: this request only
            errs, dm, failed = [], [], str(e)
        state = [pl.get_tracer(t) for t in range(req.tracers)] if self.keep_state else None
        fin = self.clock() - t0
        tr = time.perf_counter()
        pl.release(self.stream)
        self._release_s += time.perf_counter() - tr
        res = Result(req.rid, req.N, req.tracers, req.steps, req.arrival if realtime else 0.0, admitted, fin, errs,
                     dm, 0 if failed else 6 * req.N * req.N * req.tracers * req.steps, error=failed)
        res.state = state
        return res

    def run(self, requests, realtime=True, on_step=None):
        """Serve `requests` (sorted by arrival).  realtime: arrivals follow the wall clock;
        otherwise every request is available at once.  Returns (results, summary)."""
        import concurrent.futures as cf
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        queue = collections.deque()
        building = collections.deque()  # [req, future, bytes reserved]
        retiring = []                     # [future of Result, plan, bytes]
        active = {}      # id(plan) -> [plan, req, remaining, admitted, mass0, bytes]
        used = 0
        results = []
        batch = Batch(self.max_active)
        if self.threads:  # finished solves are seen (and their memory freed) within two ticks
            batch.set_queue_depth(self.queue_depth)
        t0 = self.clock()
        steps = 0
        peak = 0
        members_changed = 0
        build_s = 0.0
        self._release_s = 0.0
        advance_s = 0.0
        switch = sys.getswitchinterval()
        if self.threads:  # the loop, builders and retirement hand the interpreter over quickly
            sys.setswitchinterval(min(switch, 2e-4))
        builder = retirer = None
        if self.threads:
            builder = cf.ThreadPoolExecutor(max_workers=self.builders, initializer=self._thread_init)
            retirer = cf.ThreadPoolExecutor(max_workers=1, initializer=self._thread_init)

        def run_inline(fn, *a):
            f = cf.Future()
            try:
                f.set_result(fn(*a))
            except BaseException as e:  # noqa: B902 -- delivered like a worker's exception
                f.set_exception(e)
            return f

        def collect_retired(block=False):  # results of the plans read out and freed
            nonlocal used
            keep = []
            for item in retiring:
                if block or item[0].done():
                    results.append(item[0].result())
                    used -= item[2]
                else:
                    keep.append(item)
            retiring[:] = keep

        try:
            while pending or queue or building or active or retiring:
                now = self.clock() - t0
                while pending and (not realtime or pending[0].arrival <= now):
                    queue.append(pending.popleft())
                collect_retired()
                # admission deadlines, for every queued request
                if any(r.deadline is not None for r in queue):
                    keep = collections.deque()
                    for req in queue:
                        waited = now - (req.arrival if realtime else 0.0)
                        if req.deadline is not None and waited > req.deadline:
                            results.append(self._failed(req, realtime, t0, "not admitted within %.3g s" % req.deadline))
                        else:
                            keep.append(req)
                    queue = keep
                # admission by memory budget, in arrival order: reserve the estimate, build beside the loop
                while queue and len(active) + len(building) < self.max_active:
                    req = queue[0]
                    need = self.estimate(req)
                    if used + need > self.budget and (active or building or retiring):
                        break
                    queue.popleft()
                    used += need
                    fut = builder.submit(self._build, req) if builder else run_inline(self._build, req)
                    building.append([req, fut, need])
                # plans that are ready join the batch at this step boundary
                if building and not active:  # nothing to step: the requests admitted together start together
                    cf.wait([b[1] for b in building], return_when=cf.ALL_COMPLETED)
                still = collections.deque()
                for req, fut, need in building:
                    if not fut.done():
                        still.append([req, fut, need])
                        continue
                    try:
                        pl, mass0, nbytes, bs = fut.result()
                    except L.CsadvError as e:
                        used -= need
                        results.append(self._failed(req, realtime, t0, str(e)))
                        continue
                    build_s += bs
                    used += nbytes - need
                    batch.add(pl)
                    members_changed += 1
                    active[id(pl)] = [pl, req, req.steps, self.clock() - t0, mass0, nbytes]
                building = still
                peak = max(peak, used)
                if not active:
                    if retiring:
                        cf.wait([r[0] for r in retiring], return_when=cf.FIRST_COMPLETED)
                    elif pending and realtime and not queue and not building:
                        time.sleep(max(0.0, min(0.01, pending[0].arrival - (self.clock() - t0))))
                    continue
                k = min(v[2] for v in active.values())
                k = max(1, min(k, self.max_steps_per_tick))
                ta = time.perf_counter()
                batch.advance(k, self.stream)
                advance_s += time.perf_counter() - ta
                steps += k
                if on_step:
                    on_step(steps, len(active), used)
                done = []
                for key, v in active.items():
                    v[2] -= k
                    if v[2] <= 0:
                        done.append(key)
                for key in done:
                    pl, req, _, admitted, mass0, nbytes = active.pop(key)
                    batch.remove(pl)
                    members_changed += 1
                    args = (pl, req, admitted, mass0, t0, realtime)
                    fut = retirer.submit(self._retire, *args) if retirer else run_inline(self._retire, *args)
                    retiring.append([fut, pl, nbytes])
            collect_retired(block=True)
        finally:
            for req, fut, need in building:
                try:
                    fut.result()[0].close()
                except Exception:
                    pass
            for v in active.values():
                v[0].close()
            for item in retiring:
                try:
                    item[0].result()
                except Exception:
                    pass
                item[1].close()
            if builder:
                builder.shutdown(wait=True)
            if retirer:
                retirer.shutdown(wait=True)
            graph_builds, graph_ms = 0, 0.0
            if hasattr(batch, "stats"):
                st = batch.stats()
                graph_builds, graph_ms = st.get("graph_builds", 0), round(st.get("graph_build_ms", 0.0), 1)
            batch.close()
            sys.setswitchinterval(switch)
        wall = self.clock() - t0
        served = [r for r in results if r.error is None]
        lat = np.array([r.latency for r in served]) if served else np.zeros(1)
        cs = sum(r.cell_steps for r in served)
        summary = {"requests": len(served), "failed": len(results) - len(served), "wall_s": wall,
                   "tracer_cell_steps": cs,
                   "throughput": cs / wall if wall > 0 else 0.0,
                   "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
                   "batch_steps": steps, "peak_bytes": peak, "budget_bytes": self.budget,
                   "membership_changes": members_changed, "plan_build_s": round(build_s, 3),
                   "release_s": round(self._release_s, 3), "advance_s": round(advance_s, 3), "graph_builds": graph_builds, "graph_build_ms": graph_ms,
                   "max_mass_change": max((max(r.mass_change) for r in served), default=0.0)}
        return results, summary

    def _failed(self, req, realtime, t0, why):
        now = self.clock() - t0
        return Result(req.rid, req.N, req.tracers, req.steps, req.arrival if realtime else 0.0, now, now, [], [], 0,
                      error=why)
