"""Object wrapper over one csadv plan (one solve: grid + winds + tracers on the GPU)."""
import ctypes
import weakref

import numpy as np

from . import _lib as L


def host_array(shape):
    """A zeroed FP64 numpy array in page-locked host memory (csadv_host_alloc), freed when the
    last array that uses it is collected.  The tracer copies read and write such arrays in place
    (Plan.set_tracer, get_tracer, advance_host), and advance_host overlaps their copies with the
    steps."""
    count = max(int(np.prod(shape)), 1)
    ptr = ctypes.c_void_p()
    L.check(L.lib().csadv_host_alloc(ctypes.byref(ptr), count * 8), "csadv_host_alloc")
    cbuf = (ctypes.c_double * count).from_address(ptr.value)
    weakref.finalize(cbuf, L.lib().csadv_host_free, ptr.value)
    arr = np.ctypeslib.as_array(cbuf)[:int(np.prod(shape))].reshape(shape)
    arr[...] = 0.0
    return arr


class Plan:
    """A solve resident on the GPU.

    ``dt`` > 0 is the time step; ``dt`` < 0 asks for the time step of CFL number -dt.
    Parameters mirror the reference's ``adv_simulation_par`` option codes (advection.par):
    recon 1-4, dp 1-2, opsplit 1-3, et 1-3, mt 1-2, mf 1-3, and ``vf`` (reference wind
    codes 1-4 or the benchmark winds 101-103 with ``wind_param``).  ``precision`` is 64
    (plain form) or 32 (state, PPM and fluxes in float32).
    """

    def __init__(self, N, dt, recon=3, dp=1, opsplit=1, et=3, mt=1, mf=3, vf=1, ntracers=1, precision=64,
                 engine=L.ENGINE_AUTO, wind_param=(0.0, 0.0, 0.0, 0.0), stream=None, tile=0):
        self.N, self.dt, self.ntracers, self.precision = int(N), float(dt), int(ntracers), int(precision)
        self.options = dict(recon=recon, dp=dp, opsplit=opsplit, et=et, mt=mt, mf=mf, vf=vf)
        self.stream = L.stream_handle(stream)
        o = L.Options()
        o.recon, o.dp, o.opsplit, o.et, o.mt, o.mf, o.vf = recon, dp, opsplit, et, mt, mf, vf
        o.precision, o.engine, o.tile = precision, engine, tile
        for c in range(4):
            o.wind_param[c] = float(wind_param[c]) if c < len(wind_param) else 0.0
        self._opts = o
        self.inline_ghosts = None  # the form's default until set_inline_ghosts is called
        h = ctypes.c_void_p()
        L.check(L.lib().csadv_plan_create(self.N, self.dt, self.ntracers, ctypes.byref(o), self.stream,
                                          ctypes.byref(h)), "csadv_plan_create")
        self._h = h
        if self.dt < 0:  # -dt was a CFL target: read the time step chosen
            v = ctypes.c_double()
            L.check(L.lib().csadv_get_dt(self._h, ctypes.byref(v)), "csadv_get_dt")
            self.dt = v.value

    # ------------------------------------------------------------------ lifecycle
    def close(self):
        """Free the plan after all work on its device has finished."""
        if getattr(self, "_h", None) and self._h.value:
            L.lib().csadv_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def release(self, stream=None):
        """Free the plan without waiting: its device memory returns to the library's pool in the
        order of ``stream`` (the stream of its last work, or one ordered after it; default: the
        plan's own stream) and is reused by later plans.  Detaches it from its batch."""
        if getattr(self, "_h", None) and self._h.value:
            st = self.stream if stream is None else L.stream_handle(stream)
            L.check(L.lib().csadv_plan_release(self._h, st), "csadv_plan_release")
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ------------------------------------------------------------------ state
    @property
    def n(self):
        return self.N + 8

    def init_tracer(self, ic, ic_param=None, tracer=0):
        prm = None
        if ic_param is not None:
            arr = (ctypes.c_double * 4)(*([float(x) for x in ic_param] + [0.0] * (4 - len(ic_param))))
            prm = ctypes.cast(arr, ctypes.POINTER(ctypes.c_double))
        L.check(L.lib().csadv_init_tracer(self._h, tracer, int(ic), prm, self.stream), "csadv_init_tracer")

    def set_tracer(self, Q, tracer=0):
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        if Q.shape == (self.n, self.n, 6):
            layout = L.LAYOUT_FULL
        elif Q.shape == (self.N, self.N, 6):
            layout = L.LAYOUT_INTERIOR
        else:
            raise ValueError("Q must have shape (N+8, N+8, 6) or (N, N, 6)")
        L.check(L.lib().csadv_set_tracer(self._h, tracer, Q.ctypes.data, layout, self.stream), "csadv_set_tracer")

    def get_tracer(self, tracer=0, full=False, out=None):
        shp = (self.n, self.n, 6) if full else (self.N, self.N, 6)
        if out is None:
            out = np.empty(shp, dtype=np.float64)
        L.check(L.lib().csadv_get_tracer(self._h, tracer, out.ctypes.data,
                                         L.LAYOUT_FULL if full else L.LAYOUT_INTERIOR, self.stream),
                "csadv_get_tracer")
        return out

    # ------------------------------------------------------------------ stepping
    def time_step(self, k):
        L.check(L.lib().csadv_time_step(self._h, int(k), self.stream), "csadv_time_step")

    def update_winds(self, t):
        L.check(L.lib().csadv_update_winds(self._h, float(t), self.stream), "csadv_update_winds")

    def advance(self, nsteps):
        L.check(L.lib().csadv_advance(self._h, int(nsteps), self.stream), "csadv_advance")

    def advance_host(self, nsteps, Q_in=None, Q_out=None, full_out=False):
        """csadv_advance_host: `nsteps` steps of a state held in host memory.  Q_in: one FP64
        array per tracer, (N+8, N+8, 6) or (N, N, 6), uploaded first (None: keep the device
        state); Q_out: one array per tracer to write at the end, or True for new arrays of the
        full (full_out) or interior shape, or None for no read-out.  Page-locked arrays
        (host_array) let the copies overlap the steps.  Returns the output arrays (or None)."""
        T = self.ntracers
        in_ptrs = out_ptrs = None
        lin = lout = L.LAYOUT_INTERIOR
        keep = []
        if Q_in is not None:
            if len(Q_in) != T:
                raise ValueError("Q_in needs one array per tracer")
            shp = {np.shape(q) for q in Q_in}
            if len(shp) != 1 or shp.pop() not in ((self.n, self.n, 6), (self.N, self.N, 6)):
                raise ValueError("every Q_in array must have shape (N+8, N+8, 6) or (N, N, 6)")
            arrs = [np.ascontiguousarray(q, dtype=np.float64) for q in Q_in]
            keep += arrs
            lin = L.LAYOUT_FULL if arrs[0].shape[0] == self.n else L.LAYOUT_INTERIOR
            in_ptrs = (ctypes.c_void_p * T)(*[a.ctypes.data for a in arrs])
        if Q_out is True:
            shp = (self.n, self.n, 6) if full_out else (self.N, self.N, 6)
            Q_out = [np.empty(shp, dtype=np.float64) for _ in range(T)]
        if Q_out is not None:
            if len(Q_out) != T:
                raise ValueError("Q_out needs one array per tracer")
            shapes = {q.shape for q in Q_out}
            ok = all(q.dtype == np.float64 and q.flags.c_contiguous for q in Q_out)
            if not ok or len(shapes) != 1 or shapes.pop() not in ((self.n, self.n, 6), (self.N, self.N, 6)):
                raise ValueError("Q_out arrays must be C-contiguous FP64 of shape (N+8, N+8, 6) or (N, N, 6)")
            lout = L.LAYOUT_FULL if Q_out[0].shape[0] == self.n else L.LAYOUT_INTERIOR
            out_ptrs = (ctypes.c_void_p * T)(*[q.ctypes.data for q in Q_out])
        L.check(L.lib().csadv_advance_host(self._h, int(nsteps), in_ptrs, lin, out_ptrs, lout, self.stream),
                "csadv_advance_host")
        del keep
        return Q_out

    @property
    def step(self):
        k = ctypes.c_int()
        L.check(L.lib().csadv_get_step(self._h, ctypes.byref(k)))
        return k.value

    @property
    def cfl(self):
        c = ctypes.c_double()
        L.check(L.lib().csadv_get_cfl(self._h, ctypes.byref(c)))
        return c.value

    # ------------------------------------------------------------------ diagnostics
    def mass(self, tracer=0):
        m = ctypes.c_double()
        L.check(L.lib().csadv_mass(self._h, tracer, ctypes.byref(m), self.stream), "csadv_mass")
        return m.value

    def errors(self, ic, t, ic_param=None, tracer=0, raise_blowup=False):
        out = (ctypes.c_double * 3)()
        prm = None
        if ic_param is not None:
            arr = (ctypes.c_double * 4)(*([float(x) for x in ic_param] + [0.0] * (4 - len(ic_param))))
            prm = ctypes.cast(arr, ctypes.POINTER(ctypes.c_double))
        rc = L.lib().csadv_errors(self._h, tracer, int(ic), prm, float(t), out, self.stream)
        if rc not in (L.OK, L.ERR_BLOWUP) or (rc == L.ERR_BLOWUP and raise_blowup):
            L.check(rc, "csadv_errors")
        return out[0], out[1], out[2]

    # ------------------------------------------------------------------ execution control
    def set_graphs(self, enable):
        L.check(L.lib().csadv_set_graphs(self._h, int(bool(enable))), "csadv_set_graphs")

    def set_profiling(self, enable):
        L.check(L.lib().csadv_set_profiling(self._h, int(bool(enable))), "csadv_set_profiling")

    def set_inline_ghosts(self, enable):
        L.check(L.lib().csadv_set_inline_ghosts(self._h, int(bool(enable))), "csadv_set_inline_ghosts")
        self.inline_ghosts = bool(enable)

    def stats(self):
        st = L.Stats()
        L.check(L.lib().csadv_get_stats(self._h, ctypes.byref(st)), "csadv_get_stats")
        return {name: getattr(st, name) for name, _ in L.Stats._fields_ if name != "reserved"}

    def reset_stats(self):
        L.check(L.lib().csadv_reset_stats(self._h), "csadv_reset_stats")

    def divergence(self, tracer=0):
        out = np.empty((self.N, self.N, 6), dtype=np.float64)
        L.check(L.lib().csadv_divergence(self._h, tracer, out.ctypes.data, self.stream), "csadv_divergence")
        return out
