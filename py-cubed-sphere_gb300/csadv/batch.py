"""Many solves advanced together: one step-kernel launch per step for all of them.

``Batch`` wraps ``csadv_batch_*`` (include/csadv.h).  Plans keep their own state and
diagnostics (``Plan.get_tracer``, ``Plan.errors`` ...); attaching a plan to a batch only
changes how its steps are launched, not their results.  ``tune`` wraps ``csadv_tune``.
"""
import ctypes

from . import _lib as L


class Batch:
    def __init__(self, capacity=256):
        h = ctypes.c_void_p()
        L.check(L.lib().csadv_batch_create(int(capacity), ctypes.byref(h)), "csadv_batch_create")
        self._h = h
        self._plans = []

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            L.lib().csadv_batch_destroy(self._h)
            self._h = ctypes.c_void_p()
            self._plans = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __len__(self):
        n = ctypes.c_int()
        L.check(L.lib().csadv_batch_size(self._h, ctypes.byref(n)), "csadv_batch_size")
        return n.value

    def add(self, plan):
        L.check(L.lib().csadv_batch_add(self._h, plan._h), "csadv_batch_add")
        self._plans.append(plan)  # keep the plan alive while attached

    def remove(self, plan):
        L.check(L.lib().csadv_batch_remove(self._h, plan._h), "csadv_batch_remove")
        self._plans = [p for p in self._plans if p is not plan]

    def advance(self, nsteps, stream=None):
        L.check(L.lib().csadv_batch_advance(self._h, int(nsteps), L.stream_handle(stream)), "csadv_batch_advance")

    def set_queue_depth(self, depth):
        """advance() waits until the call `depth` calls back has finished on the GPU (0: never)."""
        L.check(L.lib().csadv_batch_set_queue_depth(self._h, int(depth)), "csadv_batch_set_queue_depth")

    def set_graphs(self, enable):
        L.check(L.lib().csadv_batch_set_graphs(self._h, int(bool(enable))), "csadv_batch_set_graphs")

    def set_profiling(self, enable):
        L.check(L.lib().csadv_batch_set_profiling(self._h, int(bool(enable))), "csadv_batch_set_profiling")

    def reset_stats(self):
        L.check(L.lib().csadv_batch_reset_stats(self._h), "csadv_batch_reset_stats")

    def stats(self):
        st = L.Stats()
        L.check(L.lib().csadv_batch_get_stats(self._h, ctypes.byref(st)), "csadv_batch_get_stats")
        return {name: getattr(st, name) for name, _ in L.Stats._fields_ if name != "reserved"}


def tune(plan, reps=5, stream=None):
    """Pick the fastest tile configuration for ``plan`` (and later plans of its shape);
    returns the csadv_options.tile code chosen."""
    t = ctypes.c_int()
    L.check(L.lib().csadv_tune(plan._h, int(reps), L.stream_handle(stream), ctypes.byref(t)), "csadv_tune")
    return t.value
