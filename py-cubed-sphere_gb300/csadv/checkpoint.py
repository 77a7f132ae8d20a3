"""Checkpoint and resume of a solve (``.npz``).

``save(plan, path)`` writes the plan's options, grid size, time step, step count, tracers
(float64, the reference's full (N+8, N+8, 6) layout) and, for the FP32 form with the mass
fixer, each tracer's mass target; ``load(path)`` builds a new plan from them.  The resumed
plan continues with the same bits as the saved one would have: the tile shape, which fixes
the order of the mass-fixer sums, is saved too, and so is a ghost-cell choice made with
``Plan.set_inline_ghosts`` (the step kernel's own ghost cells and the separate ghost-cell
launch can differ in the last bits of FP32 corner cells).  The reference keeps no state between runs;
its grid cache (NetCDF) has no counterpart here because the grid is rebuilt on the GPU.
"""
import ctypes

import numpy as np

from . import _lib as L
from .plan import Plan

_OPTS = ("recon", "dp", "opsplit", "et", "mt", "mf", "vf", "precision", "engine", "tile")


def save(plan, path):
    o = plan._opts
    st = plan.stats()
    opts = {name: int(getattr(o, name)) for name in _OPTS}
    opts["tile"] = int(st["tile"])  # the shape in use
    data = {"options": np.array([opts[n] for n in _OPTS], dtype=np.int64),
            "wind_param": np.array(list(o.wind_param), dtype=np.float64),
            "N": plan.N, "dt": plan.dt, "ntracers": plan.ntracers, "step": plan.step,
            "inline_ghosts": -1 if plan.inline_ghosts is None else int(plan.inline_ghosts)}
    for t in range(plan.ntracers):
        data["Q%d" % t] = plan.get_tracer(t, full=True)
    targets = []
    for t in range(plan.ntracers):
        m = ctypes.c_double()
        rc = L.lib().csadv_mass_target(plan._h, t, ctypes.byref(m), None, plan.stream)
        if rc == L.ERR_UNSUPPORTED:
            break
        L.check(rc, "csadv_mass_target")
        targets.append(m.value)
    if targets:
        data["mass_target"] = np.array(targets, dtype=np.float64)
    np.savez(path, **data)


def load(path, stream=None):
    z = np.load(path)
    opts = dict(zip(_OPTS, (int(x) for x in z["options"])))
    pl = Plan(int(z["N"]), float(z["dt"]), ntracers=int(z["ntracers"]), wind_param=tuple(z["wind_param"]),
              stream=stream, **opts)
    try:
        if "inline_ghosts" in z.files and int(z["inline_ghosts"]) >= 0:
            pl.set_inline_ghosts(bool(int(z["inline_ghosts"])))
        for t in range(pl.ntracers):
            pl.set_tracer(z["Q%d" % t], tracer=t)
        if "mass_target" in z.files:
            for t, m in enumerate(z["mass_target"]):
                v = ctypes.c_double(float(m))
                L.check(L.lib().csadv_mass_target(pl._h, t, None, ctypes.byref(v), pl.stream), "csadv_mass_target")
        L.check(L.lib().csadv_set_step(pl._h, int(z["step"]), pl.stream), "csadv_set_step")
    except Exception:
        pl.close()
        raise
    return pl
