"""Run the unmodified reference (luanfs/py-cubed-sphere, pure Python) in this container.

Used only by ``make_golden.py`` to produce the committed golden fixtures; nothing in the
test suite, the library or the benchmark imports this file (the reference tree does not
exist on the GPU machine).

The reference imports four packages that are not installed here: ``numexpr``,
``netCDF4``, ``matplotlib`` and ``cartopy`` (via its ``plot`` module).  This harness puts
stand-in modules ahead of the reference's ``src/`` directory on ``sys.path``:

* ``numexpr.evaluate(expr, local_dict=None)`` evaluates the expression string with numpy,
  over the caller frame's globals and locals (plus ``local_dict`` when given), which is
  how the reference's call sites use it (e.g. ``averaged_velocity.py:42`` passes
  ``vars(U_pu)``; ``advection_ic.py:297`` reads the module global ``pi``).  numpy's
  elementwise ops are the same IEEE operations in the same order, so the stand-in differs
  from real numexpr at most in the last bits of transcendental calls.
* ``netCDF4``, ``matplotlib``, ``matplotlib.pyplot`` and ``plot`` are no-op modules
  (they are only touched by grid caching and plotting, which are not on the time-step
  path).

``main.py``, ``operator_accuracy.py`` and ``interpolation_test.py`` are never imported:
they import ``scipy.special.sph_harm``, which scipy 1.18 removed.
"""
import os
import sys
import types

import numpy as np

# the reference's src/ directory: make_golden.py --ref sets it; there is no default location
REF_SRC = os.environ.get("CSADV_REFERENCE_SRC", "")


def _stub_module(name):
    mod = types.ModuleType(name)

    def _noop(*args, **kwargs):
        return None

    def __getattr__(attr):  # any attribute is a no-op callable
        if attr.startswith("__"):
            raise AttributeError(attr)
        return _noop

    mod.__getattr__ = __getattr__
    return mod


def _numexpr_module():
    mod = types.ModuleType("numexpr")
    funcs = {
        "sin": np.sin, "cos": np.cos, "tan": np.tan, "exp": np.exp, "log": np.log,
        "sqrt": np.sqrt, "abs": np.abs, "arctan2": np.arctan2, "arctan": np.arctan,
        "arcsin": np.arcsin, "arccos": np.arccos, "where": np.where,
    }

    def evaluate(expr, local_dict=None, global_dict=None, **kwargs):
        frame = sys._getframe(1)
        ns = dict(frame.f_globals)
        ns.update(frame.f_locals)
        if local_dict is not None:
            ns.update(local_dict)
        ns.update(funcs)
        with np.errstate(all="ignore"):
            out = eval(expr, {"__builtins__": {}}, ns)
        return np.asarray(out)

    mod.evaluate = evaluate
    return mod


_installed = False


def install():
    """Install the stand-ins and put the reference's src/ on sys.path (idempotent)."""
    global _installed
    if _installed:
        return
    if not REF_SRC or not os.path.isdir(REF_SRC):
        raise RuntimeError("set CSADV_REFERENCE_SRC (or make_golden.py --ref) to the reference's src/ "
                           "directory; not found: %r" % REF_SRC)
    sys.modules["numexpr"] = _numexpr_module()
    sys.modules["netCDF4"] = _stub_module("netCDF4")
    mpl = _stub_module("matplotlib")
    sys.modules["matplotlib"] = mpl
    sys.modules["matplotlib.pyplot"] = _stub_module("matplotlib.pyplot")
    sys.modules["plot"] = _stub_module("plot")
    sys.path.insert(0, REF_SRC)
    _installed = True


def modules():
    """Import and return the reference modules used on the advection path."""
    install()
    import importlib
    names = ["constants", "cs_datastruct", "advection_ic", "advection_vars",
             "advection_timestep", "discrete_operators", "flux", "reconstruction_1d",
             "edges_treatment", "interpolation", "halo_data", "lagrange",
             "averaged_velocity", "diagnostics", "errors", "sphgeo", "cs_transform",
             "cfl", "configuration"]
    return types.SimpleNamespace(**{n: importlib.import_module(n) for n in names})


def make_sim(N, dt, Tf, ic, vf, tc, recon, dp, opsplit, et, mt, mf):
    """Build the reference grid + simulation object and run ``init_vars_adv``."""
    m = modules()
    grid = m.cs_datastruct.cubed_sphere(N, "gnomonic_equiangular", False, False)
    sim = m.advection_ic.adv_simulation_par(grid, dt, Tf, ic, vf, tc, recon, dp,
                                            opsplit, et, mt, mf)
    m.advection_vars.init_vars_adv(grid, sim)
    return m, grid, sim


def run_steps(m, grid, sim, nsteps, k0=1):
    """The body of ``adv_sphere``'s time loop (advection_sphere.py:45-57), plot=False."""
    for k in range(k0, k0 + nsteps):
        t = k * sim.dt
        m.advection_timestep.adv_time_step(grid, sim, k, t)
        m.advection_timestep.update_adv(grid, sim, t)
