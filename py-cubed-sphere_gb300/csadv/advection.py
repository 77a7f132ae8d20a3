"""Drop-in replacements for the reference's advection entry points, backed by libcsadv.

Same names, arguments and error behaviour as the reference:

* ``cubed_sphere(N, transformation, showonscreen, gridload)``  -- cs_datastruct.py:25
* ``adv_simulation_par(cs_grid, dt, Tf, ic, vf, tc, recon, dp, opsplit, et, mt, mf)`` -- advection_ic.py:21
* ``init_vars_adv(cs_grid, simulation)``                       -- advection_vars.py:19
* ``adv_time_step(cs_grid, simulation, k, t)``                 -- advection_timestep.py:19
* ``update_adv(cs_grid, simulation, t)``                       -- advection_timestep.py:48
* ``adv_sphere(cs_grid, ll_grid, simulation, map_projection, plot, divtest_flag)`` -- advection_sphere.py:13
* ``mass_computation(Q, cs_grid, total_mass0)``                -- diagnostics.py:14
* ``compute_errors(Q, Qref)``                                  -- errors.py:99
* ``latlon_grid``, ``ll2cs``, ``nearest_neighbour`` (re-exported from ``csadv.latlon``)

The grid geometry, winds and tracer live on the GPU; ``simulation.Q`` reads return a
float64 copy in the reference layout (N+8, N+8, 6) and assignments upload one.  Plots
(matplotlib/cartopy) are not produced.
"""
import numpy as np

from . import _lib as L
from .latlon import latlon_grid, ll2cs, nearest_neighbour  # noqa: F401
from .plan import Plan

# where adv_sphere(plot=True) writes the lat-lon fields (the reference's graph directory)
output_dir = "graphs"

_RECON = {1: "PPM-0", 2: "PPM-CW84", 3: "PPM-PL07", 4: "PPM-L04"}
_DP = {1: "RK1", 2: "RK2"}
_SPLIT = {1: "SP-AVLT", 2: "SP-L04", 3: "SP-PL07"}
_ET = {1: "ET-S72", 2: "ET-PL07", 3: "ET-DG"}
_MT = {1: "MT-0", 2: "MT-PL07"}
_MF = {1: "MF-0", 2: "MF-AF", 3: "MF-PR"}


class UnsupportedSplitting(UnboundLocalError):
    """Raised where the reference fails with UnboundLocalError (discrete_operators.py:49-73):
    SP-AVLT and SP-L04 need MT-0, SP-PL07 needs MT-PL07."""


class cubed_sphere:
    """Gnomonic equiangular cubed sphere of N cells per panel edge, 4 ghost layers.

    The geometry itself is generated on the GPU when a simulation is initialised; this
    object carries the index bookkeeping of the reference (i0, iend, j0, jend, dx ...).
    """

    def __init__(self, N, transformation="gnomonic_equiangular", showonscreen=False, gridload=False):
        if transformation != "gnomonic_equiangular":
            print("ERROR: invalid grid transformation.")
            raise SystemExit(1)
        if N < 8:
            print("ERROR: N must be at least 8.")
            raise SystemExit(1)
        self.N = int(N)
        self.projection = transformation
        self.R = 1.0
        self.ngl = self.ngr = 4
        self.ng = 8
        self.i0, self.iend = 4, 4 + self.N
        self.j0, self.jend = 4, 4 + self.N
        a = np.pi / 4.0
        self.a = a
        self.dx = (a - (-a)) / self.N
        self.dy = self.dx
        self.name = self.projection + "_cs_" + str(self.N)
        if showonscreen:
            print("--------------------------------------------------------")
            print("Cubed sphere " + self.projection + " with " + str(6 * N * N) + " cells (generated on the GPU)")


class adv_simulation_par:
    """Options and state of one advection run (advection_ic.py:21-203)."""

    def __init__(self, cs_grid, dt, Tf, ic, vf, tc, recon, dp, opsplit, et, mt, mf, precision=64, ntracers=1,
                 engine=L.ENGINE_AUTO, wind_param=(0.0, 0.0, 0.0, 0.0)):
        self.ic, self.vf, self.tc = ic, vf, tc
        self.dt, self.dto2, self.twodt, self.Tf = dt, dt * 0.5, dt * 2.0, Tf
        self.recon, self.dp, self.opsplit = recon, dp, opsplit
        self.edge_treatment, self.metric_tensor, self.mass_fixer = et, mt, mf
        self.degree = 3
        if ic not in (1, 2, 3, 4):
            print("Error in adv_simulation_par - invalid initial condition")
            raise SystemExit(1)
        if vf not in (1, 2, 3, 4, L.WIND_SOLID, L.WIND_DEFORM, L.WIND_SOLID_DIV):
            print("Error in adv_simulation_par - invalid vector field")
            raise SystemExit(1)
        if recon not in _RECON:
            print("Error in adv_simulation_par - invalid reconstruction method")
            raise SystemExit(1)
        if dp not in _DP:
            print("Error in simulation_adv_par - invalid departure point scheme", dp)
            raise SystemExit(1)
        if opsplit not in _SPLIT:
            print("Error in adv_simulation_par - invalid operator splitting method")
            raise SystemExit(1)
        if et not in _ET:
            print("ERROR in adv_simulation_par: invalid ET")
            raise SystemExit(1)
        if mt not in _MT:
            print("ERROR in adv_simulation_par: invalid MT")
            raise SystemExit(1)
        if mf not in _MF:
            print("ERROR in adv_simulation_par: invalid MF")
            raise SystemExit(1)
        if tc not in (1, 2):
            print("Error in adv_simulation_par- invalid test case")
            raise SystemExit(1)
        self.recon_name, self.dp_name, self.opsplit_name = _RECON[recon], _DP[dp], _SPLIT[opsplit]
        self.et_name, self.mt_name, self.mf_name = _ET[et], _MT[mt], _MF[mf]
        self.precision, self.ntracers, self.engine = precision, ntracers, engine
        self.wind_param = tuple(wind_param)
        self.plan = None
        self._deferred = None
        self.CFL = 0.0
        self.total_mass0 = self.total_mass = self.mass_change = 0.0
        self.error_linf = self.error_l1 = self.error_l2 = None
        self.N = cs_grid.N

    @property
    def Q(self):
        self._require()
        return self.plan.get_tracer(0, full=True)

    @Q.setter
    def Q(self, value):
        self._require()
        self.plan.set_tracer(value, 0)

    def _require(self):
        if self._deferred is not None:
            raise self._deferred
        if self.plan is None:
            raise RuntimeError("init_vars_adv has not been called")


def init_vars_adv(cs_grid, simulation):
    """Build the grid, winds and tracer on the GPU and set Q0 (advection_vars.py:19-107)."""
    s = simulation
    try:
        s.plan = Plan(cs_grid.N, s.dt, s.recon, s.dp, s.opsplit, s.edge_treatment, s.metric_tensor, s.mass_fixer,
                      s.vf, ntracers=s.ntracers, precision=s.precision, engine=s.engine, wind_param=s.wind_param)
    except L.CsadvError as e:
        if e.status == L.ERR_OPTION_PAIR:
            # the reference only fails in the first divergence evaluation
            s._deferred = UnsupportedSplitting("local variable referenced before assignment (%s with %s)"
                                               % (s.opsplit_name, s.mt_name))
            return
        raise
    s.CFL = s.plan.cfl
    for t in range(s.ntracers):
        s.plan.init_tracer(s.ic, tracer=t)


def adv_time_step(cs_grid, simulation, k, t):
    """advection_timestep.py:19-43 (every tracer of the simulation)."""
    simulation._require()
    simulation.plan.time_step(k)


def update_adv(cs_grid, simulation, t):
    """advection_timestep.py:48-75."""
    simulation._require()
    simulation.plan.update_winds(t)


def mass_computation(Q, cs_grid, total_mass0):
    """diagnostics.py:14-26.  ``Q`` is a simulation (device reduction) or a host array."""
    if isinstance(Q, adv_simulation_par):
        Q._require()
        total_mass = Q.plan.mass(0)
    else:
        raise TypeError("mass_computation expects the simulation object (its Q lives on the GPU); got %r"
                        % (type(Q),))
    if abs(total_mass0) > 10 ** (-10):
        mass_change = abs(total_mass0 - total_mass) / abs(total_mass0)
    else:
        mass_change = abs(total_mass0 - total_mass)
    return total_mass, mass_change


def compute_errors(Q, Qref):
    """errors.py:99-113 on host arrays: (Linf, L1, L2) of |Q - Qref|."""
    E = np.abs(np.asarray(Qref) - np.asarray(Q))
    n = E.size
    return np.amax(E), np.sum(E) / n, np.sqrt(np.sum(E * E) / n)


def print_diagnostics_adv(error_linf, error_l1, error_l2, mass_change, t, Nsteps):
    """output.py:14-17."""
    print("\nStep", t, "from", Nsteps)
    print("Error (Linf, L1, L2) :", "{:.2e}".format(error_linf), "{:.2e}".format(error_l1),
          "{:.2e}".format(error_l2))
    print("Total mass variation:", "{:.2e}".format(mass_change))


def output_adv(cs_grid, ll_grid, simulation, plot, k, t, Nsteps, plotstep, map_projection, divtest_flag):
    """Diagnostics part of output.py:22-54 (errors vs exact solution, mass, blow-up stop)."""
    if not (plot or k == Nsteps):
        return
    s = simulation
    linf, l1, l2 = s.plan.errors(s.ic, t)
    s.error_linf[k], s.error_l1[k], s.error_l2[k] = linf, l1, l2
    if linf > 100.0:
        print("Stopping due to large errors.")
        print("The CFL number is:", s.CFL)
        raise SystemExit(1)
    s.total_mass, s.mass_change = mass_computation(s, cs_grid, s.total_mass0)
    if k > 0 and not divtest_flag:
        print_diagnostics_adv(linf, l1, l2, s.mass_change, k, Nsteps)
    # the reference's lat-lon plots (output.py:56-110), headless: Q on the lat-lon grid as .npy
    if plot and ll_grid is not None and not divtest_flag and (k % max(plotstep, 1) == 0 or k == 0 or k == Nsteps):
        import os
        from .latlon import save_latlon
        os.makedirs(output_dir, exist_ok=True)
        name = "adv_Q_ic%d_vf%d_%s_%s_%s_%s_%s_interp%d_t%d" % (s.ic, s.vf, s.opsplit_name, s.recon_name, s.dp_name,
                                                                s.et_name, s.mt_name, s.degree, k)
        save_latlon(os.path.join(output_dir, name + ".npy"), s, cs_grid, ll_grid)


def adv_sphere(cs_grid, ll_grid, simulation, map_projection, plot, divtest_flag):
    """advection_sphere.py:13-61: run Tf/dt steps; returns (Linf, L1, L2) at the last step."""
    s = simulation
    dt, Tf = s.dt, s.Tf
    Nsteps = int(Tf / dt)
    plotstep = int(Nsteps / 5)
    if divtest_flag:
        Nsteps = 1
        plotstep = 1
    s.error_linf, s.error_l1, s.error_l2 = np.zeros(Nsteps + 1), np.zeros(Nsteps + 1), np.zeros(Nsteps + 1)
    init_vars_adv(cs_grid, s)
    s._require()
    s.total_mass0, _ = mass_computation(s, cs_grid, 1.0)
    if divtest_flag:
        div = s.plan.divergence(0)
        if s.vf > 2:
            raise NotImplementedError("divergence test against div_exact is implemented for vf <= 2")
        s.div = div
        s.error_linf[1], s.error_l1[1], s.error_l2[1] = compute_errors(div, np.zeros_like(div))
        adv_time_step(cs_grid, s, 1, dt)
        return s.error_linf[1], s.error_l1[1], s.error_l2[1]
    output_adv(cs_grid, ll_grid, s, plot, 0, 0.0, Nsteps, plotstep, map_projection, divtest_flag)
    if not plot and Nsteps > 0:
        # nothing is output before the last step: the same steps (time step, then wind update
        # at k dt), replayed on the device without a host round trip per step
        s.plan.advance(Nsteps - 1)
        adv_time_step(cs_grid, s, Nsteps, Nsteps * dt)
        output_adv(cs_grid, ll_grid, s, plot, Nsteps, Nsteps * dt, Nsteps, plotstep, map_projection, divtest_flag)
        update_adv(cs_grid, s, Nsteps * dt)
        return s.error_linf[Nsteps], s.error_l1[Nsteps], s.error_l2[Nsteps]
    for k in range(1, Nsteps + 1):
        t = k * dt
        adv_time_step(cs_grid, s, k, t)
        output_adv(cs_grid, ll_grid, s, plot, k, t, Nsteps, plotstep, map_projection, divtest_flag)
        update_adv(cs_grid, s, t)
    return s.error_linf[Nsteps], s.error_l1[Nsteps], s.error_l2[Nsteps]


def print_errors_simul(error_linf, error_l1, error_l2, i):
    """errors.py:87-94."""
    if i > 0:
        print("Norms          (Linf,    L1,       L2) ")
        print("Error E_" + str(i) + "    :", "{:.2e}".format(error_linf[i]), "{:.2e}".format(error_l1[i]),
              "{:.2e}".format(error_l2[i]))
        print("Ratio E_" + str(i) + "/E_" + str(i - 1) + ":", "{:.2e}".format(error_linf[i - 1] / error_linf[i]),
              "{:.2e}".format(error_l1[i - 1] / error_l1[i]), "{:.2e}".format(error_l2[i - 1] / error_l2[i]))
    else:
        print("Error(Linf, L1, L2) :", "{:.2e}".format(error_linf[i]), "{:.2e}".format(error_l1[i]),
              "{:.2e}".format(error_l2[i]))


# the four schemes of the reference's convergence study (advection_error.py:66-71):
# (recon, split, et, mt, dp, mf) -> PL07-RK1, PL07-RK1-DG-PR, AVLT-RK2-DG-AF, AVLT-RK2-DG-PR
CONVERGENCE_SCHEMES = ((3, 3, 2, 2, 1, 1), (3, 3, 3, 2, 1, 3), (3, 1, 3, 1, 2, 2), (3, 1, 3, 1, 2, 3))
CONVERGENCE_NAMES = ("PL07-RK1", "PL07-RK1-DG-PR", "AVLT-RK2-DG-AF", "ALVT-RK2-DG-PR")


def error_analysis_adv(simulation, map_projection, plot, transformation, showonscreen, gridload, Ntest=6,
                       pardir=None):
    """advection_error.py:21-188: N = 16, 32, ... (Ntest resolutions), dt halved with N, one
    period (Tf = 5) of each of the four schemes, errors against the exact solution at Tf.
    Returns (Nc, error_linf, error_l1, error_l2, rates) with errors of shape (Ntest, 4) and
    rates[norm] = log2(E_i-1 / E_i).  Figures are not drawn (plot is ignored)."""
    from .configuration import PARDIR, get_advection_parameters
    vf = simulation.vf
    tc = simulation.tc
    dt0 = {1: 0.025, 2: 0.0125, 3: 0.00625, 4: 0.0125}.get(vf)
    if dt0 is None:
        print("ERROR: invalid vector field, ", vf)
        raise SystemExit(1)
    Nc = np.array([16 * 2 ** i for i in range(Ntest)], dtype=float)
    dts = np.array([dt0 * 0.5 ** i for i in range(Ntest)])
    errs = [np.zeros((Ntest, len(CONVERGENCE_SCHEMES))) for _ in range(3)]
    dt, Tf, tc_par, ic, vf_par, recon, dp, opsplit, et, mt, mf = get_advection_parameters(pardir or PARDIR, verbose=False)
    Tf = 5
    for d, (rec, sp, ET, MT, DP, MF) in enumerate(CONVERGENCE_SCHEMES):
        for i in range(Ntest):
            N = int(Nc[i])
            cs_grid = cubed_sphere(N, transformation, False, gridload)
            sim = adv_simulation_par(cs_grid, dts[i], Tf, ic, vf, tc, rec, DP, sp, ET, MT, MF)
            print("\nParameters: N=" + str(N) + ", dt=" + str(dts[i]), ", recon=", sim.recon_name, ", split=",
                  sim.opsplit_name, ", dp=", sim.dp_name, ", et=", sim.et_name)
            errs[0][i, d], errs[1][i, d], errs[2][i, d] = adv_sphere(cs_grid, None, sim, map_projection, False, False)
            print_errors_simul(errs[0][:, d], errs[1][:, d], errs[2][:, d], i)
            sim.plan.close()
    rates = {name: np.abs(np.log(e[1:]) - np.log(e[:-1])) / np.log(2.0) for name, e in zip(("linf", "l1", "l2"), errs)}
    for name, r in rates.items():
        print("Convergence rate (" + name + "):", " ".join("%s %s" % (CONVERGENCE_NAMES[d], np.array2string(r[:, d], precision=2))
                                                       for d in range(len(CONVERGENCE_SCHEMES))))
    return Nc, errs[0], errs[1], errs[2], rates
