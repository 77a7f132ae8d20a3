"""Advection time step and driver (oracle restatement).

* ``Simulation``     -- option decoding and state (advection_ic.py:21-203,
                        cs_datastruct.py:635-735), initialisation (advection_vars.py:19-107)
* ``divergence``     -- discrete_operators.py:18-138
* ``adv_time_step``  -- advection_timestep.py:19-43
* ``update_adv``     -- advection_timestep.py:48-75
* ``time_averaged_velocity`` -- averaged_velocity.py:14-62
* ``adv_sphere``     -- advection_sphere.py:13-61 (plot=False path)
* ``mass_computation`` / ``compute_errors`` -- diagnostics.py:14-26, errors.py:99-113
"""
import numpy as np

from . import cases, halo, ppm
from .grid import CubedSphere, NBFACES

RECON = {1: "PPM-0", 2: "PPM-CW84", 3: "PPM-PL07", 4: "PPM-L04"}
DP = {1: "RK1", 2: "RK2"}
SPLIT = {1: "SP-AVLT", 2: "SP-L04", 3: "SP-PL07"}
ET = {1: "ET-S72", 2: "ET-PL07", 3: "ET-DG"}
MT = {1: "MT-0", 2: "MT-PL07"}
MF = {1: "MF-0", 2: "MF-AF", 3: "MF-PR"}


class OptionError(ValueError):
    pass


def check_options(recon, dp, opsplit, et, mt, mf):
    """Option validation: the reference exits on unknown codes (advection_ic.py:85-149) and
    fails with UnboundLocalError on unsupported splitting/metric pairs
    (discrete_operators.py:49-73): SP-AVLT and SP-L04 need MT-0, SP-PL07 needs MT-PL07."""
    for name, v, tab in (("recon", recon, RECON), ("dp", dp, DP), ("opsplit", opsplit, SPLIT),
                         ("et", et, ET), ("mt", mt, MT), ("mf", mf, MF)):
        if v not in tab:
            raise OptionError("invalid %s %r" % (name, v))
    if (opsplit in (1, 2)) != (mt == 1):
        raise OptionError("splitting %s requires %s" % (SPLIT[opsplit], "MT-0" if opsplit in (1, 2) else "MT-PL07"))


class Simulation:
    """State of one advection solve on one grid.

    ``ic``/``vf`` are the reference's integer cases; alternatively ``ic_spec``/``wind``
    give a benchmark IC/wind (``cases.ICSpec``/``cases.WindSpec``).
    """

    def __init__(self, grid, dt, Tf, ic, vf, recon, dp, opsplit, et, mt, mf,
                 ic_spec=None, wind=None, q0=None):
        check_options(recon, dp, opsplit, et, mt, mf)
        self.grid = grid
        self.dt, self.Tf = dt, Tf
        self.dto2 = dt * 0.5
        self.ic, self.vf = ic, vf
        self.ic_spec, self.wind = ic_spec, wind
        self.recon_name, self.dp_name = RECON[recon], DP[dp]
        self.opsplit_name, self.et_name = SPLIT[opsplit], ET[et]
        self.mt_name, self.mf_name = MT[mt], MF[mf]
        self.degree = 3
        n = grid.N + grid.ng
        shp_c, shp_u, shp_v = (n, n, NBFACES), (n + 1, n, NBFACES), (n, n + 1, NBFACES)
        self.Q = np.zeros(shp_c)
        self.div = np.zeros(shp_c)
        self.w = {
            "u_pu": np.zeros(shp_u), "vc_pu": np.zeros(shp_u), "ulon_pu": np.zeros(shp_u),
            "vlat_pu": np.zeros(shp_u), "u_pu_old": np.zeros(shp_u), "u_pu_avg": np.zeros(shp_u),
            "v_pv": np.zeros(shp_v), "uc_pv": np.zeros(shp_v), "ulon_pv": np.zeros(shp_v),
            "vlat_pv": np.zeros(shp_v), "v_pv_old": np.zeros(shp_v), "v_pv_avg": np.zeros(shp_v),
            "uc_pc": np.zeros(shp_c), "vc_pc": np.zeros(shp_c),
            "ulon_pc": np.zeros(shp_c), "vlat_pc": np.zeros(shp_c),
        }
        self.dF_x = np.zeros(shp_c)
        self.dF_y = np.zeros(shp_c)
        self.f_x = np.zeros(shp_u)
        self.f_y = np.zeros(shp_v)
        self.upos = None
        self.vpos = None
        self.cx = np.zeros(shp_u)
        self.cy = np.zeros(shp_v)
        self._init_vars(q0)

    @property
    def time_dependent(self):
        if self.wind is not None:
            return self.wind.time_dependent
        return self.vf >= 2

    def velocity(self, lon, lat, t):
        if self.wind is not None:
            return self.wind(lon, lat, t)
        return cases.velocity_ref(lon, lat, t, self.vf)

    def qexact(self, lon, lat, t):
        if self.ic_spec is not None:
            return self.ic_spec(lon, lat, t, self.wind)
        return cases.qexact_ref(lon, lat, t, self.ic, self.vf)

    def _interior_winds(self, t):
        """Analytic winds at interior edges -> contravariant (advection_vars.py:38-53)."""
        g, w = self.grid, self.w
        i0, iend, j0, jend = g.i0, g.iend, g.j0, g.jend
        iu = (slice(i0, iend + 1), slice(j0, jend), slice(None))
        iv = (slice(i0, iend), slice(j0, jend + 1), slice(None))
        w["ulon_pu"][iu], w["vlat_pu"][iu] = self.velocity(g.pu.lon[iu], g.pu.lat[iu], t)
        w["ulon_pv"][iv], w["vlat_pv"][iv] = self.velocity(g.pv.lon[iv], g.pv.lat[iv], t)
        w["u_pu"][iu], w["vc_pu"][iu] = halo.latlon_to_contravariant(w["ulon_pu"][iu], w["vlat_pu"][iu], g.pu, iu)
        w["uc_pv"][iv], w["v_pv"][iv] = halo.latlon_to_contravariant(w["ulon_pv"][iv], w["vlat_pv"][iv], g.pv, iv)

    def vector_halo(self):
        """edges_treatment.py:296-347."""
        if self.et_name == "ET-DG":
            halo.vector_halo_dg(self.w, self.grid, self.Wt, self.Kmin)
        elif self.dp_name == "RK2":
            halo.vector_halo_adjacent_rk2(self.w["u_pu"], self.w["v_pv"], self.grid)

    def _init_vars(self, q0):
        """advection_vars.py:19-107."""
        g, w = self.grid, self.w
        self._interior_winds(0.0)
        self.Wt, self.Kmin = halo.lagrange_tables(g, self.degree)
        self.vector_halo()
        w["u_pu_old"][...] = w["u_pu"]
        w["v_pv_old"][...] = w["v_pv"]
        time_averaged_velocity(self)
        cx = w["u_pu"] * self.dt / g.dx
        cy = w["v_pv"] * self.dt / g.dy
        self.CFL = max(abs(np.amax(cx[g.i0:g.iend + 1])), abs(np.amax(cy[:, g.j0:g.jend + 1])))
        it = g.interior
        if q0 is None:
            self.Q[it] = self.qexact(g.pc.lon[it], g.pc.lat[it], 0.0)
        else:
            self.Q[it] = q0

    def fill_scalar_halo(self, Qx, Qy):
        """edges_treatment.py:284-290."""
        if self.et_name == "ET-DG":
            halo.dg_fill(Qx, self.grid, self.Wt, self.Kmin)
        else:
            halo.adjacent_fill(Qx, Qy, self.grid)


def time_averaged_velocity(sim):
    """averaged_velocity.py:14-62: upwind masks from the current wind, departure-point wind."""
    g, w = sim.grid, sim.w
    i0, iend, j0, jend = g.i0, g.iend, g.j0, g.jend
    sim.upos = w["u_pu"][i0:iend + 1] >= 0
    sim.vpos = w["v_pv"][:, j0:jend + 1] >= 0
    if sim.dp_name == "RK1":
        w["u_pu_avg"][...] = w["u_pu"]
        w["v_pv_avg"][...] = w["v_pv"]
        return
    for U, Uold, Uavg, pos, d, T in (("u_pu", "u_pu_old", "u_pu_avg", sim.upos, g.dx, False),
                                     ("v_pv", "v_pv_old", "v_pv_avg", sim.vpos, g.dy, True)):
        u = w[U].transpose(1, 0, 2) if T else w[U]
        uo = w[Uold].transpose(1, 0, 2) if T else w[Uold]
        ua = w[Uavg].transpose(1, 0, 2) if T else w[Uavg]
        p = pos.transpose(1, 0, 2) if T else pos
        ui = 1.5 * u - 0.5 * uo
        a = u[i0:iend + 1] * sim.dto2 / d
        fpos = (1.0 - a) * ui[i0:iend + 1] + a * ui[i0 - 1:iend]
        fneg = -a * ui[i0 + 1:iend + 2] + (1.0 + a) * ui[i0:iend + 1]
        ua[i0:iend + 1] = np.where(p, fpos, fneg)


def compute_fluxes(sim, Qa, Qb):
    """flux.py:9-15: x-reconstruction/flux of Qa, y-reconstruction/flux of Qb."""
    g = sim.grid
    i0, iend = g.i0, g.iend
    n = g.N + g.ng
    qLx, qRx = np.zeros((n, n, NBFACES)), np.zeros((n, n, NBFACES))
    qLy, qRy = np.zeros((n, n, NBFACES)), np.zeros((n, n, NBFACES))
    ppm.reconstruct(Qa, qLx, qRx, sim.recon_name, i0, iend)
    ppm.reconstruct(ppm.T(Qb), ppm.T(qLy), ppm.T(qRy), sim.recon_name, g.j0, g.jend)
    if sim.et_name == "ET-PL07":
        ppm.edges_extrapolation(Qa, Qb, qLx, qRx, qLy, qRy, g, sim.recon_name)
    w = sim.w
    sim.f_x[i0:iend + 1] = ppm.upwind_flux(Qa, qLx, qRx, sim.cx, w["u_pu_avg"], sim.upos,
                                           g.metric_tensor_pu, g.metric_tensor_pc, sim.mt_name, i0, iend)
    fy = ppm.upwind_flux(ppm.T(Qb), ppm.T(qLy), ppm.T(qRy), ppm.T(sim.cy), ppm.T(w["v_pv_avg"]),
                         ppm.T(sim.vpos), ppm.T(g.metric_tensor_pv), ppm.T(g.metric_tensor_pc),
                         sim.mt_name, g.j0, g.jend)
    ppm.T(sim.f_y)[g.j0:g.jend + 1] = fy
    return qLx, qRx, qLy, qRy


def _flux_difference(sim):
    """F_operator / G_operator (discrete_operators.py:109-138)."""
    g = sim.grid
    i0, iend, j0, jend = g.i0, g.iend, g.j0, g.jend
    dt = sim.dt
    sim.dF_x[i0:iend] = -(sim.f_x[i0 + 1:iend + 1] - sim.f_x[i0:iend])
    sim.dF_x[i0:iend] = sim.dF_x[i0:iend] * dt / g.dx
    sim.dF_y[:, j0:jend] = -(sim.f_y[:, j0 + 1:jend + 1] - sim.f_y[:, j0:jend])
    sim.dF_y[:, j0:jend] = sim.dF_y[:, j0:jend] * dt / g.dy


def divergence(sim):
    """discrete_operators.py:18-101.  Returns the intermediate (Qx, Qy) for inspection."""
    g = sim.grid
    i0, iend, j0, jend = g.i0, g.iend, g.j0, g.jend
    N, ng, dt = g.N, g.ng, sim.dt
    G = g.metric_tensor_pc
    Q = sim.Q
    gQ = Q * G
    sim.cx[...] = sim.w["u_pu_avg"] * dt / g.dx
    sim.cy[...] = sim.w["v_pv_avg"] * dt / g.dy
    compute_fluxes(sim, Q, Q)
    _flux_difference(sim)
    dFx, dFy = sim.dF_x, sim.dF_y
    if sim.opsplit_name == "SP-AVLT":
        gQx = gQ + 0.5 * dFx
        gQy = gQ + 0.5 * dFy
    else:
        c1x = g.metric_tensor_pu[1:] * sim.cx[1:]
        c2x = g.metric_tensor_pu[:N + ng] * sim.cx[:N + ng]
        c1y = g.metric_tensor_pv[:, 1:] * sim.cy[:, 1:]
        c2y = g.metric_tensor_pv[:, :N + ng] * sim.cy[:, :N + ng]
        if sim.opsplit_name == "SP-L04":
            gQx = gQ + 0.5 * dFx + 0.5 * (c1x - c2x) * Q
            gQy = gQ + 0.5 * dFy + 0.5 * (c1y - c2y) * Q
        else:
            Qx = 0.5 * (Q + (Q + dFx) / (1.0 - (c1x - c2x)))
            Qy = 0.5 * (Q + (Q + dFy) / (1.0 - (c1y - c2y)))
    if sim.mt_name == "MT-0":
        Qx, Qy = gQx / G, gQy / G
    if sim.et_name in ("ET-S72", "ET-PL07"):
        sim.fill_scalar_halo(Qx, Qy)
    compute_fluxes(sim, Qy, Qx)
    if sim.mf_name == "MF-AF":
        ppm.average_flux_cube_edges(sim.f_x, sim.f_y, g)
    _flux_difference(sim)
    sim.div[...] = -(sim.dF_x + sim.dF_y) / (dt * G)
    if sim.mf_name == "MF-PR":
        it = g.interior
        m0 = np.sum(sim.div[it] * G[it])
        a2 = np.sum(G[it] * G[it])
        sim.div[it] = sim.div[it] - G[it] * m0 / a2
    return Qx, Qy


def adv_time_step(sim, k, t):
    """advection_timestep.py:19-43."""
    g = sim.grid
    sim.fill_scalar_halo(sim.Q, sim.Q)
    if sim.time_dependent:
        sim.vector_halo()
        time_averaged_velocity(sim)
    divergence(sim)
    it = g.interior
    sim.Q[it] = sim.Q[it] - sim.dt * sim.div[it]


def update_adv(sim, t):
    """advection_timestep.py:48-75 (vf >= 2 only).

    New analytic winds on interior edges, old <- current, lat-lon -> contravariant.  The
    reference converts the full edge arrays; entries outside the interior keep the lat-lon
    values written by the last wind halo, so their contravariant values are recomputed
    from unchanged inputs and are restated here the same way.
    """
    if not sim.time_dependent:
        return
    g, w = sim.grid, sim.w
    i0, iend, j0, jend = g.i0, g.iend, g.j0, g.jend
    iu = (slice(i0, iend + 1), slice(j0, jend), slice(None))
    iv = (slice(i0, iend), slice(j0, jend + 1), slice(None))
    w["ulon_pu"][iu], w["vlat_pu"][iu] = sim.velocity(g.pu.lon[iu], g.pu.lat[iu], t)
    w["ulon_pv"][iv], w["vlat_pv"][iv] = sim.velocity(g.pv.lon[iv], g.pv.lat[iv], t)
    w["u_pu_old"][...] = w["u_pu"]
    w["v_pv_old"][...] = w["v_pv"]
    full = (slice(None), slice(None), slice(None))
    w["u_pu"][...], w["vc_pu"][...] = halo.latlon_to_contravariant(w["ulon_pu"], w["vlat_pu"], g.pu, full)
    w["uc_pv"][...], w["v_pv"][...] = halo.latlon_to_contravariant(w["ulon_pv"], w["vlat_pv"], g.pv, full)


def run_steps(sim, nsteps, k0=1):
    """Time loop body of advection_sphere.py:45-57 (no output)."""
    for k in range(k0, k0 + nsteps):
        t = k * sim.dt
        adv_time_step(sim, k, t)
        update_adv(sim, t)


def mass_computation(Q, grid, total_mass0):
    """diagnostics.py:14-26."""
    it = grid.interior
    m = np.sum(Q[it] * grid.metric_tensor_pc[it] * grid.dx * grid.dy)
    if abs(total_mass0) > 1e-10:
        change = abs(total_mass0 - m) / abs(total_mass0)
    else:
        change = abs(total_mass0 - m)
    return m, change


def compute_errors(Q, Qref):
    """errors.py:99-113: Linf, L1 (mean), L2 (RMS) of |Q - Qref|."""
    E = np.abs(Qref - Q)
    n = E.size
    return np.amax(np.abs(E)), np.sum(E) / n, np.sqrt(np.sum(E * E) / n)


def adv_sphere(sim, nsteps=None):
    """advection_sphere.py:13-61 without plots: returns (Linf, L1, L2) at the last step."""
    g = sim.grid
    if nsteps is None:
        nsteps = int(sim.Tf / sim.dt)
    sim.total_mass0, _ = mass_computation(sim.Q, g, 1.0)
    run_steps(sim, nsteps)
    it = g.interior
    t = nsteps * sim.dt
    qex = sim.qexact(g.pc.lon[it], g.pc.lat[it], t)
    return compute_errors(sim.Q[it], qex)
