"""Generate the golden fixtures in this directory by running the reference itself.

Usage (only where the reference tree exists; the fixtures are committed):

    python tests/golden/make_golden.py --ref /path/to/py-cubed-sphere/src

It imports the unmodified reference modules through ``refharness`` (stand-ins for the
uninstalled numexpr / netCDF4 / matplotlib, see that file) and records:

* ``combos_N10.npz``  -- final interior Q after 3 steps at N=10 for every valid option
                         tuple (216 = 4 recon x 2 dp x 3 split/metric pairs x 3 et x 3 mf),
                         ic=2 Gaussian hill, vf=2 (time-dependent wind: exercises the wind
                         halo and the RK2 departure point); plus the same for vf=1 and a
                         subset; plus the option tuples the reference rejects.
* ``grid_N12.npz``    -- geometry (points, metric tensors, lat-lon/contravariant
                         coefficients) and the Lagrange ghost-cell weights/stencils.
* ``stages_N16.npz``  -- one step of three schemes (ET-DG, ET-PL07, ET-S72) with the
                         intermediate arrays: filled halo, winds, parabolas, fluxes, div.
* ``run_N16.npz``     -- 40 steps of the reference's default scheme from par/advection.par
                         (PPM-PL07, RK1, AVLT, ET-DG, MT-0, MF-PR) with per-step errors and
                         mass; and 30 steps of PPM-CW84/RK2/vf=2.
* ``cases_N12.npz``   -- qexact_adv for ic 1-4 x vf 1-4 and velocity_adv for vf 1-4.
* ``par.npz``         -- the reference's parse of its own par/*.par files.
* ``latlon.npz``      -- ll2cs (panel and cell indices of lat-lon points) and
                         nearest_neighbour for three (N, Nlat, Nlon), with the lat-lon
                         points' X, Y, Z (``--only latlon`` writes just this file).
"""
import argparse
import itertools
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def valid_combos():
    out = []
    for c in itertools.product((1, 2, 3, 4), (1, 2), (1, 2, 3), (1, 2, 3), (1, 2), (1, 2, 3)):
        recon, dp, sp, et, mt, mf = c
        if (sp in (1, 2)) == (mt == 1):
            out.append(c)
    return out


def invalid_combos():
    out = []
    for c in itertools.product((3,), (1,), (1, 2, 3), (3,), (1, 2), (3,)):
        recon, dp, sp, et, mt, mf = c
        if (sp in (1, 2)) != (mt == 1):
            out.append(c)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", required=True, help="the reference's src/ directory")
    ap.add_argument("--only", default=None, choices=("latlon",))
    args = ap.parse_args()
    os.environ["CSADV_REFERENCE_SRC"] = os.path.abspath(args.ref)
    sys.path.insert(0, HERE)
    import refharness as rh
    if args.only == "latlon":
        latlon_fixtures(rh.modules())
        return

    m = rh.modules()
    interior = lambda g: (slice(g.i0, g.iend), slice(g.j0, g.jend), slice(None))  # noqa: E731

    # ---------------------------------------------------------------- all combos
    combos = valid_combos()
    res = {}
    for vf, sel in ((2, combos), (1, combos[::5]), (3, combos[::17]), (4, combos[::23])):
        Qs = []
        for c in sel:
            mod, g, s = rh.make_sim(10, 0.02, 5.0, 2, vf, 1, *c)
            rh.run_steps(mod, g, s, 3)
            Qs.append(s.Q[interior(g)].copy())
        res["combos_vf%d" % vf] = np.array(sel, dtype=np.int32)
        res["Q_vf%d" % vf] = np.array(Qs)
    rejected = []
    for c in invalid_combos():
        try:
            mod, g, s = rh.make_sim(10, 0.02, 5.0, 2, 1, 1, *c)
            rh.run_steps(mod, g, s, 1)
            rejected.append(0)
        except Exception:  # the reference fails (UnboundLocalError) on these
            rejected.append(1)
    res["invalid_combos"] = np.array(invalid_combos(), dtype=np.int32)
    res["invalid_rejected"] = np.array(rejected, dtype=np.int32)
    np.savez_compressed(os.path.join(HERE, "combos_N10.npz"), N=10, dt=0.02, ic=2, nsteps=3, **res)

    # ---------------------------------------------------------------- grid
    N = 12
    g = m.cs_datastruct.cubed_sphere(N, "gnomonic_equiangular", False, False)
    sim = m.advection_ic.adv_simulation_par(g, 0.01, 5.0, 2, 1, 1, 3, 1, 1, 3, 1, 3)
    m.lagrange.lagrange_poly_ghostcell_pc(g, sim)
    grid = {"N": N, "dx": g.dx}
    for pn in ("pc", "pu", "pv"):
        ps = getattr(g, pn)
        for f in ("X", "Y", "Z", "lon", "lat"):
            grid["%s_%s" % (pn, f)] = getattr(ps, f)
        for f in ("ex_elon", "ex_elat", "ey_elon", "ey_elat"):
            grid["%s_%s" % (pn, f)] = getattr(g, "prod_%s_%s" % (f, pn))
        grid["%s_det" % pn] = getattr(g, "determinant_ll2contra_%s" % pn)
        grid["%s_metric" % pn] = getattr(g, "metric_tensor_%s" % pn)
    grid["lagrange_w_east"] = sim.lagrange_poly_ghost_pc[0]
    grid["lagrange_kmin_east"] = sim.stencil_ghost_pc[0][0]
    # reference halo gathers of a test field (for the connectivity table)
    F = np.random.default_rng(0).standard_normal((N + 8, N + 8, 6))
    hd = m.halo_data.get_halo_data_interpolation(F, g)
    grid["halo_field"] = F
    for name, arr in zip(("east", "west", "north", "south"), hd):
        grid["halo_%s" % name] = arr
    np.savez_compressed(os.path.join(HERE, "grid_N12.npz"), **grid)

    # ---------------------------------------------------------------- stages
    st = {}
    schemes = {"dg": (2, 2, 1, 3, 1, 3), "pl07": (3, 2, 3, 2, 2, 2), "s72": (4, 1, 2, 1, 1, 1)}
    for name, c in schemes.items():
        mod, g, s = rh.make_sim(16, 0.01, 5.0, 3, 2, 1, *c)
        rh.run_steps(mod, g, s, 2)
        k = 3
        t = k * s.dt
        st[name + "_Q_before"] = s.Q.copy()
        mod.advection_timestep.adv_time_step(g, s, k, t)
        st[name + "_Q_after"] = s.Q.copy()  # ghosts hold the halo filled at step start
        st[name + "_div"] = s.div.copy()
        st[name + "_u_pu"] = s.U_pu.ucontra.copy()
        st[name + "_v_pv"] = s.U_pv.vcontra.copy()
        st[name + "_u_avg"] = s.U_pu.ucontra_averaged.copy()
        st[name + "_v_avg"] = s.U_pv.vcontra_averaged.copy()
        st[name + "_fx"] = s.px.f_upw.copy()
        st[name + "_fy"] = s.py.f_upw.copy()
        st[name + "_qLx"] = s.px.q_L.copy()
        st[name + "_qRx"] = s.px.q_R.copy()
        st[name + "_qLy"] = s.py.q_L.copy()
        st[name + "_qRy"] = s.py.q_R.copy()
        st[name + "_dFx"] = s.px.dF.copy()
        st[name + "_dFy"] = s.py.dF.copy()
        st[name + "_scheme"] = np.array(c, dtype=np.int32)
        if name == "dg":
            st[name + "_ulon_pc"] = s.U_pc.ulon.copy()
            st[name + "_vlat_pc"] = s.U_pc.vlat.copy()
    np.savez_compressed(os.path.join(HERE, "stages_N16.npz"), N=16, dt=0.01, ic=3, vf=2, step=3, **st)

    # ---------------------------------------------------------------- runs
    runs = {}
    for name, (dt, ic, vf, c, nsteps) in {
        "default": (0.0025 * 8, 2, 1, (3, 1, 1, 3, 1, 3), 40),
        "cw84_rk2": (0.01, 2, 2, (2, 2, 1, 3, 1, 3), 30),
    }.items():
        mod, g, s = rh.make_sim(16, dt, 5.0, ic, vf, 1, *c)
        it = interior(g)
        mass0, _ = mod.diagnostics.mass_computation(s.Q, g, 1.0)
        errs, mass = [], []
        for k in range(1, nsteps + 1):
            t = k * s.dt
            mod.advection_timestep.adv_time_step(g, s, k, t)
            qex = mod.advection_ic.qexact_adv(g.pc.lon[it], g.pc.lat[it], t, s)
            errs.append(mod.errors.compute_errors(s.Q[it], qex))
            mass.append(mod.diagnostics.mass_computation(s.Q, g, mass0))
            mod.advection_timestep.update_adv(g, s, t)
        runs[name + "_Q"] = s.Q[it].copy()
        runs[name + "_errors"] = np.array(errs)
        runs[name + "_mass"] = np.array(mass)
        runs[name + "_CFL"] = s.CFL
        runs[name + "_cfg"] = np.array([dt, ic, vf, *c, nsteps])
    np.savez_compressed(os.path.join(HERE, "run_N16.npz"), N=16, **runs)

    # ---------------------------------------------------------------- cases
    cs = {}
    g = m.cs_datastruct.cubed_sphere(12, "gnomonic_equiangular", False, False)
    it = interior(g)
    for ic in (1, 2, 3, 4):
        for vf in (1, 2, 3, 4):
            s = m.advection_ic.adv_simulation_par(g, 0.01, 5.0, ic, vf, 1, 3, 1, 1, 3, 1, 3)
            for t in (0.0, 1.3):
                cs["q_ic%d_vf%d_t%s" % (ic, vf, t)] = m.advection_ic.qexact_adv(g.pc.lon[it], g.pc.lat[it], t, s)
    for vf in (1, 2, 3, 4):
        s = m.advection_ic.adv_simulation_par(g, 0.01, 5.0, 2, vf, 1, 3, 1, 1, 3, 1, 3)
        u, v = m.advection_ic.velocity_adv(g.pu.lon, g.pu.lat, 0.7, s)
        cs["ulon_vf%d" % vf] = u
        cs["vlat_vf%d" % vf] = v
    np.savez_compressed(os.path.join(HERE, "cases_N12.npz"), **cs)

    # ---------------------------------------------------------------- par files
    ref_root = os.path.dirname(rh.REF_SRC)
    cwd = os.getcwd()
    os.chdir(ref_root)
    try:
        import contextlib
        import io
        with contextlib.redirect_stdout(io.StringIO()):
            conf = m.configuration.get_parameters()
            adv = m.configuration.get_advection_parameters()
    finally:
        os.chdir(cwd)
    np.savez_compressed(os.path.join(HERE, "par.npz"),
                        configuration=np.array([str(x) for x in conf]),
                        advection=np.array([repr(x) for x in adv]))
    latlon_fixtures(m)
    print("golden fixtures written to", HERE)


def latlon_fixtures(m):
    """ll2cs and nearest_neighbour of the reference (interpolation.py:38-150)."""
    out = {}
    # (lat-lon sizes for which no point lies on a panel edge: the reference indexes past the
    # panel there, interpolation.py:148)
    for N, nlat, nlon in ((16, 46, 91), (48, 90, 180), (25, 31, 63)):
        grid = m.cs_datastruct.cubed_sphere(N, "gnomonic_equiangular", False, False)
        ll = m.cs_datastruct.latlon_grid(nlat, nlon)
        i, j, p = m.interpolation.ll2cs(grid, ll)
        ll.ix, ll.jy, ll.mask = i, j, p
        f = np.arange(N * N * 6, dtype=np.float64).reshape(N, N, 6) * 0.5 - 7.0
        q = m.interpolation.nearest_neighbour(type("F", (), {"f": f})(), grid, ll)
        key = "N%d_%dx%d" % (N, nlat, nlon)
        out[key + "_X"], out[key + "_Y"], out[key + "_Z"] = ll.X, ll.Y, ll.Z
        out[key + "_i"], out[key + "_j"], out[key + "_panel"] = i, j, p
        out[key + "_nn"] = q
    np.savez_compressed(os.path.join(HERE, "latlon.npz"), **out)


if __name__ == "__main__":
    main()
