"""Pin the CPU oracle (oracle/) against golden vectors produced by the reference itself.

The fixtures in tests/golden/ were generated by tests/golden/make_golden.py, which runs the
unmodified reference.  On the machine that generated them the oracle reproduces them
bit for bit; elsewhere (another libm / SIMD dispatch for sin, tan, arctan ...) the grid
can differ in the last bit, so comparisons allow a relative 1e-12 of the field scale.
"""
import os

import numpy as np
import pytest

from oracle import solver, halo
from oracle.grid import CubedSphere
from oracle import cases

RTOL = 1e-12


def load(golden_dir, name):
    return np.load(os.path.join(golden_dir, name))


def assert_close(a, b, rtol=RTOL):
    scale = max(np.max(np.abs(b)), 1e-300)
    err = np.max(np.abs(a - b)) / scale
    assert err <= rtol, "relative max error %.3e > %.1e" % (err, rtol)


def test_grid_geometry(golden_dir):
    z = load(golden_dir, "grid_N12.npz")
    g = CubedSphere(int(z["N"]))
    assert g.dx == float(z["dx"])
    for pn in ("pc", "pu", "pv"):
        ps = getattr(g, pn)
        for f in ("X", "Y", "Z", "lon", "lat", "ex_elon", "ex_elat", "ey_elon", "ey_elat", "det"):
            assert_close(getattr(ps, f), z["%s_%s" % (pn, f)], 1e-14)
        assert_close(getattr(g, "metric_tensor_" + pn), z["%s_metric" % pn], 1e-14)


def test_lagrange_tables(golden_dir):
    z = load(golden_dir, "grid_N12.npz")
    g = CubedSphere(int(z["N"]))
    Wt, Kmin = halo.lagrange_tables(g)
    np.testing.assert_array_equal(Kmin, z["lagrange_kmin_east"].astype(np.int64))
    assert_close(Wt, z["lagrange_w_east"], 1e-13)
    # degree-3 Lagrange weights sum to one
    np.testing.assert_allclose(Wt.sum(axis=2), 1.0, rtol=0, atol=1e-13)


def test_connectivity_table_matches_reference_gathers(golden_dir):
    z = load(golden_dir, "grid_N12.npz")
    g = CubedSphere(int(z["N"]))
    F = z["halo_field"]
    for p in range(6):
        for s, name in ((halo.E, "east"), (halo.W, "west"), (halo.N_, "north"), (halo.S, "south")):
            H = halo.gather(F, g, p, s)  # [depth, along]
            ref = z["halo_" + name][..., p]
            if name == "east":
                exp = ref                     # [g, k], g = depth
            elif name == "west":
                exp = ref[::-1]               # row g <-> depth 3-g
            elif name == "north":
                exp = ref.T                   # [k, g] -> [g, k]
            else:
                exp = ref.T[::-1]
            np.testing.assert_array_equal(H, exp)


def test_connectivity_is_symmetric():
    for (p, s), (q, qs, rev) in halo.CONNECT.items():
        assert halo.CONNECT[(q, qs)] == (p, s, rev)


@pytest.mark.parametrize("vf", [1, 2, 3, 4])
def test_cases(golden_dir, vf):
    z = load(golden_dir, "cases_N12.npz")
    g = CubedSphere(12)
    it = g.interior
    for ic in (1, 2, 3, 4):
        for t in (0.0, 1.3):
            q = cases.qexact_ref(g.pc.lon[it], g.pc.lat[it], t, ic, vf)
            assert_close(q, z["q_ic%d_vf%d_t%s" % (ic, vf, t)], 1e-13)
    u, v = cases.velocity_ref(g.pu.lon, g.pu.lat, 0.7, vf)
    assert_close(u, z["ulon_vf%d" % vf], 1e-13)
    assert_close(v, z["vlat_vf%d" % vf], 1e-13)


def _run(c, vf, N=10, dt=0.02, ic=2, nsteps=3):
    g = CubedSphere(N)
    s = solver.Simulation(g, dt, 5.0, ic, vf, *c)
    solver.run_steps(s, nsteps)
    return s.Q[g.interior]


@pytest.mark.parametrize("vf", [2, 1, 3, 4])
def test_all_option_combos(golden_dir, vf):
    z = load(golden_dir, "combos_N10.npz")
    combos = z["combos_vf%d" % vf]
    Qs = z["Q_vf%d" % vf]
    if vf == 2:
        assert len(combos) == 216
    for c, Qref in zip(combos, Qs):
        assert_close(_run(tuple(int(x) for x in c), vf), Qref)


def test_invalid_combos_rejected(golden_dir):
    z = load(golden_dir, "combos_N10.npz")
    for c, rej in zip(z["invalid_combos"], z["invalid_rejected"]):
        assert rej == 1
        with pytest.raises(solver.OptionError):
            solver.check_options(*[int(x) for x in c])


@pytest.mark.parametrize("name", ["dg", "pl07", "s72"])
def test_stage_arrays(golden_dir, name):
    z = load(golden_dir, "stages_N16.npz")
    c = tuple(int(x) for x in z[name + "_scheme"])
    g = CubedSphere(16)
    s = solver.Simulation(g, float(z["dt"]), 5.0, int(z["ic"]), int(z["vf"]), *c)
    solver.run_steps(s, 2)
    assert_close(s.Q, z[name + "_Q_before"])
    k = int(z["step"])
    solver.adv_time_step(s, k, k * s.dt)
    it = g.interior
    assert_close(s.Q[it], z[name + "_Q_after"][it])
    # ghost cells: ET-DG fills every ghost cell; ET-S72/ET-PL07 corners are never read
    if name == "dg":
        assert_close(s.Q, z[name + "_Q_after"])
        assert_close(s.w["ulon_pc"], z["dg_ulon_pc"])
        assert_close(s.w["vlat_pc"], z["dg_vlat_pc"])
    assert_close(s.div[it], z[name + "_div"][it])
    for key, arr in (("u_pu", s.w["u_pu"]), ("v_pv", s.w["v_pv"]), ("u_avg", s.w["u_pu_avg"]),
                     ("v_avg", s.w["v_pv_avg"]), ("fx", s.f_x), ("fy", s.f_y),
                     ("dFx", s.dF_x), ("dFy", s.dF_y)):
        assert_close(arr, z[name + "_" + key])


@pytest.mark.parametrize("name", ["default", "cw84_rk2"])
def test_long_run_errors_and_mass(golden_dir, name):
    z = load(golden_dir, "run_N16.npz")
    cfg = z[name + "_cfg"]
    dt, ic, vf = float(cfg[0]), int(cfg[1]), int(cfg[2])
    c = tuple(int(x) for x in cfg[3:9])
    nsteps = int(cfg[9])
    g = CubedSphere(int(z["N"]))
    s = solver.Simulation(g, dt, 5.0, ic, vf, *c)
    assert s.CFL == pytest.approx(float(z[name + "_CFL"]), rel=1e-13)
    mass0, _ = solver.mass_computation(s.Q, g, 1.0)
    it = g.interior
    for k in range(1, nsteps + 1):
        t = k * dt
        solver.adv_time_step(s, k, t)
        qex = s.qexact(g.pc.lon[it], g.pc.lat[it], t)
        e = solver.compute_errors(s.Q[it], qex)
        np.testing.assert_allclose(e, z[name + "_errors"][k - 1], rtol=1e-10)
        m, dm = solver.mass_computation(s.Q, g, mass0)
        np.testing.assert_allclose(m, z[name + "_mass"][k - 1][0], rtol=1e-12)
        solver.update_adv(s, t)
    assert_close(s.Q[it], z[name + "_Q"])


def test_latlon_oracle_matches_reference(golden_dir):
    """ll2cs / nearest_neighbour restated (oracle/latlon.py) against the reference's own output."""
    from oracle import latlon
    z = np.load(os.path.join(golden_dir, "latlon.npz"))
    keys = sorted({k.rsplit("_", 1)[0] for k in z.files})
    assert len(keys) == 3
    for key in keys:
        N = int(key.split("_")[0][1:])
        i, j, p = latlon.ll2cs(N, z[key + "_X"], z[key + "_Y"], z[key + "_Z"])
        np.testing.assert_array_equal(i, z[key + "_i"])
        np.testing.assert_array_equal(j, z[key + "_j"])
        np.testing.assert_array_equal(p, z[key + "_panel"])
        f = np.arange(N * N * 6, dtype=np.float64).reshape(N, N, 6) * 0.5 - 7.0
        np.testing.assert_array_equal(latlon.nearest_neighbour(f, i, j, p), z[key + "_nn"])


def test_parameterised_cases_reproduce_the_reference_default_run(golden_dir):
    """Known answer for the benchmark cases: solid-body wind 101 with alpha = -pi/4, u0 = 2 pi/5
    and Gaussian hill 101 at (pi/4, pi/6) with b0 = 10 are the reference's own vf = 1 wind and
    ic = 2 hill (advection_ic.py:221-246, :288-292), so the oracle run with them must reproduce
    the reference's 40-step default run: fields, per-step errors against the exact rotated
    hill, and mass."""
    import math
    z = load(golden_dir, "run_N16.npz")
    cfg = z["default_cfg"]
    dt = float(cfg[0])
    c = tuple(int(x) for x in cfg[3:9])
    nsteps = int(cfg[9])
    assert (int(cfg[1]), int(cfg[2])) == (2, 1)
    g = CubedSphere(int(z["N"]))
    it = g.interior
    wind = cases.WindSpec("solid", alpha=-math.pi / 4.0, u0=2.0 * math.pi / 5.0)
    hill = cases.ICSpec("hill", lon=math.pi / 4.0, lat=math.pi / 6.0, b0=10.0)
    s = solver.Simulation(g, dt, 5.0, 0, 0, *c, ic_spec=hill, wind=wind,
                          q0=hill(g.pc.lon[it], g.pc.lat[it]))
    assert s.CFL == pytest.approx(float(z["default_CFL"]), rel=1e-13)
    for k in range(1, nsteps + 1):
        t = k * dt
        solver.adv_time_step(s, k, t)
        e = solver.compute_errors(s.Q[it], s.qexact(g.pc.lon[it], g.pc.lat[it], t))
        np.testing.assert_allclose(e, z["default_errors"][k - 1], rtol=1e-10)
        m, _ = solver.mass_computation(s.Q, g, 1.0)
        np.testing.assert_allclose(m, z["default_mass"][k - 1][0], rtol=1e-12)
        solver.update_adv(s, t)
    assert_close(s.Q[it], z["default_Q"])
