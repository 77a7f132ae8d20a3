"""GPU parity of the FP64 ("plain") form against the reference.

Each test drives libcsadv through its C ABI (csadv.Plan wraps the ctypes calls) and
compares with golden vectors from the reference (tests/golden/) or with the CPU oracle on
the same inputs.  Tolerance: |gpu - ref| <= RTOL * max|ref| with RTOL = 1e-12 (the
parity bar for the FP64 form).  Differences come only from CUDA's transcendental
functions in the geometry and winds (within 2 ulp of libm) and from reduction order.
"""
import os

import numpy as np
import pytest

from oracle import solver
from oracle.grid import CubedSphere

pytestmark = pytest.mark.gpu

RTOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build()


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def plan(N, dt, c, vf, **kw):
    from csadv import Plan
    recon, dp, sp, et, mt, mf = c
    return Plan(N, dt, recon=recon, dp=dp, opsplit=sp, et=et, mt=mt, mf=mf, vf=vf, **kw)


@pytest.mark.parametrize("vf", [2, 1, 3, 4])
def test_every_option_combination_vs_reference_golden(golden_dir, vf):
    z = np.load(os.path.join(golden_dir, "combos_N10.npz"))
    combos, Qs = z["combos_vf%d" % vf], z["Q_vf%d" % vf]
    worst = 0.0
    for c, Qref in zip(combos, Qs):
        with plan(10, float(z["dt"]), tuple(int(x) for x in c), vf) as pl:
            pl.init_tracer(int(z["ic"]))
            pl.advance(int(z["nsteps"]))
            e = rel(pl.get_tracer(), Qref)
        assert e <= RTOL, (tuple(c), e)
        worst = max(worst, e)
    print("vf=%d: %d combos, worst relative difference %.2e" % (vf, len(combos), worst))


@pytest.mark.parametrize("name", ["default", "cw84_rk2"])
def test_errors_and_mass_each_step_vs_reference(golden_dir, name):
    z = np.load(os.path.join(golden_dir, "run_N16.npz"))
    cfg = z[name + "_cfg"]
    dt, ic, vf = float(cfg[0]), int(cfg[1]), int(cfg[2])
    c = tuple(int(x) for x in cfg[3:9])
    nsteps = int(cfg[9])
    with plan(int(z["N"]), dt, c, vf) as pl:
        pl.init_tracer(ic)
        assert pl.cfl == pytest.approx(float(z[name + "_CFL"]), rel=1e-12)
        for k in range(1, nsteps + 1):
            pl.time_step(k)
            e = pl.errors(ic, k * dt)
            np.testing.assert_allclose(e, z[name + "_errors"][k - 1], rtol=1e-10)
            np.testing.assert_allclose(pl.mass(), z[name + "_mass"][k - 1][0], rtol=1e-12)
            pl.update_winds(k * dt)
        assert rel(pl.get_tracer(), z[name + "_Q"]) <= RTOL


@pytest.mark.parametrize("name", ["dg", "pl07", "s72"])
def test_divergence_and_halo_vs_reference_stages(golden_dir, name):
    z = np.load(os.path.join(golden_dir, "stages_N16.npz"))
    c = tuple(int(x) for x in z[name + "_scheme"])
    with plan(16, float(z["dt"]), c, int(z["vf"])) as pl:
        pl.init_tracer(int(z["ic"]))
        pl.advance(2)
        assert rel(pl.get_tracer(full=True)[4:20, 4:20], z[name + "_Q_before"][4:20, 4:20]) <= RTOL
        div = pl.divergence()
        # the golden div is the reference's after MF (mass fixer) of step 3
        assert rel(div, z[name + "_div"][4:20, 4:20]) <= 1e-11
        pl.time_step(3)
        full = pl.get_tracer(full=True)
        assert rel(full[4:20, 4:20], z[name + "_Q_after"][4:20, 4:20]) <= RTOL
        if name == "dg":  # every ghost cell, corners included
            assert rel(full, z[name + "_Q_after"]) <= RTOL


@pytest.mark.parametrize("c,vf,ic", [((2, 2, 1, 3, 1, 3), 2, 3), ((3, 1, 1, 3, 1, 3), 1, 2),
                                     ((4, 2, 2, 3, 1, 2), 3, 2), ((3, 2, 3, 2, 2, 1), 2, 3),
                                     ((1, 1, 1, 1, 1, 3), 4, 4)])
def test_oracle_parity_N48(c, vf, ic):
    N, dt, nsteps = 48, 0.004, 12
    g = CubedSphere(N)
    sim = solver.Simulation(g, dt, 5.0, ic, vf, *c)
    solver.run_steps(sim, nsteps)
    with plan(N, dt, c, vf) as pl:
        pl.init_tracer(ic)
        pl.advance(nsteps)
        assert rel(pl.get_tracer(), sim.Q[g.interior]) <= RTOL


def test_set_get_roundtrip_and_layouts():
    rng = np.random.default_rng(1)
    with plan(12, 0.01, (3, 1, 1, 3, 1, 3), 1) as pl:
        full = rng.standard_normal((20, 20, 6))
        pl.set_tracer(full)
        np.testing.assert_array_equal(pl.get_tracer(full=True), full)
        inner = rng.standard_normal((12, 12, 6))
        pl.set_tracer(inner)
        np.testing.assert_array_equal(pl.get_tracer(), inner)
        with pytest.raises(ValueError):
            pl.set_tracer(np.zeros((5, 5, 6)))


def test_set_get_page_locked_host_memory():
    """Page-locked host arrays are read and written by the device directly (no staging copy):
    the same fields as through pageable arrays, for both layouts, FP64 and FP32 state, across a
    step with a pending MF-PR correction."""
    import ctypes
    from csadv import Plan, _lib
    L = _lib.lib()
    rng = np.random.default_rng(7)
    N, n = 16, 24
    bufs = []
    try:
        for shp in ((n, n, 6), (N, N, 6)):
            p = ctypes.c_void_p()
            _lib.check(L.csadv_host_alloc(ctypes.byref(p), int(np.prod(shp)) * 8))
            bufs.append((p, np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_double)), shape=shp)))
        for prec in (64, 32):
            with Plan(N, 0.01, recon=2, dp=2, opsplit=1, et=3, mt=1, mf=3, vf=2, ntracers=2, precision=prec) as pa, \
                    Plan(N, 0.01, recon=2, dp=2, opsplit=1, et=3, mt=1, mf=3, vf=2, ntracers=2, precision=prec) as pb:
                full = 1.0 + 0.1 * rng.standard_normal((n, n, 6))
                bufs[0][1][...] = full
                pa.set_tracer(full, tracer=1)
                _lib.check(L.csadv_set_tracer(pb._h, 1, bufs[0][0], _lib.LAYOUT_FULL, pb.stream))
                pa.init_tracer(2)
                pb.init_tracer(2)
                pa.advance(3)
                pb.advance(3)
                for t in range(2):
                    for k, full_layout in ((0, True), (1, False)):
                        _lib.check(L.csadv_get_tracer(pb._h, t, bufs[k][0],
                                                      _lib.LAYOUT_FULL if full_layout else _lib.LAYOUT_INTERIOR,
                                                      pb.stream))
                        np.testing.assert_array_equal(bufs[k][1], pa.get_tracer(t, full=full_layout))
                inner = rng.standard_normal((N, N, 6))
                bufs[1][1][...] = inner
                _lib.check(L.csadv_set_tracer(pb._h, 0, bufs[1][0], _lib.LAYOUT_INTERIOR, pb.stream))
                np.testing.assert_array_equal(pb.get_tracer(0), inner if prec == 64 else inner.astype(np.float32))
    finally:
        for p, _ in bufs:
            L.csadv_host_free(p)


def test_several_tracers_equal_single_runs():
    c, vf, dt = (2, 2, 1, 3, 1, 3), 2, 0.01
    with plan(16, dt, c, vf, ntracers=3) as pl:
        for t, ic in enumerate((2, 3, 4)):
            pl.init_tracer(ic, tracer=t)
        pl.advance(6)
        multi = [pl.get_tracer(t) for t in range(3)]
    for t, ic in enumerate((2, 3, 4)):
        with plan(16, dt, c, vf) as pl:
            pl.init_tracer(ic)
            pl.advance(6)
            np.testing.assert_array_equal(pl.get_tracer(), multi[t])


def test_minimum_grid_size_runs():
    with plan(8, 0.02, (2, 2, 1, 3, 1, 3), 2) as pl:
        pl.init_tracer(2)
        pl.advance(3)
        assert np.all(np.isfinite(pl.get_tracer()))


def test_linearity_of_the_unlimited_scheme_large_N():
    # PPM-PL07 + ET-DG + MF-PR is linear in Q: step(2 q0 - q1/2) = 2 step(q0) - step(q1)/2
    with plan(384, 0.0025, (3, 2, 1, 3, 1, 3), 2, ntracers=3) as pl:
        pl.init_tracer(2, tracer=0)
        pl.init_tracer(3, tracer=1)
        a, b = pl.get_tracer(0, full=True), pl.get_tracer(1, full=True)
        pl.set_tracer(2.0 * a - 0.5 * b, tracer=2)
        pl.advance(4)
        q0, q1, q2 = (pl.get_tracer(t) for t in range(3))
        assert rel(q2, 2.0 * q0 - 0.5 * q1) < 1e-12


def test_runs_are_deterministic_large_N():
    outs = []
    for _ in range(2):
        with plan(384, 0.0025, (2, 2, 1, 3, 1, 3), 2) as pl:
            pl.init_tracer(2)
            pl.advance(3)
            outs.append(pl.get_tracer())
    np.testing.assert_array_equal(outs[0], outs[1])


def test_mass_conserved_with_projection_large_N():
    with plan(384, 0.0025, (2, 2, 1, 3, 1, 3), 2) as pl:
        pl.init_tracer(3)
        m0 = pl.mass()
        pl.advance(8)
        assert abs(pl.mass() - m0) / abs(m0) < 1e-13
