"""Accuracy runs to their end times: one full revolution at N = 48 and the deformational flow at
N = 384 to t = T, in FP64 and FP32, with the reference's end-of-run error norms
(advection_sphere.py:45-61 with errors.py:99-113: unweighted Linf, mean |E|, RMS of |E| over
the interior against the exact solution) and mass (diagnostics.py:14-26).

The time step comes from the reference's CFL definition (advection_vars.py:89-98) at CFL 0.5,
rounded down so that a whole number of steps ends exactly at the final time.
"""
import math

import numpy as np
import pytest

from oracle import cases, solver
from oracle.grid import CubedSphere

pytestmark = pytest.mark.gpu

SCHEME = dict(recon=2, dp=2, opsplit=1, et=3, mt=1, mf=3)  # PPM-CW84 RK2 AVLT ET-DG MT-0 MF-PR


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build()


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def steps_to(N, vf, wp, tf, cfl=0.5):
    """(nsteps, dt): the smallest whole number of steps reaching tf at CFL <= cfl."""
    from csadv import Plan
    with Plan(N, -cfl, vf=vf, wind_param=wp, **SCHEME) as pl:
        n = int(math.ceil(tf / pl.dt - 1e-9))
    return n, tf / n


def run(N, dt, nsteps, vf, wp, ics, precision):
    """Fields, errors at the end time and relative mass change of each tracer."""
    from csadv import Plan
    with Plan(N, dt, vf=vf, wind_param=wp, ntracers=len(ics), precision=precision, **SCHEME) as pl:
        for t, (ic, ip) in enumerate(ics):
            pl.init_tracer(ic, ic_param=ip, tracer=t)
        m0 = [pl.mass(t) for t in range(len(ics))]
        pl.advance(nsteps)
        out = []
        for t, (ic, ip) in enumerate(ics):
            dm = abs(pl.mass(t) - m0[t]) / abs(m0[t])
            out.append((pl.get_tracer(t), np.array(pl.errors(ic, nsteps * dt, ic_param=ip, tracer=t)), dm))
        return out


def test_one_revolution_N48_fp64_and_fp32():
    """N = 48, Gaussian hill b0 = 5 at (0, 0), solid-body rotation at alpha = pi/4 with
    u0 = 2 pi/5 (one revolution in T = 5), CFL 0.5: 614 steps.  FP64 against the oracle's run of
    the same steps (the whole revolution) and the exact rotated hill; FP32 L2 within 1 % of
    FP64's, mass within 1e-6 (MF-PR)."""
    N, vf, wp = 48, 101, (math.pi / 4.0, 2.0 * math.pi / 5.0, 0.0, 0.0)
    hill = (101, (0.0, 0.0, 5.0, 0.0))
    nsteps, dt = steps_to(N, vf, wp, 5.0)
    assert nsteps == 614
    (q64, e64, dm64), = run(N, dt, nsteps, vf, wp, [hill], 64)
    (q32, e32, dm32), = run(N, dt, nsteps, vf, wp, [hill], 32)
    g = CubedSphere(N)
    it = g.interior
    w = cases.WindSpec("solid", alpha=wp[0], u0=wp[1])
    ic = cases.ICSpec("hill", lon=0.0, lat=0.0, b0=5.0)
    s = solver.Simulation(g, dt, 5.0, 0, 0, 2, 2, 1, 3, 1, 3, ic_spec=ic, wind=w, q0=ic(g.pc.lon[it], g.pc.lat[it]))
    assert s.CFL <= 0.5
    eo = np.array(solver.adv_sphere(s, nsteps))
    print("N=48 one revolution (%d steps, dt %.6e): FP64 Linf/L1/L2 %s, oracle %s, FP32 %s; "
          "FP64 vs oracle %.2e, FP32 vs oracle %.2e; mass change FP64 %.2e FP32 %.2e"
          % (nsteps, dt, e64, eo, e32, rel(q64, s.Q[it]), rel(q32, s.Q[it]), dm64, dm32))
    assert rel(q64, s.Q[it]) <= 1e-12
    assert rel(q32, s.Q[it]) < 1e-4  # the FP32 form against the oracle directly
    np.testing.assert_allclose(e64, eo, rtol=1e-9)
    assert dm64 < 1e-13
    assert abs(e32[2] - e64[2]) <= 0.01 * e64[2]
    assert dm32 < 1e-6
    assert rel(q32, q64) < 1e-4


def test_deformational_flow_N384_to_T_fp64_and_fp32():
    """N = 384, cosine bells and smooth bells in the deformational wind (k = 0.48, T = 5), to
    t = T where the exact solution is the initial field; mass within 1e-6 (FP32) and 1e-12 (FP64).

    The cosine bells' FP32 L2 error is within 1 % of FP64's.  The smooth bells (0.95 + 0.05 h)
    have an FP64 L2 error of about 2e-6 at this resolution, some 35 float32 ulps of their values
    (~1): the FP32 state is rounded to 2^-24 relative at every one of the ~4800 steps, so its
    error is bounded by FP64's plus that rounding's random walk, sqrt(steps) 2^-24 max|q|, and
    not by 1 % of FP64's."""
    N, vf, wp = 384, 102, (0.48, 5.0, 0.0, 0.0)
    ics = [(102, None), (103, None)]
    nsteps, dt = steps_to(N, vf, wp, 5.0)
    r64 = run(N, dt, nsteps, vf, wp, ics, 64)
    r32 = run(N, dt, nsteps, vf, wp, ics, 32)
    for t in range(2):
        q64, e64, dm64 = r64[t]
        q32, e32, dm32 = r32[t]
        print("N=384 deformational to t=T (%d steps), tracer %d: FP64 %s FP32 %s; FP32 vs FP64 %.2e; "
              "mass change FP64 %.2e FP32 %.2e" % (nsteps, t, e64, e32, rel(q32, q64), dm64, dm32))
        if t == 0:
            assert abs(e32[2] - e64[2]) <= 0.01 * e64[2]
        walk = math.sqrt(nsteps) * 2.0 ** -24 * np.max(np.abs(q64))
        assert e32[2] <= 1.01 * e64[2] + walk
        assert dm64 < 1e-12
        assert dm32 < 1e-6
        assert rel(q32, q64) < 1e-3


def test_fp32_mass_sums_hold_at_N1536():
    """The FP32 form sums its MF-PR partials (sum of Q g per tracer) in FP32 within a thread's
    march line (up to 55 cells) and a warp's butterfly, and in FP64 across warps and CTAs.  At
    N = 1536 (14.2 M cells per tracer, 4704 tiles), an error e in those sums would move each
    tracer's mass by about e: over 50 steps of the divergent wind at CFL 0.7 the mass, computed in
    FP64 from the FP32 state, stays within 1e-7 of its initial value (the FP32 state's own
    rounding is 6e-8 per cell)."""
    from csadv import Plan
    kw = dict(vf=103, wind_param=(math.pi / 4, 2 * math.pi / 5, 0.3, 0.0), ntracers=2, precision=32, **SCHEME)
    with Plan(1536, -0.7, **kw) as pl:
        pl.init_tracer(101, ic_param=(0.0, 0.2, 5.0, 0.0), tracer=0)
        pl.init_tracer(102, tracer=1)
        m0 = [pl.mass(t) for t in range(2)]
        pl.advance(50)
        dm = [abs(pl.mass(t) - m0[t]) / abs(m0[t]) for t in range(2)]
        q = pl.get_tracer(0)
    print("N=1536 FP32, 50 steps: relative mass change %s" % dm)
    assert np.all(np.isfinite(q))
    assert max(dm) < 1e-7
