"""GPU tests of failure reporting and isolation, and of a symmetry of the discrete scheme.

* A NaN seeded in one solve of a batch stays in that solve: the other members give the bits they
  give alone, and the seeded one reports CSADV_ERR_NONFINITE from its diagnostics.
* Blow-up: errors above 100 are reported as CSADV_ERR_BLOWUP, and the reference mirror stops
  with SystemExit as output.py:44-47 does.
* Turning the problem by 180 degrees of longitude (a solid-body wind about the polar axis and a
  hill moved by pi) maps panel p to p + 2 (mod 4) with the same local indices and turns each
  polar panel about its centre: the fields agree under that map and the error norms agree, to
  1e-12 relative (the per-panel tangent-vector formulas and atan2 round differently, so not bit
  for bit).  A quarter turn is not a symmetry of the scheme: it swaps the local axes of the
  polar panels, whose corner ghost cells are filled in a fixed order (interpolation.py:250-314).
"""
import ctypes
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCHEME = dict(recon=2, dp=2, opsplit=1, et=3, mt=1, mf=3)


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build()


MEMBERS = [  # (N, tracers, wind, wind_param, [(ic, ic_param)])
    (24, 1, 101, (0.7, 2 * math.pi / 5, 0, 0), [(101, (0.3, -0.2, 5.0, 0))]),
    (40, 2, 102, (0.48, 5.0, 0, 0), [(102, None), (103, None)]),
    (33, 3, 101, (1.2, 2 * math.pi / 5, 0, 0), [(101, (1.0, 0.4, 8.0, 0)), (102, None), (103, None)]),
]


def make(member, precision):
    from csadv import Plan
    N, T, vf, wp, ics = member
    pl = Plan(N, 0.25 / N, vf=vf, wind_param=wp, ntracers=T, precision=precision, **SCHEME)
    for t, (ic, prm) in enumerate(ics):
        pl.init_tracer(ic, ic_param=prm, tracer=t)
    return pl


@pytest.mark.parametrize("precision", [32, 64])
def test_nan_in_one_solve_stays_in_that_solve(precision):
    from csadv import Batch, CsadvError, _lib
    nsteps = 5
    alone = {}
    for m in (0, 2):
        with make(MEMBERS[m], precision) as pl:
            pl.advance(nsteps)
            alone[m] = [pl.get_tracer(t) for t in range(pl.ntracers)]
    plans = [make(m, precision) for m in MEMBERS]
    try:
        bad = plans[1]
        q = bad.get_tracer(0, full=True)
        q[10, 12, 3] = np.nan
        bad.set_tracer(q, tracer=0)
        with Batch(4) as b:
            for pl in plans:
                b.add(pl)
            b.advance(nsteps)
            for m in (0, 2):
                for t in range(plans[m].ntracers):
                    np.testing.assert_array_equal(plans[m].get_tracer(t), alone[m][t])
            assert np.isnan(bad.get_tracer(0)).any()
            with pytest.raises(CsadvError) as e:
                bad.errors(102, bad.step * bad.dt, tracer=0)
            assert e.value.status == _lib.ERR_NONFINITE
    finally:
        for pl in plans:
            pl.close()


def test_blowup_is_reported():
    from csadv import CsadvError, Plan, _lib
    with Plan(16, 0.01, vf=1, precision=64, **SCHEME) as pl:
        pl.init_tracer(1)
        q = pl.get_tracer(0, full=True) * 1e3
        pl.set_tracer(q)
        out = (ctypes.c_double * 3)()
        rc = _lib.lib().csadv_errors(pl._h, 0, 1, None, 0.0, out, pl.stream)
        assert rc == _lib.ERR_BLOWUP and out[0] > 100.0
        linf, _, _ = pl.errors(1, 0.0)          # reported, not raised, by default
        assert linf > 100.0
        with pytest.raises(CsadvError):
            pl.errors(1, 0.0, raise_blowup=True)


def test_reference_mirror_stops_on_blowup():
    from csadv import advection
    cs = advection.cubed_sphere(16)
    sim = advection.adv_simulation_par(cs, 0.01, 0.05, 1, 1, 1, 2, 2, 1, 3, 1, 3)
    advection.init_vars_adv(cs, sim)
    # the per-step error arrays that adv_sphere allocates before its first output
    sim.error_linf, sim.error_l1, sim.error_l2 = np.zeros(6), np.zeros(6), np.zeros(6)
    sim.Q = sim.Q * 1e3
    with pytest.raises(SystemExit):
        advection.output_adv(cs, None, sim, False, 5, 0.05, 5, 1, "sphere", False)


def rotate_half(Q):
    """Q of the problem turned by 180 degrees of longitude, from Q of the original problem
    (interior arrays [i][j][panel])."""
    R = np.empty_like(Q)
    for p in range(4):
        R[:, :, (p + 2) % 4] = Q[:, :, p]
    for p in (4, 5):  # the point of local (x, y) goes to local (-x, -y)
        R[:, :, p] = Q[::-1, ::-1, p]
    return R


@pytest.mark.parametrize("N", [24, 31])
def test_half_turn_symmetry(N):
    from csadv import Plan
    wp = (0.0, 2 * math.pi / 5, 0, 0)  # solid body about the polar axis
    hill = (0.3, 0.25, 5.0, 0)
    turned = (0.3 + math.pi, 0.25, 5.0, 0)
    with Plan(N, 0.3 / N, vf=101, wind_param=wp, precision=64, **SCHEME) as a, \
            Plan(N, 0.3 / N, vf=101, wind_param=wp, precision=64, **SCHEME) as b:
        a.init_tracer(101, ic_param=hill)
        b.init_tracer(101, ic_param=turned)
        np.testing.assert_allclose(rotate_half(a.get_tracer()), b.get_tracer(), rtol=0, atol=1e-13)
        a.advance(12)
        b.advance(12)
        qa, qb = a.get_tracer(), b.get_tracer()
        scale = np.max(np.abs(qa))
        np.testing.assert_allclose(rotate_half(qa), qb, rtol=0, atol=1e-12 * scale)
        ea = a.errors(101, a.step * a.dt, ic_param=hill)
        eb = b.errors(101, b.step * b.dt, ic_param=turned)
        np.testing.assert_allclose(ea, eb, rtol=1e-10)
