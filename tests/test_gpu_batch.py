"""GPU tests of batches (many solves, one step-kernel launch per step) and the tile autotuner.

The bar: a solve gives the SAME BITS alone and in a batch (the step kernel's mass-fixer
sums run in a fixed order per solve), whatever the other members, their sizes, winds and
tracer counts, and across membership changes.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCHEME = dict(recon=2, dp=2, opsplit=1, et=3, mt=1, mf=3)


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build()


# (N, tracers, wind, wind_param, ic list)
MEMBERS = [
    (24, 1, 101, (0.7, 2 * np.pi / 5, 0, 0), [(101, (0.3, -0.2, 5.0, 0))]),
    (40, 2, 102, (0.48, 5.0, 0, 0), [(102, None), (103, None)]),
    (61, 3, 101, (1.2, 2 * np.pi / 5, 0, 0), [(101, (1.0, 0.4, 8.0, 0)), (102, None), (101, (-2.0, -0.5, 3.0, 0))]),
    (130, 1, 102, (0.48, 5.0, 0, 0), [(103, None)]),
    (16, 2, 103, (0.3, 2 * np.pi / 5, 0.3, 0), [(101, (0.0, 0.0, 5.0, 0)), (101, (3.0, 0.2, 4.0, 0))]),
]


def make(member, precision, dt_scale=0.5, **kw):
    from csadv import Plan
    N, T, vf, wp, ics = member
    dt = dt_scale / N * 0.5
    pl = Plan(N, dt, vf=vf, wind_param=wp, ntracers=T, precision=precision, **SCHEME, **kw)
    for t, (ic, prm) in enumerate(ics):
        pl.init_tracer(ic, ic_param=prm, tracer=t)
    return pl


def state(pl):
    return [pl.get_tracer(t) for t in range(pl.ntracers)]


@pytest.mark.parametrize("precision", [32, 64])
def test_batch_results_identical_to_alone(precision):
    from csadv import Batch
    nsteps = 7
    alone = []
    for m in MEMBERS:
        with make(m, precision) as pl:
            pl.advance(nsteps)
            alone.append((state(pl), pl.mass(), pl.step))
    plans = [make(m, precision) for m in MEMBERS]
    with Batch(8) as b:
        for pl in plans:
            b.add(pl)
        assert len(b) == len(MEMBERS)
        b.advance(3)
        b.advance(nsteps - 3)
        st = b.stats()
        assert st["steps"] == nsteps
        for pl, (ref, mass, k) in zip(plans, alone):
            for a, r in zip(state(pl), ref):
                np.testing.assert_array_equal(a, r)
            assert pl.mass() == mass
            assert pl.step == k
    for pl in plans:
        pl.close()


def test_batch_membership_changes_keep_results():
    # a solve that joins late, one that leaves, one stepped alone in between: each ends
    # with the bits of the same steps taken alone
    from csadv import Batch
    ref = {}
    for i, m in enumerate(MEMBERS[:3]):
        with make(m, 32) as pl:
            pl.advance(6)
            ref[i] = state(pl)
    p0, p1, p2 = (make(m, 32) for m in MEMBERS[:3])
    with Batch(4) as b:
        b.add(p0)
        b.add(p1)
        b.advance(2)
        b.add(p2)          # p2 joins at its step 0
        b.advance(2)
        b.remove(p1)       # p1 at step 4 continues alone
        p1.advance(2)
        b.advance(1)       # p0 at 5, p2 at 3
        p0.advance(1)      # attached plan stepped outside the batch (p0 at 6): the batch rebuilds
        b.remove(p0)
        b.advance(3)       # p2 at 6
        for pl, i in ((p0, 0), (p1, 1), (p2, 2)):
            assert pl.step == 6
            for a, r in zip(state(pl), ref[i]):
                np.testing.assert_array_equal(a, r)
    for pl in (p0, p1, p2):
        pl.close()


def test_batch_rejects_incompatible_plans():
    from csadv import Batch, CsadvError, Plan
    with Batch(2) as b, make(MEMBERS[0], 32) as a, make(MEMBERS[1], 64) as c, \
            Plan(24, 0.01, vf=1, engine=1, **SCHEME) as staged, Plan(24, 0.01, vf=1, tile=1, **SCHEME) as old:
        b.add(a)
        for bad in (c, staged, old):
            with pytest.raises(CsadvError):
                b.add(bad)
        with make(MEMBERS[2], 32) as d, make(MEMBERS[3], 32) as e:
            b.add(d)
            with pytest.raises(CsadvError):  # capacity 2
                b.add(e)
            b.remove(d)


def test_destroying_attached_plan_detaches_it():
    from csadv import Batch
    with Batch(4) as b:
        a, c = make(MEMBERS[0], 32), make(MEMBERS[1], 32)
        b.add(a)
        b.add(c)
        b.advance(1)
        b._plans.remove(a)
        a.close()
        assert len(b) == 1
        b.advance(1)
        assert c.step == 2
        c.close()


def test_tune_keeps_state_and_is_remembered():
    from csadv import tune
    m = (72, 2, 102, (0.48, 5.0, 0, 0), [(102, None), (103, None)])
    with make(m, 32) as pl:  # tuning does not change the state
        pl.advance(2)
        before = state(pl)
        tile = tune(pl, reps=2)
        assert 5 <= tile <= 8
        assert pl.stats()["tile"] == tile
        for a, r in zip(state(pl), before):
            np.testing.assert_array_equal(a, r)
    with make(m, 32) as pl, make(m, 32, tile=tile) as ref:  # nor the steps after it
        pl.advance(2)
        assert tune(pl, reps=1) == tile
        pl.advance(2)
        ref.advance(4)
        for a, r in zip(state(pl), state(ref)):
            np.testing.assert_array_equal(a, r)
    with make(m, 32) as later:  # default tile = the tuned one
        assert later.stats()["tile"] == tile


def test_queue_depth_keeps_results():
    """With the host held at most one or three advance calls ahead of the GPU the batch gives the
    same bits as without; depths outside 0..64 are refused."""
    from csadv import Batch, CsadvError
    ref = []
    for depth in (0, 1, 3):
        plans = [make(m, 32) for m in MEMBERS[:3]]
        with Batch(8) as b:
            b.set_queue_depth(depth)
            for pl in plans:
                b.add(pl)
            for _ in range(7):
                b.advance(2)
            out = [pl.get_tracer(t) for pl in plans for t in range(pl.ntracers)]
            for pl in plans:
                b.remove(pl)
        for pl in plans:
            pl.close()
        if depth == 0:
            ref = out
        else:
            for a, r in zip(out, ref):
                np.testing.assert_array_equal(a, r)
    with Batch(2) as b:
        with pytest.raises(CsadvError):
            b.set_queue_depth(65)
