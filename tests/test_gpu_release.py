"""GPU tests of csadv_plan_release: a plan freed in the order of a stream, without waiting for the
device, returns its memory (and its grid, when no other plan shares it) to the library's pool.

The bar: plans made from memory that released plans left behind, while the released plans' work
may still be queued, give the same bits as plans made on a fresh device; a plan that shares its
grid with a released plan is unaffected; a released plan leaves its batch.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HILL = (101, (0.0, 0.0, 5.0, 0.0))
SCHEME = dict(recon=2, dp=2, opsplit=1, et=3, mt=1, mf=3, vf=101, wind_param=(0.7, 1.2, 0.0, 0.0))


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build()


def make(N, precision, stream=None, lon=0.0):
    from csadv import Plan
    pl = Plan(N, -0.5, ntracers=1, precision=precision, stream=stream, **SCHEME)
    pl.init_tracer(HILL[0], ic_param=(lon, 0.0, 5.0, 0.0))
    return pl


def alone(N, precision, steps, lon=0.0):
    with make(N, precision, lon=lon) as pl:
        pl.advance(steps)
        return pl.get_tracer(0)


@pytest.mark.parametrize("precision", [32, 64])
def test_memory_of_released_plans_reused_bit_exact(precision):
    """Plans released while their steps may still run, then new plans of the same and other sizes
    made at once from the pool on another stream: every field equals the one run alone."""
    import torch
    sa, sb = torch.cuda.Stream(), torch.cuda.Stream()
    want = {N: alone(N, precision, 12, lon=0.3) for N in (40, 64)}
    for rep in range(3):
        old = [make(N, precision, stream=sa, lon=1.0) for N in (40, 64, 64)]
        for pl in old:
            pl.advance(20)  # queued on sa
        for pl in old:
            pl.release()  # nothing waits: freed in sa's order
        new = [make(N, precision, stream=sb, lon=0.3) for N in (64, 40)]
        for pl in new:
            pl.advance(12)
            np.testing.assert_array_equal(pl.get_tracer(0), want[pl.N])
            pl.release()
    torch.cuda.synchronize()


def test_shared_grid_survives_release_of_other_plan():
    """Two plans share the N = 48 grid; the first is released mid-run on its stream, the second
    keeps stepping on another stream and then releases the grid itself; a third plan rebuilds it."""
    import torch
    sa, sb = torch.cuda.Stream(), torch.cuda.Stream()
    want = alone(48, 64, 30)
    p1 = make(48, 64, stream=sa, lon=2.0)
    p2 = make(48, 64, stream=sb)
    p1.advance(40)
    p2.advance(10)
    p1.release()
    p2.advance(20)
    np.testing.assert_array_equal(p2.get_tracer(0), want)
    p2.release()
    p3 = make(48, 64, stream=sa)
    p3.advance(30)
    np.testing.assert_array_equal(p3.get_tracer(0), want)
    p3.close()


def test_release_detaches_from_batch():
    """A plan released while attached to a batch leaves it; the batch's other plan steps on and
    gives the same bits as run alone."""
    import torch
    from csadv import Batch
    st = torch.cuda.Stream()
    want = alone(56, 32, 16)
    keep, gone = make(56, 32, stream=st), make(72, 32, stream=st, lon=1.0)
    with Batch(4) as b:
        b.add(keep)
        b.add(gone)
        b.advance(8, st)
        gone.release(st)
        assert len(b) == 1
        b.advance(8, st)
        np.testing.assert_array_equal(keep.get_tracer(0), want)
        b.remove(keep)
    keep.close()
