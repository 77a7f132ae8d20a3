"""csadv_advance_host (a host-resident state: upload, steps, read-out in one call, the copies on
the copy engines beside per-tracer step kernels) against the same work as separate calls
(csadv_set_tracer, csadv_advance, csadv_get_tracer): equal bit for bit, FP64 and FP32, for one,
two and three steps, one to three tracers, both layouts each way, page-locked and pageable host
arrays, a time-dependent and a static wind, and a plan of the staged engine (which runs the
separate calls itself)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCHEME = dict(recon=2, dp=2, opsplit=1, et=3, mt=1, mf=3)   # the benchmark's scheme
DEFORM = (0.48, 5.0, 0.0, 0.0)                              # deformational wind, k = 0.48, T = 5
ICS = (102, 103, 101)
HILL = (np.pi / 4, np.pi / 6, 10.0, 0.0)


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build()


def make(N, T, precision, vf=102, wp=DEFORM, **kw):
    from csadv import Plan
    sch = dict(SCHEME)
    sch.update(kw)
    return Plan(N, -0.5, vf=vf, ntracers=T, precision=precision, wind_param=wp, **sch)


def initial(N, T, precision, vf=102, wp=DEFORM, full=True, **kw):
    """Full-layout (or interior) initial fields from a plan: the cases' exact values."""
    with make(N, T, precision, vf, wp, **kw) as pl:
        out = []
        for t in range(T):
            ic = ICS[t % len(ICS)]
            pl.init_tracer(ic, HILL if ic == 101 else None, tracer=t)
            out.append(pl.get_tracer(t, full=full))
        return out


def separate(N, T, precision, Q0, nsteps, full_out, vf=102, wp=DEFORM, **kw):
    with make(N, T, precision, vf, wp, **kw) as pl:
        for t in range(T):
            pl.set_tracer(Q0[t], t)
        pl.advance(nsteps)
        return [pl.get_tracer(t, full=full_out) for t in range(T)], pl.step


def one_call(N, T, precision, Q0, nsteps, full_out, pinned=True, vf=102, wp=DEFORM, **kw):
    from csadv import host_array
    with make(N, T, precision, vf, wp, **kw) as pl:
        if pinned:
            src = [host_array(q.shape) for q in Q0]
            for a, q in zip(src, Q0):
                a[...] = q
            shp = (pl.n, pl.n, 6) if full_out else (N, N, 6)
            dst = [host_array(shp) for _ in range(T)]
            out = pl.advance_host(nsteps, src, dst)
        else:
            out = pl.advance_host(nsteps, [q.copy() for q in Q0], True, full_out=full_out)
        return [np.array(o) for o in out], pl.step


@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("T", [1, 2, 3])
def test_one_call_equals_separate_calls(precision, T):
    N = 40
    Q0 = initial(N, T, precision)
    for nsteps in (1, 2, 3):
        ref, k_ref = separate(N, T, precision, Q0, nsteps, False)
        got, k = one_call(N, T, precision, Q0, nsteps, False)
        assert k == k_ref == nsteps
        for t in range(T):
            np.testing.assert_array_equal(got[t], ref[t], err_msg="T=%d t=%d nsteps=%d" % (T, t, nsteps))


@pytest.mark.parametrize("precision", [64, 32])
def test_layouts_each_way(precision):
    N, T = 32, 2
    Q_full = initial(N, T, precision, full=True)
    Q_int = [q[4:-4, 4:-4].copy() for q in Q_full]
    for Q0 in (Q_full, Q_int):
        for full_out in (False, True):
            ref, _ = separate(N, T, precision, Q0, 2, full_out)
            got, _ = one_call(N, T, precision, Q0, 2, full_out)
            for t in range(T):
                np.testing.assert_array_equal(got[t], ref[t])


def test_pageable_arrays_and_in_place():
    N, T = 32, 2
    Q0 = initial(N, T, 64)
    ref, _ = separate(N, T, 64, Q0, 2, False)
    got, _ = one_call(N, T, 64, Q0, 2, False, pinned=False)
    for t in range(T):
        np.testing.assert_array_equal(got[t], ref[t])
    # in[t] == out[t]: each step writes its result over its input
    from csadv import host_array
    with make(N, T, 64) as pl:
        Q = [host_array(q.shape) for q in Q0]
        for a, q in zip(Q, Q0):
            a[...] = q
        for _ in range(2):
            pl.advance_host(1, Q, Q)
        with make(N, T, 64) as p2:
            for t in range(T):
                p2.set_tracer(Q0[t], t)
            for _ in range(2):
                p2.advance(1)
                for t in range(T):
                    p2.set_tracer(p2.get_tracer(t, full=True), t)
            for t in range(T):
                np.testing.assert_array_equal(np.array(Q[t]), p2.get_tracer(t, full=True))


def test_static_wind_and_no_upload():
    N, T = 32, 2
    wp = (-np.pi / 4, 2 * np.pi / 5, 0.0, 0.0)
    Q0 = initial(N, T, 64, vf=101, wp=wp)
    ref, _ = separate(N, T, 64, Q0, 3, False, vf=101, wp=wp)
    got, _ = one_call(N, T, 64, Q0, 3, False, vf=101, wp=wp)
    for t in range(T):
        np.testing.assert_array_equal(got[t], ref[t])
    with make(N, T, 64, vf=101, wp=wp) as pl:   # Q_in None: the device state steps on
        for t in range(T):
            pl.set_tracer(Q0[t], t)
        out = pl.advance_host(3, None, True)
        for t in range(T):
            np.testing.assert_array_equal(out[t], ref[t])


def test_staged_engine_runs_the_separate_calls():
    from csadv import _lib as L
    N, T = 24, 2
    Q0 = initial(N, T, 64, engine=L.ENGINE_STAGED)
    ref, _ = separate(N, T, 64, Q0, 2, False, engine=L.ENGINE_STAGED)
    got, _ = one_call(N, T, 64, Q0, 2, False, engine=L.ENGINE_STAGED)
    for t in range(T):
        np.testing.assert_array_equal(got[t], ref[t])


def test_bad_arguments():
    from csadv import CsadvError
    with make(16, 2, 64) as pl:
        with pytest.raises(ValueError):
            pl.advance_host(1, [np.zeros((16, 16, 6))])
        with pytest.raises(CsadvError):
            pl.advance_host(-1)
