"""GPU tests of the continuous-batching request loop (csadv.serve).

The bar: every request's result is the same bit for bit when served in the mix (admitted
while others are resident, stepped in a shared batch, retired at different times) as when
run alone; the memory budget bounds what is resident; the run reports p50/p99 latency.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build()


def small_stream(n=14, seed=3):
    from csadv import serve
    return serve.poisson_requests(n, rate=1000.0, seed=seed, n_range=(12, 72), steps_range=(3, 40), tracers=(1, 3))


def alone(req, precision):
    from csadv import serve
    with serve.make_plan(req, precision) as pl:
        pl.advance(req.steps)
        return [pl.get_tracer(t) for t in range(req.tracers)]


@pytest.mark.parametrize("precision", [32, 64])
def test_served_results_identical_to_alone(precision):
    from csadv import serve
    reqs = small_stream()
    srv = serve.Server(budget_bytes=8 << 30, precision=precision, keep_state=True, max_steps_per_tick=5)
    results, summary = srv.run(reqs, realtime=False)
    assert summary["requests"] == len(reqs)
    by_id = {r.rid: r for r in results}
    for req in reqs:
        got = by_id[req.rid]
        assert got.steps == req.steps
        for a, b in zip(got.state, alone(req, precision)):
            np.testing.assert_array_equal(a, b)
        assert max(got.mass_change) < (1e-6 if precision == 32 else 1e-12)


def test_budget_limits_residency_and_latency_is_reported():
    from csadv import serve
    reqs = small_stream(n=10, seed=5)
    srv = serve.Server(budget_bytes=1, precision=32)   # room for one solve at a time
    seen = []
    results, summary = srv.run(reqs, realtime=False, on_step=lambda s, n, used: seen.append(n))
    assert summary["requests"] == len(reqs)
    assert max(seen) == 1
    assert summary["p99_latency_s"] >= summary["p50_latency_s"] > 0
    srv2 = serve.Server(budget_bytes=8 << 30, precision=32)
    seen2 = []
    srv2.run(reqs, realtime=False, on_step=lambda s, n, used: seen2.append(n))
    assert max(seen2) > 1


def test_realtime_arrivals_overlap():
    # requests arriving while others run are admitted at step boundaries
    from csadv import serve
    reqs = serve.poisson_requests(8, rate=400.0, seed=11, n_range=(16, 48), steps_range=(20, 60), tracers=(1, 2))
    srv = serve.Server(budget_bytes=8 << 30, precision=32)
    seen = []
    results, summary = srv.run(reqs, realtime=True, on_step=lambda s, n, used: seen.append(n))
    assert summary["requests"] == len(reqs)
    assert all(r.finished >= r.arrival for r in results)


def test_failed_requests_stay_with_their_request():
    # failures are injected on the host: a size the library refuses, a hill whose width is NaN
    # (its state turns non-finite), and a deadline that cannot be met; the other requests are
    # served with the bits they get alone
    import dataclasses
    import math
    from csadv import serve
    good = small_stream(n=6, seed=7)
    bad_size = dataclasses.replace(good[0], rid=100, N=20000)
    bad_nan = dataclasses.replace(good[1], rid=101, wind="solid", hills=((0.0, 0.0, math.nan),) * good[1].tracers)
    late = dataclasses.replace(good[2], rid=102, deadline=0.0)
    reqs = good[:3] + [bad_size, bad_nan] + good[3:] + [late]
    srv = serve.Server(budget_bytes=1, precision=32, keep_state=True)  # one at a time: `late` must wait
    results, summary = srv.run(reqs, realtime=False)
    by_id = {r.rid: r for r in results}
    assert set(by_id) == {r.rid for r in reqs}
    assert summary["requests"] == len(good) and summary["failed"] == 3
    assert "invalid argument" in by_id[100].error
    assert "non-finite" in by_id[101].error and by_id[101].cell_steps == 0
    assert "not admitted" in by_id[102].error
    for req in good:
        got = by_id[req.rid]
        assert got.error is None
        for a, b in zip(got.state, alone(req, 32)):
            np.testing.assert_array_equal(a, b)


def test_threaded_loop_on_own_streams_identical_to_alone():
    """Plans made by builder threads on their own stream and read out by the retirement thread:
    every request's fields are the same bits as run alone, FP32 and FP64, with arrivals in real
    time and all at once."""
    import torch
    from csadv import serve
    reqs = small_stream(n=12, seed=9)
    for precision, realtime in ((32, True), (64, False)):
        srv = serve.Server(budget_bytes=8 << 30, precision=precision, keep_state=True, max_steps_per_tick=5,
                           stream=torch.cuda.Stream(), build_stream=torch.cuda.Stream())
        assert srv.threads
        results, summary = srv.run(reqs, realtime=realtime)
        assert summary["requests"] == len(reqs) and summary["failed"] == 0
        assert summary["graph_builds"] >= 1
        by_id = {r.rid: r for r in results}
        for req in reqs:
            for a, b in zip(by_id[req.rid].state, alone(req, precision)):
                np.testing.assert_array_equal(a, b)
