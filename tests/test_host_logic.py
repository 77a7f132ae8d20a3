"""Host-side logic of the drop-in layer (CPU only): parameter files, option decoding, errors."""
import os

import numpy as np
import pytest

import csadv
from csadv import advection, configuration
from oracle.solver import check_options, OptionError

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_par_files_parse_like_the_reference(golden_dir):
    z = np.load(os.path.join(golden_dir, "par.npz"))
    conf = configuration.get_parameters(os.path.join(ROOT, "par"), verbose=False)
    adv = configuration.get_advection_parameters(os.path.join(ROOT, "par"), verbose=False)
    assert [str(x) for x in conf] == list(z["configuration"])
    assert [repr(x) for x in adv] == list(z["advection"])


def test_par_file_errors_exit(tmp_path):
    (tmp_path / "configuration.par").write_text("#t\n#N\n16\n#grid\n9\n#l\n0\n#s\n0\n#tc\n5\n#m\n2\n")
    with pytest.raises(SystemExit):
        configuration.get_parameters(str(tmp_path), verbose=False)
    with pytest.raises(SystemExit):
        configuration.get_advection_parameters(str(tmp_path / "missing"), verbose=False)


@pytest.mark.parametrize("bad", [dict(ic=9), dict(vf=7), dict(recon=5), dict(dp=3), dict(opsplit=0), dict(et=4),
                                 dict(mt=3), dict(mf=0), dict(tc=3)])
def test_invalid_option_codes_exit_like_the_reference(bad, capsys):
    g = advection.cubed_sphere(16)
    args = dict(dt=0.01, Tf=5.0, ic=2, vf=1, tc=1, recon=3, dp=1, opsplit=1, et=3, mt=1, mf=3)
    args.update(bad)
    with pytest.raises(SystemExit):
        advection.adv_simulation_par(g, **args)
    assert "invalid" in capsys.readouterr().out.lower()


def test_option_pairs_match_the_oracle_and_reference():
    # SP-AVLT / SP-L04 need MT-0; SP-PL07 needs MT-PL07 (discrete_operators.py:49-73)
    for sp in (1, 2, 3):
        for mt in (1, 2):
            ok = (sp in (1, 2)) == (mt == 1)
            if ok:
                check_options(3, 1, sp, 3, mt, 3)
            else:
                with pytest.raises(OptionError):
                    check_options(3, 1, sp, 3, mt, 3)


def test_unsupported_splitting_is_an_unbound_local_error():
    assert issubclass(advection.UnsupportedSplitting, UnboundLocalError)


def test_only_the_equiangular_grid_is_built():
    with pytest.raises(SystemExit):
        advection.cubed_sphere(16, "gnomonic_equidistant")
    g = advection.cubed_sphere(24)
    assert (g.i0, g.iend, g.ng) == (4, 28, 8)
    assert g.dx == (np.pi / 4 - (-np.pi / 4)) / 24


def test_compute_errors_host():
    a = np.zeros((4, 4, 6))
    b = np.ones((4, 4, 6)) * 2.0
    b[0, 0, 0] = 5.0
    linf, l1, l2 = csadv.compute_errors(a, b)
    assert linf == 5.0
    assert l1 == pytest.approx((95 * 2 + 5) / 96)
    assert l2 == pytest.approx(np.sqrt((95 * 4 + 25) / 96))


def _replica_rank(rank, world, port, out_dir):
    import json
    import os
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        bench.replica_barrier(world)
        # rank r took (1 + r) ms per step and (5 - r) s end to end: the job takes the slowest
        ms, e2e = bench.max_over_ranks([1.0 + rank, 5.0 - rank], world, device="cpu")
        rate = bench.job_rate(100, world, ms)
        bench.replica_barrier(world)
    finally:
        dist.destroy_process_group()
    with open(os.path.join(out_dir, "rank%d.json" % rank), "w") as f:
        json.dump({"ms": ms, "e2e": e2e, "rate": rate}, f)


def test_bench_replicas_take_the_slowest_rank(tmp_path):
    """bench.py --gpus N runs N independent replicas (the solve does not shard): every timed
    region is bracketed by a barrier, times are maximised over the ranks, and the whole-job
    rate counts the units of all ranks.  Checked with two gloo ranks on the CPU."""
    import json
    import socket

    import torch.multiprocessing as mp
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    mp.start_processes(_replica_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    for r in range(2):
        got = json.load(open(tmp_path / ("rank%d.json" % r)))
        assert got["ms"] == 2.0 and got["e2e"] == 5.0
        assert abs(got["rate"] - 2 * 100 / 2e-3) < 1e-6


class _FakePlan:
    """Stands in for csadv.Plan in the serving loop's host logic: memory, mass and error norms
    of a solve that takes no GPU; `nan` makes its state non-finite."""

    def __init__(self, req, nan=False):
        self.req, self.nan, self.step, self.dt, self.closed = req, nan, 0, 0.01, False

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def stats(self):
        return {"device_bytes": 1000 * self.req.N}

    def mass(self, t):
        return float("nan") if self.nan and self.step else 1.0

    def errors(self, ic, t, ic_param=None, tracer=0):
        if self.nan:
            raise csadv.CsadvError(csadv._lib.ERR_NONFINITE, "csadv_errors")
        return (0.1, 0.01, 0.02)

    def get_tracer(self, t):
        return np.zeros(3)

    def close(self):
        self.closed = True

    def release(self, stream=None):
        self.closed = True


class _FakeBatch:
    def __init__(self, capacity):
        self.members, self.max_members = [], 0

    def add(self, pl):
        self.members.append(pl)
        self.max_members = max(self.max_members, len(self.members))

    def remove(self, pl):
        self.members.remove(pl)

    def advance(self, k, stream=None):
        for pl in self.members:
            pl.step += k

    def set_queue_depth(self, depth):
        self.depth = depth

    def close(self):
        pass


def test_serving_loop_reports_failures_per_request(monkeypatch):
    """The request loop's host logic with failures injected on the host (no GPU): a plan that
    cannot be made, a solve whose state turns non-finite, a request that misses its admission
    deadline.  Each failed request gets a result with `error` set; the others are served."""
    from csadv import serve
    made = []

    def make_plan(req, precision=32, cfl=0.5, stream=None):
        if req.N > 16384:
            raise csadv.CsadvError(csadv._lib.ERR_ARG, "csadv_plan_create")
        pl = _FakePlan(req, nan=req.rid == 3)
        made.append(pl)
        return pl

    monkeypatch.setattr(serve, "make_plan", make_plan)
    monkeypatch.setattr(serve, "Batch", _FakeBatch)
    hill = ((0.0, 0.0, 5.0),)
    reqs = [serve.Request(rid=i, N=16, steps=5 + i, tracers=1, wind="solid", hills=hill) for i in range(6)]
    reqs[1].N = 20000           # refused by the library
    reqs[5].deadline = 0.0      # cannot be admitted in time: four solves are ahead of it
    ticks = iter(range(10 ** 6))
    srv = serve.Server(budget_bytes=10 ** 9, precision=32, clock=lambda: float(next(ticks)), max_active=2)
    results, summary = srv.run(reqs, realtime=False)
    by_id = {r.rid: r for r in results}
    assert set(by_id) == set(range(6))
    # (without the library loaded the status has no text: check its number)
    assert "csadv_plan_create" in by_id[1].error and "status %d" % csadv._lib.ERR_ARG in by_id[1].error
    assert "status %d" % csadv._lib.ERR_NONFINITE in by_id[3].error and by_id[3].cell_steps == 0
    assert "not admitted" in by_id[5].error
    for i in (0, 2, 4):
        assert by_id[i].error is None and by_id[i].steps == 5 + i
        assert by_id[i].cell_steps == 6 * 16 * 16 * (5 + i)
    assert summary["requests"] == 3 and summary["failed"] == 3
    assert all(pl.closed for pl in made)  # every plan made (probes included) is released
