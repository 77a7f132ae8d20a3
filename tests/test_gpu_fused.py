"""GPU tests of the fused engine (one tile kernel per step) against the reference goldens,
the staged engine and the CPU oracle, plus the FP32 form's accuracy and mass budget.

Tolerances: FP64 fused vs reference / oracle / staged: 1e-12 relative to the field
maximum (the FP64 parity bar).  FP32 vs FP64: 2e-5 relative after tens of steps, and
mass conserved to 1e-6 relative with MF-PR (the FP32 form's stated bars).
"""
import os

import numpy as np
import pytest

from oracle import solver
from oracle.grid import CubedSphere

pytestmark = pytest.mark.gpu

RTOL = 1e-12
FUSED = 2
STAGED = 1


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


def test_fused_rejects_schemes_it_does_not_cover():
    from csadv import CsadvError
    for c in ((3, 1, 1, 1, 1, 3), (3, 1, 1, 2, 1, 3), (3, 1, 1, 3, 1, 2)):
        with pytest.raises(CsadvError):
            plan(16, 0.01, c, 1, engine=FUSED)


@pytest.mark.parametrize("vf", [2, 1])
def test_fused_fp64_vs_reference_golden(golden_dir, vf):
    z = np.load(os.path.join(golden_dir, "combos_N10.npz"))
    n = 0
    for c, Qref in zip(z["combos_vf%d" % vf], z["Q_vf%d" % vf]):
        c = tuple(int(x) for x in c)
        if c[3] != 3 or c[5] == 2:
            continue
        with plan(10, float(z["dt"]), c, vf, engine=FUSED) as pl:
            pl.init_tracer(int(z["ic"]))
            pl.advance(int(z["nsteps"]))
            assert rel(pl.get_tracer(), Qref) <= RTOL, c
        n += 1
    assert n > 0


@pytest.mark.parametrize("tile", [1, 2, 3, 4, 5, 6, 7, 8])
@pytest.mark.parametrize("N", [40, 50, 64])
def test_fused_fp64_partial_tiles_vs_oracle(N, tile):
    c, vf, ic, dt, nsteps = (2, 2, 1, 3, 1, 3), 2, 3, 0.004, 6
    g = CubedSphere(N)
    sim = solver.Simulation(g, dt, 5.0, ic, vf, *c)
    solver.run_steps(sim, nsteps)
    with plan(N, dt, c, vf, engine=FUSED, tile=tile) as pl:
        pl.init_tracer(ic)
        pl.advance(nsteps)
        assert rel(pl.get_tracer(), sim.Q[g.interior]) <= RTOL


def _et_dg_schemes():
    out = []
    for recon in (1, 2, 3, 4):
        for dp in (1, 2):
            for sp, mt in ((1, 1), (2, 1), (3, 2)):
                for mf in (1, 3):
                    out.append((recon, dp, sp, 3, mt, mf))
    return out


@pytest.mark.parametrize("N", [8, 61, 130])
def test_sweep_kernel_equals_tile_kernel_every_scheme(N):
    # the line-marching kernel (tiles 5-8) against the per-edge tile kernel (tiles 1-4):
    # same arithmetic, so FP64 agrees at the parity bar and FP32 to rounding
    dt = 0.25 / N
    for c in _et_dg_schemes():
        for prec, tol in ((64, RTOL), (32, 1e-5)):
            outs = []
            for tile in (1, 5 if N >= 100 else 8):
                with plan(N, dt, c, 2, engine=FUSED, precision=prec, tile=tile) as pl:
                    pl.init_tracer(3)
                    pl.advance(4)
                    outs.append(pl.get_tracer())
            assert rel(outs[1], outs[0]) <= tol, (c, prec)


@pytest.mark.parametrize("c", [(1, 1, 1, 3, 1, 1), (2, 2, 1, 3, 1, 3), (3, 2, 2, 3, 1, 3), (4, 1, 3, 3, 2, 3),
                               (4, 2, 3, 3, 2, 1), (3, 1, 1, 3, 1, 3)])
def test_fused_equals_staged_long_run_fp64(c):
    N, dt, nsteps = 96, 0.002, 60
    outs = []
    for eng in (STAGED, FUSED):
        with plan(N, dt, c, 2, engine=eng) as pl:
            pl.init_tracer(3)
            pl.advance(nsteps)
            outs.append((pl.get_tracer(), pl.mass()))
    assert rel(outs[1][0], outs[0][0]) <= RTOL
    assert abs(outs[1][1] - outs[0][1]) <= 1e-12 * abs(outs[0][1])


def test_fused_tracers_equal_single_runs():
    c, vf, dt = (2, 2, 1, 3, 1, 3), 2, 0.004
    with plan(48, dt, c, vf, ntracers=3, engine=FUSED) as pl:
        for t, ic in enumerate((2, 3, 4)):
            pl.init_tracer(ic, tracer=t)
        pl.advance(5)
        multi = [pl.get_tracer(t) for t in range(3)]
    for t, ic in enumerate((2, 3, 4)):
        with plan(48, dt, c, vf, engine=FUSED) as pl:
            pl.init_tracer(ic)
            pl.advance(5)
            np.testing.assert_array_equal(pl.get_tracer(), multi[t])


def test_fused_set_get_between_steps_keeps_state():
    # reading/writing the state in the middle of a run applies the pending mass-fixer correction
    c, vf, dt = (2, 2, 1, 3, 1, 3), 2, 0.004
    with plan(48, dt, c, vf, engine=FUSED) as a, plan(48, dt, c, vf, engine=FUSED) as b:
        a.init_tracer(3)
        b.init_tracer(3)
        a.advance(4)
        b.advance(2)
        q = b.get_tracer(full=True)
        b.set_tracer(q)
        b.advance(2)
        assert rel(b.get_tracer(), a.get_tracer()) <= RTOL


@pytest.mark.parametrize("prec", [64, 32])
def test_upload_of_one_tracer_leaves_the_others_pending(prec):
    # set_tracer / get_tracer with a pending MF-PR correction on the other tracers give the bits
    # of materialise-then-copy (here forced by a mass diagnostic before the upload)
    c, vf, dt, N = (2, 2, 1, 3, 1, 3), 2, 0.004, 32
    rng = np.random.default_rng(11)
    q = 1.0 + 0.1 * rng.standard_normal((N + 8, N + 8, 6))
    with plan(N, dt, c, vf, engine=FUSED, ntracers=3, precision=prec) as a, \
            plan(N, dt, c, vf, engine=FUSED, ntracers=3, precision=prec) as b:
        for pl in (a, b):
            for t, ic in enumerate((2, 3, 4)):
                pl.init_tracer(ic, tracer=t)
            pl.advance(3)
        lazy = [b.get_tracer(t, full=True) for t in range(3)]
        a.mass(0)  # materialises the correction of every tracer
        for t in range(3):
            np.testing.assert_array_equal(lazy[t], a.get_tracer(t, full=True))
        for pl in (a, b):
            pl.set_tracer(q, tracer=1)
            pl.advance(3)
        for t in range(3):
            np.testing.assert_array_equal(b.get_tracer(t), a.get_tracer(t))


@pytest.mark.parametrize("full", [True, False])
def test_fp32_upload_records_the_mass_target(full):
    # the FP32 upload records sum(Q g) over the interior (FP64 products of the stored FP32
    # values and the FP32 metric) as the tracer's mass target, in the same pass; 1e-9 relative
    # allows an ulp of difference between the oracle's metric and the device's in a few cells
    import ctypes
    from csadv import _lib
    N, dt = 40, 0.004
    rng = np.random.default_rng(5)
    q = 1.0 + 0.1 * rng.standard_normal((N + 8, N + 8, 6) if full else (N, N, 6))
    g32 = CubedSphere(N).metric_tensor_pc[4:N + 4, 4:N + 4].astype(np.float32).astype(np.float64)
    with plan(N, dt, (2, 2, 1, 3, 1, 3), 2, engine=FUSED, ntracers=2, precision=32) as pl:
        pl.init_tracer(2, tracer=0)
        pl.advance(2)
        pl.set_tracer(q, tracer=1)
        m = ctypes.c_double()
        _lib.check(_lib.lib().csadv_mass_target(pl._h, 1, ctypes.byref(m), None, pl.stream))
        qi = (q[4:N + 4, 4:N + 4] if full else q).astype(np.float32).astype(np.float64)
        want = float(np.sum(qi * g32))
        assert abs(m.value - want) <= 1e-9 * abs(want)
        np.testing.assert_array_equal(pl.get_tracer(1), qi)


@pytest.mark.parametrize("c", [(2, 2, 1, 3, 1, 3), (3, 1, 1, 3, 1, 3)])
def test_fp32_form_accuracy_and_mass(c):
    N, dt, nsteps, ic, vf = 96, 0.002, 80, 3, 2
    res = {}
    for prec in (64, 32):
        with plan(N, dt, c, vf, precision=prec, engine=FUSED) as pl:
            pl.init_tracer(ic)
            m0 = pl.mass()
            pl.advance(nsteps)
            res[prec] = (pl.get_tracer(), abs(pl.mass() - m0) / abs(m0), pl.errors(ic, nsteps * dt))
    assert rel(res[32][0], res[64][0]) < 2e-5
    assert res[32][1] < 1e-6
    # L2 error against the analytic solution within 1% of the FP64 run's
    assert abs(res[32][2][2] - res[64][2][2]) <= 0.01 * res[64][2][2]


def test_fp32_staged_and_fused_agree():
    c, N, dt = (2, 2, 1, 3, 1, 3), 64, 0.003
    outs = []
    for eng in (STAGED, FUSED):
        with plan(N, dt, c, 2, precision=32, engine=eng) as pl:
            pl.init_tracer(2)
            pl.advance(20)
            outs.append(pl.get_tracer())
    assert rel(outs[1], outs[0]) < 1e-5


def test_fp32_mass_anchored_over_long_run():
    # FP32 state with MF-PR: the correction restores each tracer's sum(Q g) as it was set, so
    # the mass stays within 1e-6 relative over thousands of steps (without the anchor, FP32
    # rounding of the update makes it drift like a random walk)
    c = (2, 2, 1, 3, 1, 3)
    with plan(32, -0.5, c, 102, precision=32, wind_param=(0.48, 5.0, 0, 0), ntracers=2) as pl:
        pl.init_tracer(101, ic_param=(0.3, 0.2, 5.0, 0.0), tracer=0)
        pl.init_tracer(102, tracer=1)
        m0 = [pl.mass(t) for t in range(2)]
        pl.advance(2000)
        for t in range(2):
            assert abs(pl.mass(t) - m0[t]) <= 1e-6 * abs(m0[t])


@pytest.mark.parametrize("prec", [32, 64])
def test_inline_ghost_cells_match_ghost_cell_kernel(prec):
    """The step kernel's own ghost cells (the default) and the separate ghost-cell launch give
    the same bits: N = 48 (one tile per panel: every tile touches all
    four panel edges and the corners), N = 120 (interior tiles too), three tracers (a pair and
    an odd one), time-dependent wind with RK2 and MF-PR, several steps; the full-layout fields
    (ghost cells included) agree as well."""
    for N in (48, 120):
        c = (2, 2, 1, 3, 1, 3)
        with plan(N, 0.004, c, 2, ntracers=3, precision=prec, engine=FUSED, tile=5) as a, \
                plan(N, 0.004, c, 2, ntracers=3, precision=prec, engine=FUSED, tile=5) as b:
            a.set_inline_ghosts(True)
            b.set_inline_ghosts(False)
            for pl in (a, b):
                for t in range(3):
                    pl.init_tracer(101 + t % 3, ic_param=(0.4 * t, 0.3, 5.0, 0.0) if t == 0 else None, tracer=t)
                pl.advance(4)
            for t in range(3):
                np.testing.assert_array_equal(a.get_tracer(t), b.get_tracer(t))
                np.testing.assert_array_equal(a.get_tracer(t, full=True), b.get_tracer(t, full=True))
            assert a.mass(2) == b.mass(2)


def test_fp32_ghost_cells_equal_fp64_interpolation_rounded():
    """The FP32 form sums the Lagrange interpolation in double-float arithmetic (FP64 weights as
    two FP32 words).  On the same FP32-representable field, its ghost cells equal the FP64 form's
    ghost cells rounded to FP32 to one unit in the last place; the side strips exactly, for all
    but a tiny fraction (values next to a rounding boundary).  The corner blocks interpolate
    side-strip values that the FP32 form holds in FP32 (the reference's two-level rule applied
    to an FP32 array), so there the two forms differ by a rounding."""
    rng = np.random.default_rng(11)
    N = 40
    q = (1.0 + 0.5 * rng.standard_normal((N, N, 6))).astype(np.float32).astype(np.float64)
    full = {}
    for prec in (64, 32):
        with plan(N, 1e-4, (2, 2, 1, 3, 1, 3), 1, precision=prec, engine=FUSED) as pl:
            pl.set_tracer(q)
            pl.advance(1)
            full[prec] = pl.get_tracer(full=True)
    inside = np.zeros(N + 8, bool)
    inside[4:N + 4] = True
    ghost = ~np.outer(inside, inside)
    side = np.outer(inside, ~inside) | np.outer(~inside, inside)
    ulp = np.abs(full[64].astype(np.float32).view(np.int32).astype(np.int64) -
                 full[32].astype(np.float32).view(np.int32).astype(np.int64))
    assert ulp[ghost & ~side].max() <= 4  # corner blocks: weights up to ~2 on inputs one rounding apart
    assert ulp[side].max() <= 1
    assert np.count_nonzero(ulp[side]) <= max(2, ulp[side].size // 1000)


def test_pipelined_wind_records_follow_every_call_pattern():
    """FP32 with a time-dependent wind computes the next step's edge records while the step
    runs.  Whatever the order of calls -- advance, the reference's time_step + update_winds
    loop, steps taken in a batch, graphs on or off, profiled steps -- a plan gives the same bits
    as one advanced straight through."""
    from csadv import Batch, Plan
    N, dt, nsteps = 40, 0.004, 9
    kw = dict(recon=2, dp=2, opsplit=1, et=3, mt=1, mf=3, vf=2, ntracers=2, precision=32)

    def make():
        pl = Plan(N, dt, **kw)
        pl.init_tracer(2, tracer=0)
        pl.init_tracer(101, ic_param=(0.5, 0.2, 5.0, 0.0), tracer=1)
        return pl

    with make() as a:
        a.advance(nsteps)
        ref = [a.get_tracer(t) for t in range(2)]
    with make() as b:
        b.advance(2)
        for k in (3, 4):  # adv_sphere's loop: time step k, then the wind at k dt
            b.time_step(k)
            b.update_winds(k * dt)
        with Batch(4) as bt:
            bt.add(b)
            bt.advance(2)
            bt.remove(b)
        b.set_graphs(False)
        b.advance(1)
        b.set_graphs(True)
        b.set_profiling(True)
        b.advance(1)
        b.set_profiling(False)
        b.advance(1)
        assert b.step == nsteps
        for t in range(2):
            np.testing.assert_array_equal(b.get_tracer(t), ref[t])


@pytest.mark.parametrize("prec,vf,wp,inline", [(64, 2, (0, 0, 0, 0), None), (32, 102, (0.48, 5.0, 0, 0), None),
                                               (32, 101, (0.7, 1.25, 0, 0), None), (32, 102, (0.48, 5.0, 0, 0), False),
                                               (64, 102, (0.48, 5.0, 0, 0), False)])
def test_checkpoint_resume_gives_the_same_bits(tmp_path, prec, vf, wp, inline):
    """A run saved after k steps and resumed in a new plan continues with the same bits as the
    run that was not interrupted (time-dependent and static winds, FP64 and FP32 forms, and
    ghost cells evaluated inside the step kernel or by the separate launch when that is not the
    form's default: the choice is saved with the plan)."""
    from csadv import Plan, checkpoint
    kw = dict(recon=2, dp=2, opsplit=1, et=3, mt=1, mf=3, vf=vf, wind_param=wp, ntracers=3, precision=prec)
    with Plan(48, -0.5, **kw) as a:
        if inline is not None:
            a.set_inline_ghosts(inline)
        for t in range(3):
            a.init_tracer(101 + t, ic_param=(0.3, 0.2, 5.0, 0.0) if t == 0 else None, tracer=t)
        a.advance(5)
        path = str(tmp_path / "ckpt.npz")
        checkpoint.save(a, path)
        a.advance(6)
        ref = [a.get_tracer(t) for t in range(3)]
        with checkpoint.load(path) as b:
            assert b.step == 5 and b.dt == a.dt
            b.advance(6)
            for t in range(3):
                np.testing.assert_array_equal(b.get_tracer(t), ref[t])
