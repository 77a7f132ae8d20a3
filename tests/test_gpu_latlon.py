"""GPU tests of the lat-lon output (ll2cs, nearest_neighbour; interpolation.py:38-150).

Integer results (panel, cell indices) must equal the reference's exactly: against the golden
fixture made by the reference (tests/golden/latlon.npz, with its own X, Y, Z) and against the
oracle on the reference's plotting grid (180 x 360).  The gathered fields are exact copies.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build()


class _LL:
    pass


def _fixture_cases(golden_dir):
    z = np.load(os.path.join(golden_dir, "latlon.npz"))
    for key in sorted({k.rsplit("_", 1)[0] for k in z.files}):
        N = int(key.split("_")[0][1:])
        ll = _LL()
        ll.X, ll.Y, ll.Z = z[key + "_X"], z[key + "_Y"], z[key + "_Z"]
        ll.Nlon, ll.Nlat = ll.X.shape
        yield N, ll, z[key + "_i"], z[key + "_j"], z[key + "_panel"], z[key + "_nn"]


def test_ll2cs_equals_reference(golden_dir):
    from csadv.advection import cubed_sphere
    from csadv.latlon import ll2cs
    for N, ll, i, j, p, _ in _fixture_cases(golden_dir):
        gi, gj, gp = ll2cs(cubed_sphere(N), ll)
        np.testing.assert_array_equal(gp, p)
        np.testing.assert_array_equal(gi, i)
        np.testing.assert_array_equal(gj, j)


@pytest.mark.parametrize("N", [16, 48, 96])
def test_ll2cs_equals_oracle_on_plotting_grid(N):
    from csadv.advection import cubed_sphere
    from csadv.latlon import latlon_grid, ll2cs
    from oracle import latlon
    ll = latlon_grid(180, 360)
    gi, gj, gp = ll2cs(cubed_sphere(N), ll)
    i, j, p = latlon.ll2cs(N, ll.X, ll.Y, ll.Z)
    np.testing.assert_array_equal(gp, p)
    np.testing.assert_array_equal(gi, i)
    np.testing.assert_array_equal(gj, j)


@pytest.mark.parametrize("prec", [64, 32])
def test_nearest_neighbour_of_a_plan_tracer(golden_dir, prec):
    """nearest_neighbour of a tracer resident in a plan gathers the plan's current state: the
    reference's result for the same field, exactly (FP64) or that field in FP32 (FP32 state);
    also after a step with a pending mass-fixer correction, against get_tracer."""
    from csadv import Plan
    from csadv.advection import cubed_sphere
    from csadv.latlon import ll2cs, nearest_neighbour
    for N, ll, i, j, p, nn in _fixture_cases(golden_dir):
        f = np.arange(N * N * 6, dtype=np.float64).reshape(N, N, 6) * 0.5 - 7.0
        ll.ix, ll.jy, ll.mask = ll2cs(cubed_sphere(N), ll)
        with Plan(N, 0.002, recon=2, dp=2, opsplit=1, et=3, mt=1, mf=3, vf=2, ntracers=2, precision=prec) as pl:
            pl.set_tracer(f, tracer=1)
            got = nearest_neighbour((pl, 1), None, ll)
            want = nn if prec == 64 else nn.astype(np.float32).astype(np.float64)
            np.testing.assert_array_equal(got, want)
            pl.init_tracer(2, tracer=0)
            pl.advance(3)
            q = pl.get_tracer(0)
            np.testing.assert_array_equal(nearest_neighbour(pl, None, ll), q[ll.ix, ll.jy, ll.mask])


def test_nearest_neighbour_rejects_indices_outside_the_panel():
    from csadv import CsadvError, Plan
    from csadv.latlon import nearest_neighbour
    ll = _LL()
    ll.Nlon, ll.Nlat = 2, 1
    ll.ix = np.array([[0], [16]], dtype=np.uint32)
    ll.jy = np.array([[0], [0]], dtype=np.uint32)
    ll.mask = np.array([[0], [0]], dtype=np.uint32)
    with Plan(16, 0.01, vf=1) as pl:
        with pytest.raises(CsadvError):
            nearest_neighbour(pl, None, ll)


def test_adv_sphere_writes_latlon_fields(tmp_path):
    """adv_sphere(plot=True) writes Q on the lat-lon grid (.npy) where the reference plots it."""
    from csadv import advection
    from csadv.latlon import latlon_grid, ll2cs
    advection.output_dir = str(tmp_path)
    cs = advection.cubed_sphere(16)
    ll = latlon_grid(46, 91)
    ll.ix, ll.jy, ll.mask = ll2cs(cs, ll)
    sim = advection.adv_simulation_par(cs, 0.05, 0.5, 2, 1, 1, 3, 1, 1, 3, 1, 3)
    advection.adv_sphere(cs, ll, sim, "mercator", True, False)
    files = sorted(os.listdir(tmp_path))
    assert len(files) == 6 and all(f.endswith(".npy") for f in files)  # k = 0, 2, 4, 6, 8, 10
    last = np.load(os.path.join(tmp_path, [f for f in files if f.endswith("_t10.npy")][0]))
    assert last.shape == (91, 46)
    np.testing.assert_array_equal(last, sim.Q[4:20, 4:20, :][ll.ix, ll.jy, ll.mask])
