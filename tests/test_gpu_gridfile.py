"""GPU tests of the grid file (save_grid_netcdf4 / csadv_grid_points) against the oracle's
geometry, and of the lat-lon index file cache of ll2cs.

Tolerance: 1e-14 absolute on the unit sphere (the device's tan/atan2/sqrt are within a few ulp
of numpy's, as for the plan's own geometry)."""
import numpy as np
import pytest

from oracle.grid import CubedSphere, _tangent, equiangular_points

pytestmark = pytest.mark.gpu
ATOL = 1e-14


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build()


def axes(g, kind):
    return {"po": (g.x_edges, g.y_edges), "pc": (g.x_centers, g.y_centers), "pu": (g.x_edges, g.y_centers),
            "pv": (g.x_centers, g.y_edges)}[kind]


@pytest.mark.parametrize("N", [8, 20])
def test_grid_points_match_the_oracle(N):
    from csadv import gridfile
    g = CubedSphere(N)
    for kind in ("po", "pc", "pu", "pv"):
        x, y = axes(g, kind)
        P, EX, EY = gridfile.grid_points(N, kind)
        assert P.shape == (x.size, y.size, 6, 5)
        for c, ref in enumerate(equiangular_points(x, y)):
            np.testing.assert_allclose(P[..., c], ref, rtol=0, atol=ATOL, err_msg="%s %d" % (kind, c))
        for T, d in ((EX, "x"), (EY, "y")):
            for c, ref in enumerate(_tangent(x, y, d)):
                np.testing.assert_allclose(T[..., c], ref, rtol=0, atol=ATOL, err_msg="%s %s %d" % (kind, d, c))
            assert not T[..., 3:].any()


def test_grid_file_round_trip(tmp_path):
    from csadv import gridfile
    from csadv.advection import cubed_sphere
    cs = cubed_sphere(12)
    path = gridfile.save_grid_netcdf4(cs, str(tmp_path / (cs.name + ".nc")))
    g = gridfile.load_grid(path)
    assert (g.N, g.ng, g.ngl, g.ngr, g.i0, g.iend, g.j0, g.jend) == (12, 8, 4, 4, 4, 16, 4, 16)
    assert g.dx == cs.dx and g.dy == cs.dy and g.a == cs.a and g.title == cs.name
    for kind in ("po", "pc", "pu", "pv"):
        P, EX, EY = gridfile.grid_points(12, kind)
        for pre, A in (("", P), ("ex_", EX), ("ey_", EY)):
            pt = getattr(g, pre + kind)
            for c, k in enumerate(("X", "Y", "Z", "lon", "lat")):
                np.testing.assert_array_equal(getattr(pt, k), A[..., c])
    sio = pytest.importorskip("scipy.io")  # an independent reader sees the same file
    f = sio.netcdf_file(path, "r", mmap=False)
    try:
        assert f.variables["N"].getValue() == 12 and f.dimensions["ix"] == 21 and f.dimensions["jy2"] == 20
        np.testing.assert_array_equal(f.variables["pu"][:], gridfile.grid_points(12, "pu")[0])
    finally:
        f.close()


def test_ll2cs_uses_the_index_file_when_the_grid_directory_exists(tmp_path, monkeypatch):
    from csadv import gridfile, latlon
    from csadv.advection import cubed_sphere
    cs = cubed_sphere(16)
    ll = latlon.latlon_grid(30, 60)
    monkeypatch.setattr(gridfile, "griddir", str(tmp_path / "grid"))
    first = latlon.ll2cs(cs, ll)  # no grid directory: nothing written
    assert not (tmp_path / "grid").exists()
    (tmp_path / "grid").mkdir()
    again = latlon.ll2cs(cs, ll)  # computed, then written
    path = tmp_path / "grid" / (cs.name + "_ll2cs.nc")
    assert path.is_file()

    def no_gpu(*a):
        raise AssertionError("the index file should have been read")
    monkeypatch.setattr(latlon, "_ll2cs_gpu", no_gpu)
    cached = latlon.ll2cs(cs, ll)
    for a, b, c in zip(first, again, cached):
        np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(a, c)
