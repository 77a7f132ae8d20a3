"""The netCDF classic reader/writer (csadv.netcdf) and the reference's lat-lon file layouts
(csadv.gridfile), on the CPU.  The format is checked against an independent implementation
(scipy.io.netcdf_file) in both directions; the grid file's GPU-computed arrays are tested in
test_gpu_gridfile.py."""
import os
from types import SimpleNamespace

import numpy as np
import pytest

from csadv import gridfile, netcdf


def sample():
    rng = np.random.default_rng(3)
    dims = {"ix": 5, "jy": 4, "panel": 6, "coorddim": 5, "k": 3}
    variables = [("dx", np.float64(0.125), ()), ("N", np.int32(16), ()),
                 ("po", rng.standard_normal((5, 4, 6, 5)), ("ix", "jy", "panel", "coorddim")),
                 ("idx", np.arange(12, dtype=np.int32).reshape(4, 3) - 5, ("jy", "k")),
                 ("f4", rng.standard_normal(3).astype(np.float32), ("k",)),
                 ("s", np.array([1, -2, 3], dtype=np.int16), ("k",)),
                 ("b", np.array([1, -2, 3], dtype=np.int8), ("k",))]
    return dims, variables


@pytest.mark.parametrize("version", [1, 2])
def test_round_trip(tmp_path, version):
    dims, variables = sample()
    p = str(tmp_path / "a.nc")
    netcdf.write(p, dims, variables, {"title": "gnomonic_equiangular_cs_16", "scale": 2.5}, version=version)
    ds = netcdf.read(p)
    assert ds.dims == dims and ds.attrs["title"] == "gnomonic_equiangular_cs_16" and ds.attrs["scale"] == 2.5
    for name, a, _ in variables:
        np.testing.assert_array_equal(ds[name], a)
        assert ds[name].dtype == np.asarray(a).dtype


@pytest.mark.parametrize("version", [1, 2])
def test_scipy_reads_ours(tmp_path, version):
    sio = pytest.importorskip("scipy.io")
    dims, variables = sample()
    p = str(tmp_path / "a.nc")
    netcdf.write(p, dims, variables, {"title": "grid"}, version=version)
    f = sio.netcdf_file(p, "r", mmap=False)
    try:
        assert f.title == b"grid" and f.version_byte == version
        for name, a, _ in variables:
            v = f.variables[name]
            got = v.getValue() if v.shape == () else v[:]
            np.testing.assert_array_equal(got, a)
    finally:
        f.close()


@pytest.mark.parametrize("version", [1, 2])
def test_we_read_scipy_with_record_variables(tmp_path, version):
    sio = pytest.importorskip("scipy.io")
    p = str(tmp_path / "s.nc")
    f = sio.netcdf_file(p, "w", version=version)
    f.title = "fields"
    f.createDimension("time", None)
    f.createDimension("lat", 3)
    t = f.createVariable("time", "f8", ("time",))
    t[:] = [0.0, 0.5, 1.0, 1.5]
    q = f.createVariable("q", "f8", ("time", "lat"))
    q[:] = np.arange(12.0).reshape(4, 3)
    c = f.createVariable("c", "i2", ("time",))
    c[:] = [1, 2, 3, 4]
    lat = f.createVariable("lat", "f8", ("lat",))
    lat[:] = [-90.0, 0.0, 90.0]
    lat.units = "degrees"
    f.close()
    ds = netcdf.read(p)
    assert ds.dims == {"time": 0, "lat": 3} and ds.attrs["title"] == "fields"
    np.testing.assert_array_equal(ds["time"], [0.0, 0.5, 1.0, 1.5])
    np.testing.assert_array_equal(ds["q"], np.arange(12.0).reshape(4, 3))
    np.testing.assert_array_equal(ds["c"], [1, 2, 3, 4])
    np.testing.assert_array_equal(ds["lat"], [-90.0, 0.0, 90.0])
    assert ds.var_attrs["lat"]["units"] == "degrees"


def test_lone_record_variable_of_shorts(tmp_path):
    # one record variable: its records follow one another without padding
    sio = pytest.importorskip("scipy.io")
    p = str(tmp_path / "r.nc")
    f = sio.netcdf_file(p, "w")
    f.createDimension("t", None)
    v = f.createVariable("v", "i2", ("t",))
    v[:] = [5, -6, 7]
    f.close()
    np.testing.assert_array_equal(netcdf.read(p)["v"], [5, -6, 7])


def test_refuses_hdf5_and_bad_shapes(tmp_path):
    p = str(tmp_path / "h.nc")
    with open(p, "wb") as f:
        f.write(b"\x89HDF\r\n\x1a\n" + b"\0" * 64)
    with pytest.raises(ValueError, match="HDF5"):
        netcdf.read(p)
    with pytest.raises(ValueError):
        netcdf.write(str(tmp_path / "x.nc"), {"a": 3}, [("v", np.zeros(4), ("a",))])


def test_ll2cs_and_latlon_files(tmp_path):
    grid = SimpleNamespace(name="gnomonic_equiangular_cs_16", N=16)
    rng = np.random.default_rng(1)
    i = rng.integers(0, 16, (8, 4)).astype(np.uint32)
    j = rng.integers(0, 16, (8, 4)).astype(np.uint32)
    p = rng.integers(0, 6, (8, 4)).astype(np.uint32)
    path = gridfile.ll2cs_netcdf(i, j, p, grid, str(tmp_path / "ll.nc"))
    ds = netcdf.read(path)
    assert ds.dims == {"lon": 8, "lat": 4} and ds.attrs["title"] == "gnomonic_equiangular_cs_16_ll2cs"
    assert all(ds[k].dtype == np.int32 for k in ("i", "j", "panel"))
    for a, b in zip(gridfile.load_ll2cs(path), (i, j, p)):
        np.testing.assert_array_equal(a, b)
        assert a.dtype == np.uint32
    q = rng.standard_normal((8, 4, 3))
    path = gridfile.latlon_netcdf("adv_Q", {"Q": q, "Q_exact": 2 * q}, [0.0, 0.1, 0.2], str(tmp_path / "f.nc"))
    ds = netcdf.read(path)
    assert ds.dims == {"time": 3, "lat": 4, "lon": 8} and ds.attrs["title"] == "adv_Q"
    np.testing.assert_array_equal(ds["lat"], np.linspace(-90.0, 90.0, 4))
    np.testing.assert_array_equal(ds["lon"], np.linspace(-180.0, 180.0, 8))
    np.testing.assert_array_equal(ds["Q_exact"], 2 * q)
    with pytest.raises(ValueError):
        gridfile.latlon_netcdf("bad", {"Q": q}, [0.0, 0.1], str(tmp_path / "g.nc"))
    assert not os.path.exists(str(tmp_path / "g.nc"))
