"""GPU tests of the convergence-study driver (error_analysis_adv, advection_error.py:21-188)
and of the par-file entry point (python -m csadv, main.py:78-95).

The coarsest resolution of each scheme is checked against the CPU oracle (the reference's
algorithm) at 1e-10 relative on the error norms; the finer ones by their convergence rate.
"""
import os

import numpy as np
import pytest

from oracle import solver
from oracle.grid import CubedSphere

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build()


def write_par(tmp_path, N=16, tc=2, vf=1, ic=2, dt=0.025, Tf=5.0):
    # the reference's positional format: a title line, then (comment, value) pairs
    def par(title, values):
        return title + "\n" + "".join("#%s\n%s\n" % kv for kv in values)
    (tmp_path / "configuration.par").write_text(par("configuration", [
        ("N", N), ("grid", 2), ("load", 0), ("show", 0), ("test case", 5), ("map", 2)]))
    (tmp_path / "advection.par").write_text(par("advection", [
        ("Tf", Tf), ("dt", dt), ("ic", ic), ("vf", vf), ("tc", tc), ("recon", 3), ("dp", 1), ("split", 3),
        ("et", 3), ("mt", 2), ("mf", 3)]))
    return str(tmp_path) + os.sep


def test_convergence_study_matches_oracle_and_converges(tmp_path):
    from csadv import advection
    pardir = write_par(tmp_path)
    cs = advection.cubed_sphere(16)
    sim = advection.adv_simulation_par(cs, 0.025, 5.0, 2, 1, 2, 3, 1, 3, 3, 1, 3)
    Nc, linf, l1, l2, rates = advection.error_analysis_adv(sim, "sphere", False, "gnomonic_equiangular", False,
                                                            False, Ntest=3, pardir=pardir)
    assert list(Nc) == [16, 32, 64]
    g = CubedSphere(16)
    for d, (rec, sp, et, mt, dp, mf) in enumerate(advection.CONVERGENCE_SCHEMES):
        ref = solver.adv_sphere(solver.Simulation(g, 0.025, 5.0, 2, 1, rec, dp, sp, et, mt, mf))
        got = (linf[0, d], l1[0, d], l2[0, d])
        for a, b in zip(got, ref):
            assert abs(a - b) <= 1e-10 * abs(b), (d, got, ref)
    # PPM on a smooth hill: errors fall at least ~ first order per halving of N and dt
    assert np.all(rates["l2"] > 1.0)


def test_module_entry_point_runs_the_par_files(tmp_path, monkeypatch):
    from csadv import __main__ as entry
    from csadv import advection, gridfile
    pardir = write_par(tmp_path, N=16, tc=1, dt=0.05, Tf=0.5)
    monkeypatch.setattr(advection, "output_dir", str(tmp_path / "graphs"))
    monkeypatch.setattr(gridfile, "griddir", str(tmp_path / "grid"))
    monkeypatch.setattr(gridfile, "datadir", str(tmp_path / "data"))
    linf, l1, l2 = entry.main([pardir])
    # the reference plots Q on its 720 x 1440 lat-lon grid at steps 0, 2, ..., 10: written as .npy
    outs = sorted(os.listdir(advection.output_dir))
    assert len(outs) == 6 and np.load(os.path.join(advection.output_dir, outs[0])).shape == (1440, 720)
    # and, as main.py and ll2cs do, the grid file and the lat-lon index file (netCDF)
    g16 = gridfile.load_grid(str(tmp_path / "grid" / "gnomonic_equiangular_cs_16.nc"))
    assert g16.N == 16 and g16.pc.lon.shape == (24, 24, 6)
    i, j, p = gridfile.load_ll2cs(str(tmp_path / "grid" / "gnomonic_equiangular_cs_16_ll2cs.nc"))
    assert i.shape == (1440, 720) and int(p.max()) == 5 and int(i.max()) <= 15
    g = CubedSphere(16)
    ref = solver.adv_sphere(solver.Simulation(g, 0.05, 0.5, 2, 1, 3, 1, 3, 3, 2, 3))
    for a, b in zip((linf, l1, l2), ref):
        assert abs(a - b) <= 1e-10 * abs(b)
