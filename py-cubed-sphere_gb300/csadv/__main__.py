"""``python -m csadv [pardir]``: the advection test case of the reference's main.py:78-95.

Reads par/configuration.par and par/advection.par (or those in `pardir`); test case 5 runs
one advection simulation (advection test case 1: adv_sphere, with the lat-lon fields written
as .npy where the reference plots them) or the convergence study (advection test case 2:
error_analysis_adv) on the GPU.  Like the reference's driver it creates grid/, data/ and the
graph directory, writes the grid file grid/<grid name>.nc and the lat-lon index file
grid/<grid name>_ll2cs.nc (netCDF classic).  Other test cases (grid generation, grid quality,
interpolation, divergence) are outside this library.
"""
import os
import sys

from . import advection, gridfile
from .advection import adv_simulation_par, adv_sphere, cubed_sphere, error_analysis_adv
from .configuration import PARDIR, get_advection_parameters, get_parameters
from .latlon import NLAT, NLON, latlon_grid, ll2cs


def create_dirs():
    """The output directories of the reference's driver (miscellaneous.py:27-45)."""
    for d in (gridfile.griddir, gridfile.datadir, advection.output_dir):
        if not os.path.exists(d):
            print("Creating directory ", d)
            os.makedirs(d)


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    pardir = argv[0] if argv else PARDIR
    N, transformation, showonscreen, gridload, test_case, map_projection = get_parameters(pardir)
    create_dirs()
    if test_case != 5:
        print("ERROR: this library runs the advection test case (5); configuration.par asks for", test_case)
        raise SystemExit(1)
    print("Test case 5: Advection test case.\n")
    cs_grid = cubed_sphere(N, transformation, showonscreen, gridload)
    # the grid file, as main.py:46-48 writes it (when absent, or always without gridload)
    gpath = os.path.join(gridfile.griddir, cs_grid.name + ".nc")
    if not os.path.isfile(gpath) or not gridload:
        gridfile.save_grid_netcdf4(cs_grid, gpath)
    dt, Tf, tc, ic, vf, recon, dp, opsplit, et, mt, mf = get_advection_parameters(pardir)
    simulation = adv_simulation_par(cs_grid, dt, Tf, ic, vf, tc, recon, dp, opsplit, et, mt, mf)
    if simulation.tc == 1:
        # the lat-lon grid of the plots (main.py:58-60)
        ll_grid = latlon_grid(NLAT, NLON)
        ll_grid.ix, ll_grid.jy, ll_grid.mask = ll2cs(cs_grid, ll_grid)
        return adv_sphere(cs_grid, ll_grid, simulation, map_projection, True, False)
    return error_analysis_adv(simulation, map_projection, False, transformation, showonscreen, gridload, pardir=pardir)


if __name__ == "__main__":
    main()
