"""Readers for the reference's positional parameter files (configuration.py:13-158).

Both files alternate comment lines and value lines; values are read by position, as the
reference does, so existing ``par/configuration.par`` / ``par/advection.par`` files work
unchanged.  Invalid values print an error and raise ``SystemExit`` like the reference's
``exit()``.
"""
import os

PARDIR = "par/"


def _read_values(path, count):
    with open(path, "r") as f:
        lines = f.readlines()
    # a title line, then (comment line, value line) pairs: value k is line 2k+2 (0-based)
    vals = []
    for k in range(count):
        idx = 2 * k + 2
        if idx >= len(lines):
            print("ERROR: parameter file %s is truncated" % path)
            raise SystemExit(1)
        vals.append(lines[idx])
    return vals


def get_parameters(pardir=PARDIR, verbose=True):
    """par/configuration.par -> (N, transformation, showonscreen, gridload, test_case, map_projection)."""
    path = os.path.join(pardir, "configuration.par")
    if not os.path.exists(path):
        print("ERROR in get_grid_parameters: file mesh.par not found in /par.")
        raise SystemExit(1)
    N, transf, gridload, show, tc, mproj = _read_values(path, 6)
    N = int(N)
    showonscreen = bool(int(show))
    gridload = bool(int(gridload))
    transf = int(transf)
    test_case = int(tc)
    mproj = int(mproj)
    maps = {1: "mercator", 2: "sphere"}
    if mproj not in maps:
        print("ERROR: invalid map projection")
        raise SystemExit(1)
    transfs = {1: "gnomonic_equidistant", 2: "gnomonic_equiangular", 3: "overlapped"}
    if transf not in transfs:
        print("ERROR: invalid transformation")
        raise SystemExit(1)
    if transf == 3:
        gridload = True
    if verbose:
        print("\n--------------------------------------------------------")
        print("Parameters from file", path, "\n")
        print("Number of cells along a coordinate axis: ", N)
        print("Show process on the screen: ", showonscreen)
        print("Loadable grid: ", gridload)
        print("Transformation:", transfs[transf])
        print("Test case to be done: ", test_case)
        print("Map projection: ", maps[mproj])
        print("--------------------------------------------------------\n")
    return N, transfs[transf], showonscreen, gridload, test_case, maps[mproj]


def get_advection_parameters(pardir=PARDIR, verbose=True):
    """par/advection.par -> (dt, Tf, tc, ic, vf, recon, dp, opsplit, et, mt, mf)."""
    path = os.path.join(pardir, "advection.par")
    if not os.path.exists(path):
        print("ERROR in get_grid_parameters: file " + path + " not found in /par.")
        raise SystemExit(1)
    v = _read_values(path, 11)
    Tf, dt = float(v[0]), float(v[1])
    ic, vf, tc, recon, dp, opsplit, et, mt, mf = (int(x) for x in v[2:])
    if verbose:
        print("\n--------------------------------------------------------")
        print("Parameters from file", path, "\n")
        for name, val in (("Total time of integration: ", Tf), ("Time step: ", dt), ("Initial condition: ", ic),
                          ("Vector field: ", vf), ("Adv test case: ", tc), ("Reconstruction scheme: ", recon),
                          ("Departure point scheme: ", dp), ("Splitting scheme: ", opsplit),
                          ("Edge treatment: ", et), ("Metric tensor treatment: ", mt), ("Mass fixer: ", mf)):
            print(name, val)
        print("--------------------------------------------------------\n")
    return dt, Tf, tc, ic, vf, recon, dp, opsplit, et, mt, mf
