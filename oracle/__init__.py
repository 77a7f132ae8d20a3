"""CPU oracle for the cubed-sphere advection time step -- TEST INFRASTRUCTURE ONLY.

This package is a plain-numpy restatement of the advection path of luanfs/py-cubed-sphere
(grid generation, Lagrange ghost cells, PPM reconstructions and limiters, upwind fluxes,
dimension splitting, mass fixers, departure-point winds, error diagnostics).  Each
function cites the reference file:line it restates.

It exists to CHECK the CUDA library, never to stand in for it:

* only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
  may import it;
* the library (``py-cubed-sphere_gb300/csadv``) never imports it and has no CPU fallback.

The oracle is pinned against golden vectors produced by running the reference itself
(``tests/golden/make_golden.py``; fixtures in ``tests/golden/*.npz``): see
``tests/test_oracle_golden.py``.

Arrays use the reference's layout ``A[i, j, p]`` (p = panel, fastest varying), with
``ng = 8`` ghost cells (4 on each side), interior ``i, j in [4, N+4)``.
"""
from .grid import CubedSphere  # noqa: F401
from .solver import Simulation, adv_sphere, run_steps  # noqa: F401
