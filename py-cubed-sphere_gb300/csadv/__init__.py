"""csadv: GPU (GB300, sm_103a) advection time step of the gnomonic cubed sphere.

A drop-in for the advection path of luanfs/py-cubed-sphere: hand-written CUDA kernels in
``libcsadv.so`` (C ABI in include/csadv.h) driven from Python through ctypes.  The
reference's entry points are re-exported with the same names (``csadv.advection``).
"""
from ._lib import CsadvError  # noqa: F401
from .plan import Plan, host_array  # noqa: F401
from .batch import Batch, tune  # noqa: F401
from . import configuration  # noqa: F401
from .advection import (adv_simulation_par, adv_sphere, adv_time_step, compute_errors, cubed_sphere,  # noqa: F401
                        init_vars_adv, mass_computation, update_adv)

__all__ = ["Plan", "host_array", "Batch", "tune", "CsadvError", "cubed_sphere", "adv_simulation_par", "init_vars_adv",
           "adv_time_step", "update_adv", "adv_sphere", "mass_computation", "compute_errors", "configuration"]
