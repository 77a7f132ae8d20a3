"""ctypes binding of libcsadv.so (C ABI declared in include/csadv.h).

The library is built in-tree by ``csadv/build.py`` (``__graft_entry__.build()``).  There is
no fallback: if the shared library is missing or a CUDA device is unavailable, the calls
raise ``CsadvError``.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcsadv.so")

OK = 0
ERR_OPTION = -1
ERR_OPTION_PAIR = -2
ERR_ARG = -3
ERR_OOM = -4
ERR_CUDA = -5
ERR_NONFINITE = -6
ERR_BLOWUP = -7
ERR_UNSUPPORTED = -8
ERR_TOO_LARGE = -9

LAYOUT_FULL = 0
LAYOUT_INTERIOR = 1

ENGINE_AUTO, ENGINE_STAGED, ENGINE_FUSED = 0, 1, 2

WIND_SOLID, WIND_DEFORM, WIND_SOLID_DIV = 101, 102, 103
IC_HILL, IC_BELLS, IC_SMOOTH_BELLS = 101, 102, 103


class CsadvError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = status_string(status) if _lib is not None else "status %d" % status
        super().__init__("%s%s (status %d)" % (what + ": " if what else "", msg, status))


class Options(ctypes.Structure):
    _fields_ = [
        ("recon", ctypes.c_int), ("dp", ctypes.c_int), ("opsplit", ctypes.c_int), ("et", ctypes.c_int),
        ("mt", ctypes.c_int), ("mf", ctypes.c_int), ("vf", ctypes.c_int), ("precision", ctypes.c_int),
        ("engine", ctypes.c_int), ("tile", ctypes.c_int), ("wind_param", ctypes.c_double * 4),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("steps", ctypes.c_longlong), ("kernel_launches", ctypes.c_longlong), ("main_launches", ctypes.c_longlong),
        ("main_ms", ctypes.c_double), ("kernels_per_step", ctypes.c_int), ("engine", ctypes.c_int),
        ("tile", ctypes.c_int), ("reserved", ctypes.c_int), ("device_bytes", ctypes.c_size_t),
        ("graph_builds", ctypes.c_longlong), ("graph_build_ms", ctypes.c_double),
    ]


_lib = None

_c_int, _c_double, _vp = ctypes.c_int, ctypes.c_double, ctypes.c_void_p
_dp = ctypes.POINTER(ctypes.c_double)
_SIGS = {
    "csadv_version": ([], ctypes.c_char_p),
    "csadv_status_string": ([_c_int], ctypes.c_char_p),
    "csadv_set_device": ([_c_int], _c_int),
    "csadv_plan_create": ([_c_int, _c_double, _c_int, ctypes.POINTER(Options), _vp, ctypes.POINTER(_vp)], _c_int),
    "csadv_plan_destroy": ([_vp], _c_int),
    "csadv_plan_release": ([_vp, _vp], _c_int),
    "csadv_get_dt": ([_vp, _dp], _c_int),
    "csadv_init_tracer": ([_vp, _c_int, _c_int, _dp, _vp], _c_int),
    "csadv_set_tracer": ([_vp, _c_int, _vp, _c_int, _vp], _c_int),
    "csadv_get_tracer": ([_vp, _c_int, _vp, _c_int, _vp], _c_int),
    "csadv_time_step": ([_vp, _c_int, _vp], _c_int),
    "csadv_update_winds": ([_vp, _c_double, _vp], _c_int),
    "csadv_advance": ([_vp, _c_int, _vp], _c_int),
    "csadv_advance_host": ([_vp, _c_int, _vp, _c_int, _vp, _c_int, _vp], _c_int),
    "csadv_mass": ([_vp, _c_int, _dp, _vp], _c_int),
    "csadv_errors": ([_vp, _c_int, _c_int, _dp, _c_double, _dp, _vp], _c_int),
    "csadv_get_cfl": ([_vp, _dp], _c_int),
    "csadv_get_step": ([_vp, ctypes.POINTER(_c_int)], _c_int),
    "csadv_divergence": ([_vp, _c_int, _vp, _vp], _c_int),
    "csadv_set_graphs": ([_vp, _c_int], _c_int),
    "csadv_set_profiling": ([_vp, _c_int], _c_int),
    "csadv_set_inline_ghosts": ([_vp, _c_int], _c_int),
    "csadv_get_stats": ([_vp, ctypes.POINTER(Stats)], _c_int),
    "csadv_reset_stats": ([_vp], _c_int),
    "csadv_batch_create": ([_c_int, ctypes.POINTER(_vp)], _c_int),
    "csadv_batch_destroy": ([_vp], _c_int),
    "csadv_batch_add": ([_vp, _vp], _c_int),
    "csadv_batch_remove": ([_vp, _vp], _c_int),
    "csadv_batch_size": ([_vp, ctypes.POINTER(_c_int)], _c_int),
    "csadv_batch_advance": ([_vp, _c_int, _vp], _c_int),
    "csadv_batch_set_queue_depth": ([_vp, _c_int], _c_int),
    "csadv_batch_set_graphs": ([_vp, _c_int], _c_int),
    "csadv_batch_get_stats": ([_vp, ctypes.POINTER(Stats)], _c_int),
    "csadv_batch_set_profiling": ([_vp, _c_int], _c_int),
    "csadv_batch_reset_stats": ([_vp], _c_int),
    "csadv_tune": ([_vp, _c_int, _vp, ctypes.POINTER(_c_int)], _c_int),
    "csadv_mass_fixer_noalloc": ([_vp, _vp, _vp, _c_int, _vp], _c_int),
    "csadv_host_alloc": ([ctypes.POINTER(_vp), ctypes.c_size_t], _c_int),
    "csadv_grid_points": ([_c_int, _c_int, _vp, _vp, _vp, _vp], _c_int),
    "csadv_ll2cs": ([_c_int, _vp, _vp, _vp, ctypes.c_longlong, _vp, _vp, _vp, _vp], _c_int),
    "csadv_set_step": ([_vp, _c_int, _vp], _c_int),
    "csadv_mass_target": ([_vp, _c_int, _dp, _dp, _vp], _c_int),
    "csadv_nearest_neighbour": ([_vp, _c_int, _vp, _vp, _vp, ctypes.c_longlong, _vp, _vp], _c_int),
    "csadv_host_free": ([_vp], _c_int),
    "csadv_fp64_rate": ([_c_int, _dp, _vp], _c_int),
}


def lib():
    """Load libcsadv.so (once) and declare the prototypes."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise CsadvError(ERR_UNSUPPORTED, "libcsadv.so not built (run __graft_entry__.build())")
        L = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def status_string(status):
    return lib().csadv_status_string(status).decode()


def check(status, what=""):
    if status != OK:
        raise CsadvError(status, what)
    return status


def stream_handle(stream):
    """Accept None, an int handle, or a torch.cuda.Stream."""
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return getattr(stream, "cuda_stream", None) or None
