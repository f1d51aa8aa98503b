"""ctypes binding of the native library libscg.so (include/scg.h).

The library must have been built (``solvcon_gb300.build.build()``); importing
this module without it raises ImportError.  There is no CPU fallback for the
march: every solver call goes through this library.
"""

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(_HERE, "_lib", "libscg.so")

if not os.path.exists(LIBPATH):
    raise ImportError(
        "solvcon_gb300 native library %s is missing; build it with "
        "python -c 'import solvcon_gb300.build as b; b.build()'" % LIBPATH)

lib = ctypes.CDLL(LIBPATH)

_c_i64p = ctypes.POINTER(ctypes.c_int64)
_vp = ctypes.c_void_p

_SIGS = {
    "scg_last_error": ([], ctypes.c_char_p),
    "scg_launch_count": ([], ctypes.c_int64),
    "scg_device_alloc_count": ([], ctypes.c_int64),
    "scg_geometry_round": ([_vp, _vp, ctypes.c_int64], ctypes.c_int),
    "scg_divide_check": ([_vp, _vp, _vp, _vp, _vp, ctypes.c_int64], ctypes.c_int),
    "scg_version": ([], ctypes.c_char_p),
    "scg_mesh_create": ([ctypes.c_int, ctypes.c_int64, ctypes.c_int64,
                         ctypes.c_int64, _vp], ctypes.c_int),
    "scg_mesh_destroy": ([_vp], ctypes.c_int),
    "scg_mesh_from_tables": ([_vp, _vp, _vp], ctypes.c_int),
    "scg_mesh_adopt_bc": ([_vp, ctypes.c_char_p, _vp, ctypes.c_int64],
                          ctypes.c_int),
    "scg_mesh_sizes": ([_vp, _vp], ctypes.c_int),
    "scg_mesh_array": ([_vp, ctypes.c_int, _vp, _vp, _vp, _vp, _vp],
                       ctypes.c_int),
    "scg_mesh_build_interior": ([_vp, ctypes.c_int, ctypes.c_int],
                                ctypes.c_int),
    "scg_mesh_build_edge": ([_vp], ctypes.c_int),
    "scg_mesh_add_bc": ([_vp, ctypes.c_char_p, _vp, ctypes.c_int64],
                        ctypes.c_int),
    "scg_mesh_bc": ([_vp, ctypes.c_int64, _vp, ctypes.c_int64, _vp, _vp],
                    ctypes.c_int),
    "scg_mesh_build_boundary": ([_vp], ctypes.c_int),
    "scg_mesh_build_ghost": ([_vp], ctypes.c_int),
    "scg_mesh_build_interior_device": ([_vp, ctypes.c_int, ctypes.c_int],
                                       ctypes.c_int),
    "scg_device_count": ([_vp], ctypes.c_int),
    "scg_mesh_from_gmsh": ([ctypes.c_char_p, ctypes.c_int64, _vp],
                           ctypes.c_int),
    "scg_mesh_from_plot3d": ([ctypes.c_char_p, ctypes.c_int64, _vp],
                             ctypes.c_int),
    "scg_euler_create": ([_vp, ctypes.c_double, ctypes.c_int, _vp],
                         ctypes.c_int),
    "scg_euler_destroy": ([_vp], ctypes.c_int),
    "scg_euler_info": ([_vp, _vp], ctypes.c_int),
    "scg_euler_get_param": ([_vp, ctypes.c_int, _vp], ctypes.c_int),
    "scg_euler_set_param": ([_vp, ctypes.c_int, ctypes.c_double],
                            ctypes.c_int),
    "scg_euler_array_shape": ([_vp, ctypes.c_int, _vp, _vp, _vp],
                              ctypes.c_int),
    "scg_euler_get": ([_vp, ctypes.c_int, _vp, ctypes.c_int64], ctypes.c_int),
    "scg_euler_set": ([_vp, ctypes.c_int, _vp, ctypes.c_int64], ctypes.c_int),
    "scg_euler_init_solution": ([_vp, ctypes.c_double, ctypes.c_double, _vp,
                                 ctypes.c_int, ctypes.c_double], ctypes.c_int),
    "scg_euler_add_bc": ([_vp, ctypes.c_int, _vp, ctypes.c_int64, _vp,
                          ctypes.c_int64], ctypes.c_int),
    "scg_euler_clear_bc": ([_vp], ctypes.c_int),
    "scg_euler_normal_matrix": ([_vp, ctypes.c_int32, _vp], ctypes.c_int),
    "scg_euler_op": ([_vp, ctypes.c_int], ctypes.c_int),
    "scg_euler_march": ([_vp, ctypes.c_int64], ctypes.c_int),
    "scg_euler_march_from_host": ([_vp, _vp, ctypes.c_int64, _vp, ctypes.c_int64,
                                   ctypes.c_int64], ctypes.c_int),
    "scg_euler_sync": ([_vp], ctypes.c_int),
    "scg_euler_deliver": ([_vp, ctypes.c_int, _vp, ctypes.c_int64],
                          ctypes.c_int),
    "scg_euler_set_stream": ([_vp, _vp], ctypes.c_int),
    "scg_euler_limiter_mask": ([_vp, _vp], ctypes.c_int),
    "scg_euler_totals": ([_vp, _vp], ctypes.c_int),
    "scg_euler_cfl_range": ([_vp, _vp], ctypes.c_int),
    "scg_euler_field": ([_vp, ctypes.c_int, _vp], ctypes.c_int),
    "scg_euler_device_bytes": ([_vp, _vp], ctypes.c_int),
    "scg_euler_stream": ([_vp, _vp], ctypes.c_int),
    "scg_euler_profile": ([_vp, ctypes.c_int], ctypes.c_int),
    "scg_euler_profile_stats": ([_vp, _vp, _vp], ctypes.c_int),
    "scg_fma_peak": ([ctypes.c_int, ctypes.c_int, _vp], ctypes.c_int),
    "scg_host_alloc": ([ctypes.c_int64, _vp], ctypes.c_int),
    "scg_host_free": ([_vp], ctypes.c_int),
    "scg_event_create": ([_vp], ctypes.c_int),
    "scg_event_destroy": ([_vp], ctypes.c_int),
    "scg_event_record": ([_vp, _vp], ctypes.c_int),
    "scg_event_elapsed": ([_vp, _vp, _vp], ctypes.c_int),
    "scg_device_sync": ([], ctypes.c_int),
}

EXPORTED = tuple(_SIGS)


def _bind(table):
    for name, (args, res) in table.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res


_bind(_SIGS)


def bind_more(table):
    """Bind further entry points (used by the 1D and batch modules)."""
    _bind(table)
    return lib


_ERRORS = {1: ValueError, 2: IndexError, 3: RuntimeError, 4: RuntimeError,
           5: MemoryError}


def check(rc):
    """Raise the Python exception matching a non-zero status code."""
    if rc != 0:
        msg = lib.scg_last_error().decode()
        raise _ERRORS.get(rc, RuntimeError)(msg)


def ptr(arr):
    """Data pointer of a contiguous numpy array as c_void_p."""
    return ctypes.c_void_p(arr.ctypes.data)


def i64buf(n):
    return np.zeros(n, dtype="int64")


def launch_count():
    """Kernels launched by libscg.so so far in this process."""
    return int(lib.scg_launch_count())


def device_alloc_count():
    """Device allocations the library has made so far in this process."""
    return int(lib.scg_device_alloc_count())
