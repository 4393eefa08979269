"""ctypes binding of libtisphi_gb300.so (the C ABI declared in include/tisphi_gb300.h).

The library is the only compute path: importing this module fails loudly when the shared
library has not been built, and there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtisphi_gb300.so")

TSG_FP64, TSG_FP32_MIXED = 0, 1
TSG_ADVECT_FULL, TSG_ADVECT_LF_HALF, TSG_ADVECT_POS, TSG_ADVECT_SOMETHING, TSG_ENFORCE_BOUNDARY, \
    TSG_RK_INIT, TSG_RK_STAGE, TSG_RK_FINAL = range(1, 9)
TSG_ERR_CELL_OOB, TSG_ERR_NONFINITE, TSG_ERR_PACK_RANGE = 1, 2, 4
PHASES = ("sort", "kernel_corr", "init_tmp", "eos_adapt", "boundary", "rates", "integrate", "advect_pos",
          "post", "other", "neighbour_lists")


class tsg_config(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int32), ("solver", ctypes.c_int32), ("kernel", ctypes.c_int32),
        ("kernel_corr", ctypes.c_int32), ("time_integration", ctypes.c_int32), ("xsph", ctypes.c_int32),
        ("boundary", ctypes.c_int32), ("precision", ctypes.c_int32), ("exponent_is_int", ctypes.c_int32),
        ("init_geostatic", ctypes.c_int32), ("grid_num", ctypes.c_int32 * 3), ("grid_num_total", ctypes.c_int64),
        ("vdomain_start", ctypes.c_double * 3), ("domain_start", ctypes.c_double * 3),
        ("domain_end", ctypes.c_double * 3), ("grid_size", ctypes.c_double), ("support_radius", ctypes.c_double),
        ("smoothing_len", ctypes.c_double), ("particle_diameter", ctypes.c_double),
        ("particle_radius", ctypes.c_double), ("gravity", ctypes.c_double * 3), ("dt", ctypes.c_double),
        ("density0", ctypes.c_double), ("viscosity", ctypes.c_double), ("stiffness", ctypes.c_double),
        ("exponent", ctypes.c_double), ("cohesion", ctypes.c_double), ("friction", ctypes.c_double),
        ("E", ctypes.c_double), ("poisson", ctypes.c_double), ("dilatancy", ctypes.c_double),
        ("damping_eps", ctypes.c_double), ("list_skin", ctypes.c_double),
    ]


_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)


class tsg_particles(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("x", _dp), ("v", _dp), ("density", _dp), ("mass", _dp), ("m_V", _dp),
                ("pressure", _dp), ("stress", _dp), ("mat_type", _ip), ("mat_id", _ip), ("obj_id", _ip),
                ("is_dynamic", _ip)]


class tsg_launch_cfg(ctypes.Structure):
    _fields_ = [("threads_per_block", ctypes.c_int32), ("cells_per_cta", ctypes.c_int32),
                ("steps_per_graph", ctypes.c_int32)]


class tsg_visual_cfg(ctypes.Structure):
    _fields_ = [("color_title", ctypes.c_int32), ("color_group", ctypes.c_int32), ("show_bdy", ctypes.c_int32),
                ("fix_max", ctypes.c_int32), ("fix_min", ctypes.c_int32), ("w2s_ratio", ctypes.c_double),
                ("given_max", ctypes.c_double), ("given_min", ctypes.c_double)]


class tsg_view(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("dtype", ctypes.c_int32), ("ndim", ctypes.c_int32),
                ("shape", ctypes.c_int64 * 3), ("strides", ctypes.c_int64 * 3)]


SYMBOLS = {
    "tsg_create": (ctypes.c_int, [ctypes.POINTER(tsg_config), ctypes.POINTER(ctypes.c_void_p)]),
    "tsg_upload": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(tsg_particles), ctypes.c_int, ctypes.c_void_p]),
    "tsg_sort": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "tsg_kernel_corr": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "tsg_init_tmp": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "tsg_one_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "tsg_advect": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "tsg_substep": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "tsg_rk_update": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]),
    "tsg_density_sum": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "tsg_solve_rigid_body": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "tsg_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "tsg_field": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(tsg_view), ctypes.c_void_p]),
    "tsg_particle_num": (ctypes.c_int64, [ctypes.c_void_p]),
    "tsg_grid": (ctypes.c_int, [ctypes.c_void_p, _ip, ctypes.c_void_p]),
    "tsg_neighbors": (ctypes.c_int, [ctypes.c_void_p, _ip, _ip, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64),
                                     ctypes.c_void_p]),
    "tsg_reduce_diag": (ctypes.c_int, [ctypes.c_void_p, _dp, ctypes.c_void_p]),
    "tsg_list_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64), ctypes.c_void_p]),
    "tsg_last_error": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "tsg_visual": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, _dp,
                                  ctypes.c_void_p]),
    "tsg_set_soil": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_double]),
    "tsg_set_fluid": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_double]),
    "tsg_snapshot_bytes": (ctypes.c_int64, [ctypes.c_void_p]),
    "tsg_snapshot_save": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "tsg_snapshot_load": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "tsg_adjoint_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "tsg_set_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "tsg_get_launch": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "tsg_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, _dp, ctypes.c_void_p]),
    "tsg_batch_create": (ctypes.c_int, [ctypes.POINTER(tsg_config), ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                                        ctypes.POINTER(ctypes.c_void_p)]),
    "tsg_batch_diag": (ctypes.c_int, [ctypes.c_void_p, _dp, ctypes.c_int32, ctypes.c_void_p]),
    "tsg_batch_pitch": (ctypes.c_double, [ctypes.c_void_p]),
    "tsg_write": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "tsg_read": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]),
    "tsg_read_fields": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_char_p),
                                       ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_void_p]),
    "tsg_launch_count": (ctypes.c_int64, []),
    "tsg_profile": (ctypes.c_int, [ctypes.c_int]),
    "tsg_profile_read": (ctypes.c_int, [_dp, ctypes.POINTER(ctypes.c_int64), ctypes.c_int]),
    "tsg_sort_noalloc": (ctypes.c_int, [ctypes.POINTER(tsg_config), ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p]),
    "tsg_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "tsg_destroy": (None, [ctypes.c_void_p]),
}

_lib = None


def load():
    """Load the shared library (no fallback: raises when it is missing)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"libtisphi_gb300.so not built ({LIB_PATH}); run tisphi_gb300/build_native.py")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SYMBOLS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


class NativeError(RuntimeError):
    def __init__(self, status, what):
        self.status = status
        super().__init__(f"{what}: status {status} ({load().tsg_status_string(status).decode()})")


def check(status, what):
    if status != 0:
        raise NativeError(status, what)
    return status


_TYPESTR = {0: "<f8", 1: "<f4", 2: "<i4"}
_ITEMSIZE = {0: 8, 1: 4, 2: 4}


class DeviceArray:
    """Strided device buffer exposed through ``__cuda_array_interface__`` (zero copy)."""

    def __init__(self, view: tsg_view, owner):
        nd = view.ndim
        item = _ITEMSIZE[view.dtype]
        self._owner = owner
        self.__cuda_array_interface__ = {
            "shape": tuple(int(view.shape[k]) for k in range(nd)),
            "typestr": _TYPESTR[view.dtype],
            "data": (int(view.data or 0), False),
            "strides": tuple(int(view.strides[k]) * item for k in range(nd)),
            "version": 3,
        }


def as_ptr(arr, ctype):
    return arr.ctypes.data_as(ctypes.POINTER(ctype)) if arr is not None else None


def host_particles(scene):
    """tsg_particles pointing at contiguous host copies of a SceneArrays (kept alive by the caller)."""
    keep = {
        "x": np.ascontiguousarray(scene.x, dtype=np.float64),
        "v": np.ascontiguousarray(scene.v, dtype=np.float64),
        "density": np.ascontiguousarray(scene.density, dtype=np.float64),
        "mass": np.ascontiguousarray(scene.mass, dtype=np.float64),
        "m_V": np.ascontiguousarray(scene.m_V, dtype=np.float64),
        "pressure": np.ascontiguousarray(scene.pressure, dtype=np.float64),
        "stress": np.ascontiguousarray(scene.stress.reshape(-1, 9), dtype=np.float64),
        "mat_type": np.ascontiguousarray(scene.mat_type, dtype=np.int32),
        "mat_id": np.ascontiguousarray(scene.mat_id, dtype=np.int32),
        "obj_id": np.ascontiguousarray(scene.obj_id, dtype=np.int32),
        "is_dynamic": np.ascontiguousarray(scene.is_dynamic, dtype=np.int32),
    }
    p = tsg_particles()
    p.n = scene.n
    for k in ("x", "v", "density", "mass", "m_V", "pressure", "stress"):
        setattr(p, k, as_ptr(keep[k], ctypes.c_double))
    for k in ("mat_type", "mat_id", "obj_id", "is_dynamic"):
        setattr(p, k, as_ptr(keep[k], ctypes.c_int32))
    return p, keep
