"""ctypes binding of include/lbm_capi.h (the library built by fluidx3d_gb300/build.py).

There is no fallback: if the shared library is missing, importing the solver raises. Every non-zero
lbm_status becomes an ``LBMError`` carrying lbm_last_error().
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

LBM_OK = 0
STATUS_NAMES = {1: "INVALID_ARGUMENT", 2: "OUT_OF_MEMORY", 3: "CUDA", 4: "NOT_INITIALIZED", 5: "UNSUPPORTED", 6: "NO_DEVICE", 7: "IO"}
SRT, TRT = 0, 1
FP32, FP16S, FP16C = 0, 1, 2
EXT_VOLUME_FORCE, EXT_FORCE_FIELD, EXT_EQUILIBRIUM_BOUNDARIES, EXT_SUBGRID, EXT_MOVING_BOUNDARIES, EXT_UPDATE_FIELDS = 1, 2, 4, 8, 16, 32
FIELD_RHO, FIELD_U, FIELD_FLAGS, FIELD_F, FIELD_FI = 0, 1, 2, 3, 4
ARITH_AUTO, ARITH_EXACT, ARITH_FAST = 0, 1, 2
ARITHMETICS = {"auto": ARITH_AUTO, "exact": ARITH_EXACT, "fast": ARITH_FAST}

COLLISIONS = {"srt": SRT, "trt": TRT}
STORAGES = {"fp32": FP32, "fp16s": FP16S, "fp16c": FP16C}
EXTENSIONS = {"volume_force": EXT_VOLUME_FORCE, "force_field": EXT_FORCE_FIELD, "equilibrium_boundaries": EXT_EQUILIBRIUM_BOUNDARIES,
              "subgrid": EXT_SUBGRID, "moving_boundaries": EXT_MOVING_BOUNDARIES, "vf": EXT_VOLUME_FORCE, "ff": EXT_FORCE_FIELD,
              "update_fields": EXT_UPDATE_FIELDS, "eq": EXT_EQUILIBRIUM_BOUNDARIES, "sg": EXT_SUBGRID, "mb": EXT_MOVING_BOUNDARIES,
              "uf": EXT_UPDATE_FIELDS}


class LBMError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"lbm status {status} ({STATUS_NAMES.get(status, '?')}): {message}")
        self.status = status


class LBMConfig(ctypes.Structure):
    _fields_ = [("Nx", ctypes.c_uint32), ("Ny", ctypes.c_uint32), ("Nz", ctypes.c_uint32),
                ("velocity_set", ctypes.c_uint32), ("collision", ctypes.c_uint32), ("storage", ctypes.c_uint32),
                ("extensions", ctypes.c_uint32), ("device", ctypes.c_int32),
                ("nu", ctypes.c_float), ("fx", ctypes.c_float), ("fy", ctypes.c_float), ("fz", ctypes.c_float),
                ("arithmetic", ctypes.c_uint32)]


class AdjointConfig(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_uint64), ("checkpoint_interval", ctypes.c_uint64), ("objective", ctypes.c_uint32),
                ("plane_x", ctypes.c_uint32), ("marker", ctypes.c_uint32), ("workspace_limit_kib", ctypes.c_uint32),
                ("window_begin", ctypes.c_uint64), ("window_end", ctypes.c_uint64)]


class AdjointStats(ctypes.Structure):
    _fields_ = [("forward_ms", ctypes.c_double), ("recompute_ms", ctypes.c_double), ("adjoint_ms", ctypes.c_double),
                ("workspace_bytes", ctypes.c_uint64), ("levels", ctypes.c_uint32), ("overlapped", ctypes.c_uint32),
                ("reverse_ms", ctypes.c_double)]


OBJECTIVES = {"ke_plane": 1, "drag_x": 2}
OBJECT_SUM_STATIC_MAX_BLOCKS = 1216  # LBM_OBJECT_SUM_STATIC_MAX_BLOCKS

# every symbol include/lbm_capi.h declares, with (argtypes, restype)
_v, _i, _u8, _u32, _u64, _f, _d, _sz = (ctypes.c_void_p, ctypes.c_int, ctypes.c_uint8, ctypes.c_uint32, ctypes.c_uint64,
                                        ctypes.c_float, ctypes.c_double, ctypes.c_size_t)
_cfg = ctypes.POINTER(LBMConfig)
SIGNATURES = {
    "lbm_domain_create": ([_cfg, ctypes.POINTER(_v)], _i),
    "lbm_domain_destroy": ([_v], _i),
    "lbm_relaxation_rate": ([_f], _f),
    "lbm_bytes_per_cell_device": ([_cfg], _u32),
    "lbm_bandwidth_bytes_per_cell": ([_cfg], _u32),
    "lbm_set_stream": ([_v, _v], _i),
    "lbm_get_stream": ([_v, ctypes.POINTER(_v)], _i),
    "lbm_synchronize": ([_v], _i),
    "lbm_write_field": ([_v, _i, _v, _sz], _i),
    "lbm_read_field": ([_v, _i, _v, _sz], _i),
    "lbm_field_device_pointer": ([_v, _i, ctypes.POINTER(_v), ctypes.POINTER(_sz)], _i),
    "lbm_initialize": ([_v], _i),
    "lbm_stream_collide": ([_v, _u64], _i),
    "lbm_update_fields": ([_v], _i),
    "lbm_get_time_step": ([_v, ctypes.POINTER(_u64)], _i),
    "lbm_set_force": ([_v, _f, _f, _f], _i),
    "lbm_is_initialized": ([_v, ctypes.POINTER(_i)], _i),
    "lbm_reset": ([_v], _i),
    "lbm_update_force_field": ([_v], _i),
    "lbm_reset_force_field": ([_v], _i),
    "lbm_update_moving_boundaries": ([_v], _i),
    "lbm_write_vtk": ([_v, _i, ctypes.c_char_p, _f, _f], _i),
    "lbm_object_center_of_mass": ([_v, _u8, ctypes.POINTER(_d)], _i),
    "lbm_object_force": ([_v, _u8, ctypes.POINTER(_d)], _i),
    "lbm_object_torque": ([_v, _u8, _d, _d, _d, ctypes.POINTER(_d)], _i),
    "lbm_object_sum_static": ([_i, _u32, _u32, _u32, _v, _v, _u8, _i, _d, _d, _d, _u32, _v, ctypes.POINTER(_d)], _i),
    "lbm_voxelize_mesh": ([_v, _v, _v, _v, _u32, _u8, ctypes.POINTER(_f), ctypes.POINTER(_f), ctypes.POINTER(_f)], _i),
    "lbm_unvoxelize_mesh": ([_v, ctypes.POINTER(_f), ctypes.POINTER(_f), _u8], _i),
    "lbm_run_adjoint": ([_v, ctypes.POINTER(AdjointConfig), ctypes.POINTER(_d), _v, ctypes.POINTER(AdjointStats)], _i),
    "lbm_host_alloc": ([_sz, ctypes.POINTER(_v)], _i),
    "lbm_host_free": ([_v], _i),
    "lbm_last_error": ([], ctypes.c_char_p),
}

_lib = None


def library_path() -> str:
    return _build.LIB_PATH


def load(path: str | None = None) -> ctypes.CDLL:
    """Load the solver library (building it first only if FX3D_BUILD_ON_IMPORT=1)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or library_path()
    if not os.path.isfile(path):
        if os.environ.get("FX3D_BUILD_ON_IMPORT") == "1":
            _build.build()
        else:
            raise ImportError(f"fluidx3d_gb300 CUDA library not built: {path} is missing "
                              "(run `python -c 'import __graft_entry__ as g; g.build()'`)")
    L = ctypes.CDLL(path)
    for name, (argtypes, restype) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = argtypes
        fn.restype = restype
    _lib = L
    return L


def check(status: int) -> None:
    if status != LBM_OK:
        msg = load().lbm_last_error()
        raise LBMError(status, msg.decode() if msg else "")


def relaxation_rate(nu: float) -> float:
    return float(load().lbm_relaxation_rate(nu))


def pinned_empty(shape, dtype):
    """numpy array over page-locked host memory (freed when the array is garbage collected)."""
    import numpy as np
    dtype = np.dtype(dtype)
    nbytes = int(np.prod(shape)) * dtype.itemsize
    p = ctypes.c_void_p()
    check(load().lbm_host_alloc(nbytes, ctypes.byref(p)))
    buf = (ctypes.c_byte * nbytes).from_address(p.value)
    arr = np.frombuffer(buf, dtype=dtype).reshape(shape)
    import weakref
    weakref.finalize(buf, load().lbm_host_free, p.value)
    arr.flags.writeable = True
    return arr
