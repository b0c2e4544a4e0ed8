"""ctypes binding of liblue_gb300.so (the C ABI declared in include/lue_gb300.h).

There is no CPU fallback: if the library is missing or cannot be loaded, every call raises.
"""
import ctypes
import os
import re

from . import _build

HEADER = os.path.join(_build.INCLUDE, "lue_gb300.h")

STATUS = {0: "OK", 1: "EINVAL", 2: "ESHAPE", 3: "ECUDA", 4: "ENOMEM", 5: "ETIMEDOUT", 6: "ERANGE"}


class LueGpuError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class TopologyStats(ctypes.Structure):
    _fields_ = [(name, ctypes.c_int64) for name in (
        "rows", "cols", "partition_rows", "partition_cols", "valid_cells", "ridge_cells", "outlet_cells",
        "sink_cells", "cycle_cells", "max_level", "device_bytes", "tile_exits", "exit_forest_depth")]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class StageSchedule(ctypes.Structure):
    _fields_ = [("cap", ctypes.c_int32), ("threads", ctypes.c_int32), ("publish_every", ctypes.c_int32),
                ("ms", ctypes.c_float)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


# int (*)(lue_gpu_topology*, void* user, void* stream): one routing call for the autotuner to time
STAGE_CALL = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p)

_lib = None


def declared_functions(header=HEADER):
    """Names of the functions declared in the public header."""
    text = open(header).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(lue_gpu_\w+)\s*\(", text, flags=re.M)))


def _declare(L):
    p, i64, i32, f, d = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_float, ctypes.c_double
    sig = {
        "lue_gpu_abi_version": ([], i32),
        "lue_gpu_last_error": ([], ctypes.c_char_p),
        "lue_gpu_kernel_launches": ([], ctypes.c_ulonglong),
        "lue_gpu_topology_create": ([p, i64, i64, i64, i64, p, ctypes.POINTER(p)], i32),
        "lue_gpu_topology_clone": ([p, ctypes.POINTER(p)], i32),
        "lue_gpu_topology_destroy": ([p], i32),
        "lue_gpu_topology_get_stats": ([p, ctypes.POINTER(TopologyStats)], i32),
        "lue_gpu_topology_prepare": ([p, p], i32),
        "lue_gpu_inflow_count_u8": ([p, i32, p, p], i32),
        "lue_gpu_accu_info_u8": ([p, p, p], i32),
        "lue_gpu_mark_no_data": ([p, i64, i32, p, p], i32),
        "lue_gpu_replace_no_data": ([p, p, i64, i32, p, p], i32),
        "lue_gpu_partial_accu_f32": ([p, i64, p, p, p], i32),
        "lue_gpu_partial_accu_f64": ([p, i64, p, p, p], i32),
        "lue_gpu_downstream_level_i32": ([p, p, p], i32),
        "lue_gpu_accu_f32": ([p, p, f, p, p], i32),
        "lue_gpu_accu_f64": ([p, p, d, p, p], i32),
        "lue_gpu_accu_threshold_f32": ([p, p, f, p, f, p, p, p], i32),
        "lue_gpu_accu_threshold_f64": ([p, p, d, p, d, p, p, p], i32),
        "lue_gpu_accu_fraction_f32": ([p, p, f, p, f, p, p, p], i32),
        "lue_gpu_accu_fraction_f64": ([p, p, d, p, d, p, p, p], i32),
        "lue_gpu_kinematic_wave_f64": ([p, p, d, p, d, p, d, p, d, d, p, d, p, p], i32),
        "lue_gpu_kinematic_wave_f64_f32in": ([p, p, d, p, d, p, d, d, d, d, p, p], i32),
        "lue_gpu_kinematic_wave_f32": ([p, p, f, p, f, p, f, p, f, f, p, f, p, p], i32),
        "lue_gpu_accu_f32_noalloc": ([p, i64, i64, i64, i64, p, f, p, p], i32),
        "lue_gpu_kinematic_wave_steps_f64_f32in": ([p, p, p, d, p, d, d, d, d, i32, p, p], i32),
        "lue_gpu_accu_capacity_f32": ([p, p, f, p, f, p, p, p], i32),
        "lue_gpu_accu_capacity_f64": ([p, p, d, p, d, p, p, p], i32),
        "lue_gpu_accu_trigger_f32": ([p, p, f, p, f, p, p, p], i32),
        "lue_gpu_accu_trigger_f64": ([p, p, d, p, d, p, p, p], i32),
        "lue_gpu_upstream_f32": ([p, i64, i64, p, p, p], i32),
        "lue_gpu_upstream_f64": ([p, i64, i64, p, p, p], i32),
        "lue_gpu_downstream_f32": ([p, i64, i64, p, p, p], i32),
        "lue_gpu_downstream_f64": ([p, i64, i64, p, p, p], i32),
        "lue_gpu_downstream_distance_f32": ([p, i64, i64, f, p, p], i32),
        "lue_gpu_downstream_distance_f64": ([p, i64, i64, d, p, p], i32),
        "lue_gpu_d8_flow_direction_f32": ([p, i64, i64, p, p], i32),
        "lue_gpu_d8_flow_direction_f64": ([p, i64, i64, p, p], i32),
        "lue_gpu_topology_get_stage_schedule": ([p, ctypes.POINTER(StageSchedule)], i32),
        "lue_gpu_topology_set_stage_schedule": ([p, ctypes.POINTER(StageSchedule)], i32),
        "lue_gpu_topology_set_stage_order": ([p, i32], i32),
        "lue_gpu_topology_get_stage_order": ([p, ctypes.POINTER(i32)], i32),
        "lue_gpu_autotune_stage_schedule": ([p, STAGE_CALL, p, i32, p, ctypes.POINTER(StageSchedule)], i32),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    return sig


def library_path():
    return os.path.join(_build.BUILD, "liblue_gb300.so")


def lib():
    """The loaded library (built first if this machine has nvcc and the .so is stale or missing)."""
    global _lib
    if _lib is None:
        path = library_path()
        if not os.path.exists(path):
            path = _build.gpu_library()
        L = ctypes.CDLL(path)
        _declare(L)
        _lib = L
    return _lib


def check(status):
    if status != 0:
        msg = lib().lue_gpu_last_error()
        raise LueGpuError(status, msg.decode() if msg else "")
