"""The C-ABI library builds, loads without a GPU and exports every function include/*.h declares."""
import ctypes
import glob
import os
import re
import subprocess

import pytest

from lue_gb300 import _build, _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        names.update(_lib.declared_functions(h))
    return sorted(names)


def test_header_declares_the_routing_operations():
    names = header_functions()
    for op in ("lue_gpu_topology_create", "lue_gpu_inflow_count_u8", "lue_gpu_accu_f32",
               "lue_gpu_accu_threshold_f32", "lue_gpu_accu_fraction_f32", "lue_gpu_kinematic_wave_f64"):
        assert op in names


def test_library_builds_and_exports_every_declared_symbol():
    path = _build.gpu_library()
    L = ctypes.CDLL(path)
    missing = [n for n in header_functions() if not hasattr(L, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (lue_gpu_\w+)", out))
    assert set(header_functions()) <= exported


def test_abi_version_without_gpu():
    L = _lib.lib()
    assert L.lue_gpu_abi_version() == 1


def test_bad_arguments_fail_without_touching_the_gpu():
    L = _lib.lib()
    h = ctypes.c_void_p()
    rc = L.lue_gpu_topology_create(None, 4, 4, 2, 2, None, ctypes.byref(h))
    assert rc == 1 and b"NULL" in L.lue_gpu_last_error()
    rc = L.lue_gpu_topology_create(ctypes.c_void_p(16), 4, 4, 8, 2, None, ctypes.byref(h))
    assert rc == 1 and b"partition" in L.lue_gpu_last_error()
    rc = L.lue_gpu_topology_create(ctypes.c_void_p(16), 0, 4, 1, 1, None, ctypes.byref(h))
    assert rc == 1
    assert L.lue_gpu_accu_f32(None, None, 1.0, None, None) == 1
    assert L.lue_gpu_topology_destroy(None) == 1


def test_schedule_and_autotune_entry_points_reject_bad_arguments_without_a_gpu():
    L = _lib.lib()
    s = _lib.StageSchedule()
    assert L.lue_gpu_topology_get_stage_schedule(None, ctypes.byref(s)) == 1
    assert L.lue_gpu_topology_set_stage_schedule(None, ctypes.byref(s)) == 1
    cb = _lib.STAGE_CALL(lambda handle, user, stream: 0)
    assert L.lue_gpu_autotune_stage_schedule(None, cb, None, 1, None, ctypes.byref(s)) == 1
    assert b"NULL" in L.lue_gpu_last_error()
    order = ctypes.c_int(-1)
    assert L.lue_gpu_topology_set_stage_order(None, 0) == 1
    assert L.lue_gpu_topology_get_stage_order(None, ctypes.byref(order)) == 1
    assert b"NULL" in L.lue_gpu_last_error() and order.value == -1
