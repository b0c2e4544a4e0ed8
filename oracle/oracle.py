"""ctypes wrapper of the CPU oracle (lue_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg, never by the lue_gb300 package.  Every function takes and returns numpy arrays in row-major
layout plus the reference's ``partition_shape``; a ``None`` raster argument means "use the scalar".
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "liblue_oracle.so")
SOURCES = [os.path.join(HERE, "lue_oracle.c"), os.path.join(HERE, "router_impl.h")]


def build(force=False):
    """Compile lue_oracle.c with gcc into oracle/_build/liblue_oracle.so (seconds)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if not force and os.path.exists(LIB_PATH):
        if os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(s) for s in SOURCES):
            return LIB_PATH
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-pthread", "-o", tmp,
                           os.path.join(HERE, "lue_oracle.c"), "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        i64, p, i32 = ctypes.c_int64, ctypes.c_void_p, ctypes.c_int
        for sfx, real in (("f32", ctypes.c_float), ("f64", ctypes.c_double)):
            f = getattr(L, f"lue_oracle_accu_{sfx}")
            f.argtypes = [p, i64, i64, i64, i64, p, real, p, i32]
            f = getattr(L, f"lue_oracle_accu_threshold_{sfx}")
            f.argtypes = [p, i64, i64, i64, i64, p, real, p, real, p, p, i32]
            f = getattr(L, f"lue_oracle_accu_fraction_{sfx}")
            f.argtypes = [p, i64, i64, i64, i64, p, real, p, real, p, p, i32]
            f = getattr(L, f"lue_oracle_kinematic_wave_{sfx}")
            f.argtypes = [p, i64, i64, i64, i64, p, real, p, real, p, real, p, real, real, p, real, p, i32]
            for op in ("accu_capacity", "accu_trigger"):
                getattr(L, f"lue_oracle_{op}_{sfx}").argtypes = [p, i64, i64, i64, i64, p, real, p, real, p, p, i32]
            getattr(L, f"lue_oracle_upstream_{sfx}").argtypes = [p, i64, i64, p, p]
            getattr(L, f"lue_oracle_downstream_{sfx}").argtypes = [p, i64, i64, p, p]
            getattr(L, f"lue_oracle_downstream_distance_{sfx}").argtypes = [p, i64, i64, real, p]
        L.lue_oracle_inflow_count.argtypes = [p, i64, i64, i64, i64, i32, p]
        L.lue_oracle_accu_info.argtypes = [p, i64, i64, i64, i64, p]
        L.lue_oracle_partial_accu.argtypes = [p, i64, i64, i64, i64, i64, i32, p]
        L.lue_oracle_downstream_level.argtypes = [p, i64, i64, p]
        L.lue_oracle_d8_flow_direction.argtypes = [p, i64, i64, p]
        d = ctypes.c_double
        L.lue_oracle_iterate_to_new_discharge_f64.argtypes = [d] * 7
        L.lue_oracle_iterate_to_new_discharge_f64.restype = d
        L.lue_oracle_iterate_to_new_discharge_f32.argtypes = [ctypes.c_float] * 7
        L.lue_oracle_iterate_to_new_discharge_f32.restype = ctypes.c_float
        _lib = L
    return _lib


def _sfx(dtype):
    return {np.dtype(np.float32): "f32", np.dtype(np.float64): "f64"}[np.dtype(dtype)]


def _raster(x, shape, dtype):
    """(pointer, scalar, keepalive) for a raster-or-scalar argument."""
    if x is None:
        raise ValueError("argument missing")
    if np.isscalar(x) or (isinstance(x, np.ndarray) and x.ndim == 0):
        return None, dtype(x), None
    a = np.ascontiguousarray(x, dtype=dtype)
    if a.shape != shape:
        raise ValueError(f"raster shape {a.shape} differs from flow direction shape {shape}")
    return a.ctypes.data, dtype(0), a


def _fd(fd):
    fd = np.ascontiguousarray(fd, dtype=np.uint8)
    if fd.ndim != 2:
        raise ValueError("flow direction must be 2-D")
    return fd


def _pshape(fd, partition_shape):
    return tuple(fd.shape) if partition_shape is None else tuple(int(v) for v in partition_shape)


def _check(rc):
    if rc != 0:
        raise RuntimeError(f"oracle returned {rc}")


def inflow_count(fd, partition_shape=None, value_policies=True):
    fd = _fd(fd)
    pr, pc = _pshape(fd, partition_shape)
    out = np.empty(fd.shape, np.uint8)
    _check(lib().lue_oracle_inflow_count(fd.ctypes.data, fd.shape[0], fd.shape[1], pr, pc,
                                         int(value_policies), out.ctypes.data))
    return out


def accu_info(fd, partition_shape=None):
    """accu_info: the class of every cell after the reference router's event sequence (uint8, 255 no-data;
    inter-partition arrivals in FIFO order)."""
    fd = _fd(fd)
    pr, pc = _pshape(fd, partition_shape)
    out = np.empty(fd.shape, np.uint8)
    _check(lib().lue_oracle_accu_info(fd.ctypes.data, fd.shape[0], fd.shape[1], pr, pc, out.ctypes.data))
    return out


def partial_accu(fd, nr_steps, partition_shape=None, order=0):
    """partial_accu: the reference router's event sequence with the PartialAccu hooks (float64; NaN for
    no-data).  order 0: inter-partition arrivals in one FIFO; order 1: the mail of the highest-numbered
    partition first (another order HPX may deliver)."""
    fd = _fd(fd)
    pr, pc = _pshape(fd, partition_shape)
    out = np.empty(fd.shape, np.float64)
    _check(lib().lue_oracle_partial_accu(fd.ctypes.data, fd.shape[0], fd.shape[1], pr, pc, int(nr_steps), int(order),
                                         out.ctypes.data))
    return out


def d8_flow_direction(elevation):
    """Reference D8 rule on a float64 elevation raster (float32 input is promoted exactly)."""
    z = np.ascontiguousarray(elevation, dtype=np.float64)
    out = np.empty(z.shape, np.uint8)
    _check(lib().lue_oracle_d8_flow_direction(z.ctypes.data, z.shape[0], z.shape[1], out.ctypes.data))
    return out


def downstream_level(fd):
    fd = _fd(fd)
    out = np.empty(fd.shape, np.int32)
    _check(lib().lue_oracle_downstream_level(fd.ctypes.data, fd.shape[0], fd.shape[1], out.ctypes.data))
    return out


def accu(fd, inflow, partition_shape=None, dtype=np.float32, nthreads=1):
    fd = _fd(fd)
    pr, pc = _pshape(fd, partition_shape)
    t = np.dtype(dtype).type
    p, s, keep = _raster(inflow, fd.shape, t)
    out = np.empty(fd.shape, dtype)
    _check(getattr(lib(), f"lue_oracle_accu_{_sfx(dtype)}")(
        fd.ctypes.data, fd.shape[0], fd.shape[1], pr, pc, p, s, out.ctypes.data, nthreads))
    del keep
    return out


def accu_threshold(fd, inflow, threshold, partition_shape=None, dtype=np.float32, nthreads=1):
    fd = _fd(fd)
    pr, pc = _pshape(fd, partition_shape)
    t = np.dtype(dtype).type
    p0, s0, k0 = _raster(inflow, fd.shape, t)
    p1, s1, k1 = _raster(threshold, fd.shape, t)
    flux = np.empty(fd.shape, dtype)
    state = np.empty(fd.shape, dtype)
    _check(getattr(lib(), f"lue_oracle_accu_threshold_{_sfx(dtype)}")(
        fd.ctypes.data, fd.shape[0], fd.shape[1], pr, pc, p0, s0, p1, s1,
        flux.ctypes.data, state.ctypes.data, nthreads))
    del k0, k1
    return flux, state


def accu_fraction(fd, inflow, fraction, partition_shape=None, dtype=np.float32, nthreads=1):
    fd = _fd(fd)
    pr, pc = _pshape(fd, partition_shape)
    t = np.dtype(dtype).type
    p0, s0, k0 = _raster(inflow, fd.shape, t)
    p1, s1, k1 = _raster(fraction, fd.shape, t)
    flux = np.empty(fd.shape, dtype)
    state = np.empty(fd.shape, dtype)
    _check(getattr(lib(), f"lue_oracle_accu_fraction_{_sfx(dtype)}")(
        fd.ctypes.data, fd.shape[0], fd.shape[1], pr, pc, p0, s0, p1, s1,
        flux.ctypes.data, state.ctypes.data, nthreads))
    del k0, k1
    return flux, state


def _two_output(op, fd, inflow, other, partition_shape, dtype, nthreads):
    fd = _fd(fd)
    pr, pc = _pshape(fd, partition_shape)
    t = np.dtype(dtype).type
    p0, s0, k0 = _raster(inflow, fd.shape, t)
    p1, s1, k1 = _raster(other, fd.shape, t)
    outflow = np.empty(fd.shape, dtype)
    remainder = np.empty(fd.shape, dtype)
    _check(getattr(lib(), f"lue_oracle_{op}_{_sfx(dtype)}")(
        fd.ctypes.data, fd.shape[0], fd.shape[1], pr, pc, p0, s0, p1, s1,
        outflow.ctypes.data, remainder.ctypes.data, nthreads))
    del k0, k1
    return outflow, remainder


def accu_capacity(fd, inflow, capacity, partition_shape=None, dtype=np.float32, nthreads=1):
    """(outflow, remainder): what flows on is capped at the capacity, the rest stays."""
    return _two_output("accu_capacity", fd, inflow, capacity, partition_shape, dtype, nthreads)


def accu_trigger(fd, inflow, trigger, partition_shape=None, dtype=np.float32, nthreads=1):
    """(outflow, remainder): the total flows on once it reaches the trigger, else it all stays."""
    return _two_output("accu_trigger", fd, inflow, trigger, partition_shape, dtype, nthreads)


def _one_hop(op, fd, material, dtype):
    fd = _fd(fd)
    m = np.ascontiguousarray(material, dtype)
    out = np.empty(fd.shape, dtype)
    _check(getattr(lib(), f"lue_oracle_{op}_{_sfx(dtype)}")(fd.ctypes.data, fd.shape[0], fd.shape[1],
                                                           m.ctypes.data, out.ctypes.data))
    return out


def upstream(fd, material, dtype=np.float64):
    return _one_hop("upstream", fd, material, dtype)


def downstream(fd, material, dtype=np.float64):
    return _one_hop("downstream", fd, material, dtype)


def downstream_distance(fd, cell_size, dtype=np.float64):
    fd = _fd(fd)
    out = np.empty(fd.shape, dtype)
    _check(getattr(lib(), f"lue_oracle_downstream_distance_{_sfx(dtype)}")(
        fd.ctypes.data, fd.shape[0], fd.shape[1], np.dtype(dtype).type(cell_size), out.ctypes.data))
    return out


def kinematic_wave(fd, current_outflow, inflow, alpha, beta, time_step_duration, channel_length,
                   partition_shape=None, dtype=np.float64, nthreads=1):
    """One time step.  Float32 rasters passed with dtype=float64 are promoted exactly."""
    fd = _fd(fd)
    pr, pc = _pshape(fd, partition_shape)
    t = np.dtype(dtype).type
    args = [_raster(x, fd.shape, t) for x in (current_outflow, inflow, alpha, beta)]
    pd, sd, kd = _raster(channel_length, fd.shape, t)
    out = np.empty(fd.shape, dtype)
    flat = []
    for p, s, _ in args:
        flat += [p, s]
    _check(getattr(lib(), f"lue_oracle_kinematic_wave_{_sfx(dtype)}")(
        fd.ctypes.data, fd.shape[0], fd.shape[1], pr, pc, *flat, t(time_step_duration), pd, sd,
        out.ctypes.data, nthreads))
    del args, kd
    return out


def iterate_to_new_discharge(upstream, current, lateral, alpha, beta, dt, dx, dtype=np.float64):
    f = (lib().lue_oracle_iterate_to_new_discharge_f64 if np.dtype(dtype) == np.float64
         else lib().lue_oracle_iterate_to_new_discharge_f32)
    return f(upstream, current, lateral, alpha, beta, dt, dx)
