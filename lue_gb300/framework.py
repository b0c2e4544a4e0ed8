"""Python mirror of LUE's routing operations (``lue.framework``) on the GB300 C ABI.

Same operation names, argument names and order, and the same raster-or-scalar overloads as the
reference's pybind11 module (source/framework/python/source/algorithm/routing_operation/{accu,
accu_threshold,accu_fraction,kinematic_wave,inflow_count}.cpp).  ``from_numpy`` / ``to_numpy`` mirror
source/framework/python/source/numpy/{from_numpy,to_numpy}.cpp.  Device memory is held in torch
CUDA tensors; every operation runs the CUDA kernels of liblue_gb300.so on torch's current stream.

The flow topology of a flow-direction array is built on first use and kept with that array, so
repeated calls (for example one kinematic_wave call per time step) do not redo it.
"""
import ctypes

import numpy as np
import torch

from . import _lib

FLOW_DIRECTION_NO_DATA = 255


class PartitionedArray:
    """A 2-D raster resident on the GPU, with the reference's partition shape kept for parity."""

    def __init__(self, data, partition_shape=None):
        if not isinstance(data, torch.Tensor) or not data.is_cuda:
            raise TypeError("PartitionedArray data must be a CUDA tensor")
        if data.dim() != 2:
            raise ValueError("PartitionedArray must be 2-D")
        self.data = data.contiguous()
        shape = tuple(self.data.shape)
        ps = tuple(int(v) for v in (partition_shape or shape))
        if len(ps) != 2 or ps[0] <= 0 or ps[1] <= 0:
            raise ValueError("Partition shape must not be empty")
        if ps[0] > shape[0] or ps[1] > shape[1]:
            raise ValueError("Partition size must be smaller than or equal to array size")
        self.partition_shape = ps
        self._topology = None

    @property
    def shape(self):
        return tuple(self.data.shape)

    @property
    def dtype(self):
        return self.data.dtype

    @property
    def shape_in_partitions(self):
        return (self.shape[0] // self.partition_shape[0], self.shape[1] // self.partition_shape[1])

    def topology(self):
        if self._topology is None:
            if self.dtype != torch.uint8:
                raise TypeError("flow direction must be uint8")
            self._topology = Topology(self.data, self.partition_shape)
        return self._topology


class Topology:
    """Owner of a lue_gpu_topology handle (resident inflow counts, upstream masks, levels, scratch)."""

    def __init__(self, flow_direction, partition_shape):
        L = _lib.lib()
        h = ctypes.c_void_p()
        fd = flow_direction.contiguous()
        stream = torch.cuda.current_stream(fd.device).cuda_stream
        _lib.check(L.lue_gpu_topology_create(fd.data_ptr(), fd.shape[0], fd.shape[1], partition_shape[0],
                                             partition_shape[1], stream, ctypes.byref(h)))
        self.handle = h
        self.shape = tuple(fd.shape)
        self.device = fd.device

    @classmethod
    def _from_handle(cls, handle, shape, device):
        t = cls.__new__(cls)
        t.handle, t.shape, t.device = handle, shape, device
        return t

    def clone(self):
        """Another handle on the same flow topology, with its own scratch (for concurrent calls)."""
        h = ctypes.c_void_p()
        _lib.check(_lib.lib().lue_gpu_topology_clone(self.handle, ctypes.byref(h)))
        return Topology._from_handle(h, self.shape, self.device)

    def prepare(self):
        """Builds the structures that the first call of a stage-engine operation (accu_threshold,
        accu_fraction, accu_capacity, accu_trigger, float64 accu, kinematic_wave) would build."""
        import torch
        _lib.check(_lib.lib().lue_gpu_topology_prepare(self.handle,
                                                       torch.cuda.current_stream(self.device).cuda_stream))

    def stage_schedule(self):
        """The stage engine's schedule for this handle: {cap, threads, publish_every} (threads 0: by the
        largest stage)."""
        s = _lib.StageSchedule()
        _lib.check(_lib.lib().lue_gpu_topology_get_stage_schedule(self.handle, ctypes.byref(s)))
        d = s.as_dict()
        del d["ms"]
        return d

    def set_stage_schedule(self, cap=0, threads=0, publish_every=0):
        """Sets the stage engine's schedule (0 keeps the cap / picks threads by stage size / default
        publication interval).  Results do not depend on it.  Another cap is refused while clones share
        the stage structures."""
        s = _lib.StageSchedule(int(cap), int(threads), int(publish_every), 0.0)
        _lib.check(_lib.lib().lue_gpu_topology_set_stage_schedule(self.handle, ctypes.byref(s)))

    STAGE_ORDERS = {"latest": 0, "earliest": 1}

    def stage_order(self):
        """The order in which a stage-engine call's CTAs take the stages: "latest" (least slack first, the
        fastest for one call alone on the GPU) or "earliest" (about the order in which inputs become
        ready: fewer waiting CTAs when many calls run at once)."""
        o = ctypes.c_int()
        _lib.check(_lib.lib().lue_gpu_topology_get_stage_order(self.handle, ctypes.byref(o)))
        return {v: k for k, v in self.STAGE_ORDERS.items()}[o.value]

    def set_stage_order(self, order):
        """Sets the stage order ("latest" or "earliest"); results do not depend on it.  Like another cap,
        another order frees the stage structures (rebuilt by the next call) and is refused while clones
        share them."""
        if order not in self.STAGE_ORDERS:
            raise ValueError(f"stage order must be one of {sorted(self.STAGE_ORDERS)}")
        _lib.check(_lib.lib().lue_gpu_topology_set_stage_order(self.handle, self.STAGE_ORDERS[order]))

    def stats(self):
        s = _lib.TopologyStats()
        _lib.check(_lib.lib().lue_gpu_topology_get_stats(self.handle, ctypes.byref(s)))
        return s.as_dict()

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            _lib.lib().lue_gpu_topology_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_ELEMENT_TYPES = {np.dtype(np.uint8): 1, np.dtype(np.int32): 2, np.dtype(np.uint32): 3, np.dtype(np.int64): 4,
                  np.dtype(np.uint64): 5, np.dtype(np.float32): 6, np.dtype(np.float64): 7}
_TORCH_DTYPES = {np.dtype(np.uint8): torch.uint8, np.dtype(np.int32): torch.int32, np.dtype(np.int64): torch.int64,
                 np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64}


def _element_type(dtype):
    try:
        return _ELEMENT_TYPES[np.dtype(dtype)]
    except KeyError:
        raise TypeError(f"element type {np.dtype(dtype)} is not one of LUE's") from None


def pinned_empty(shape, dtype):
    """An uninitialised numpy array in pinned (page-locked) host memory.  from_numpy reads such an array,
    and to_numpy / to_numpy_async write one, with asynchronous copies and no staging copy."""
    return torch.empty(tuple(shape), dtype=_TORCH_DTYPES[np.dtype(dtype)], pin_memory=True).numpy()


def _host_tensor(a):
    t = torch.from_numpy(a)
    return t, t.is_pinned()


def from_numpy(array, partition_shape=None, no_data_value=None, device="cuda"):
    """lue.framework.from_numpy (source/framework/python/source/numpy/from_numpy.cpp:44-133): a 2-D
    numpy array to a PartitionedArray on the GPU; elements equal to ``no_data_value`` become the element
    type's no-data value (NaN for floats, the minimum for signed and the maximum for unsigned integers).

    The copy runs on torch's current stream and the call returns before it completes: an array in pinned
    memory (pinned_empty) is copied directly, and must not be changed until the stream has passed the
    copy; any other array is first copied into pinned memory from torch's host allocator, which keeps
    that memory until the copy is done.  The no-data mapping runs on the device, on the same stream."""
    a = np.ascontiguousarray(array)
    if a.ndim != 2:
        raise RuntimeError("Currently only arrays of rank 2 are supported")
    et = _element_type(a.dtype)
    host, pinned = _host_tensor(a)
    if not pinned:
        host = host.pin_memory()
    dev = torch.empty(a.shape, dtype=host.dtype, device=device)
    dev.copy_(host, non_blocking=True)
    if no_data_value is not None:
        v = np.array(no_data_value, dtype=a.dtype)
        _lib.check(_lib.lib().lue_gpu_mark_no_data(dev.data_ptr(), dev.numel(), et, v.ctypes.data, _stream(dev)))
    return PartitionedArray(dev, partition_shape)


def to_numpy_async(array, out, no_data_value=None):
    """Starts the copy of a PartitionedArray into ``out`` (a numpy array of the same shape and element
    type, in pinned memory: pinned_empty) on torch's current stream; no-data elements come out as
    ``no_data_value`` when it is given (mapped on the device).  Returns a torch.cuda.Event that has
    completed once ``out`` holds the result."""
    d = array.data
    if tuple(out.shape) != tuple(d.shape) or _TORCH_DTYPES.get(np.dtype(out.dtype)) != d.dtype:
        raise ValueError("to_numpy: out must have the array's shape and element type")
    host, pinned = _host_tensor(out)
    if not pinned:
        raise ValueError("to_numpy_async: out must be in pinned memory (pinned_empty)")
    src = d
    if no_data_value is not None:
        src = torch.empty_like(d)
        v = np.array(no_data_value, dtype=out.dtype)
        _lib.check(_lib.lib().lue_gpu_replace_no_data(d.data_ptr(), src.data_ptr(), d.numel(),
                                                      _element_type(out.dtype), v.ctypes.data, _stream(d)))
    host.copy_(src, non_blocking=True)
    ev = torch.cuda.Event()
    ev.record(torch.cuda.current_stream(d.device))
    return ev


def to_numpy(array, no_data_value=None, out=None):
    """lue.framework.to_numpy (source/framework/python/source/numpy/to_numpy.cpp): the array as a numpy
    array (into ``out`` when given), no-data elements as ``no_data_value`` when it is given.  The copy
    goes to pinned memory on torch's current stream; the call returns once it is complete."""
    d = array.data
    if out is None:
        out = pinned_empty(d.shape, _numpy_dtype(d.dtype))
    if _host_tensor(out)[1]:
        to_numpy_async(array, out, no_data_value).synchronize()
        return out
    tmp = to_numpy(array, no_data_value)  # pageable out: through a pinned buffer
    np.copyto(out, tmp)
    return out


def _numpy_dtype(torch_dtype):
    for k, v in _TORCH_DTYPES.items():
        if v == torch_dtype:
            return k
    raise TypeError(f"element type {torch_dtype} is not one of LUE's")


def _stream(t):
    return torch.cuda.current_stream(t.device).cuda_stream


def _raster_or_scalar(x, shape, dtype, name):
    """(device pointer or None, scalar, keep-alive tensor) for an argument of the reference's
    PartitionedArray | Scalar | value overloads."""
    if isinstance(x, PartitionedArray):
        if x.shape != shape:
            raise _lib.LueGpuError(2, f"{name}: shape {x.shape} differs from flow direction shape {shape}")
        t = x.data if x.data.dtype == dtype else x.data.to(dtype)
        return t.data_ptr(), 0.0, t
    if isinstance(x, torch.Tensor):
        if x.dim() == 0:
            return None, float(x), None
        return _raster_or_scalar(PartitionedArray(x), shape, dtype, name)
    return None, float(x), None


def _check_partitioning(flow_direction, *arrays):
    for a in arrays:
        if isinstance(a, PartitionedArray) and a.shape_in_partitions != flow_direction.shape_in_partitions:
            raise _lib.LueGpuError(2, "arrays are not partitioned in the same way")


def _material_dtype(*args):
    """Element type of the operation: that of the first float raster, else of a numpy float64 scalar,
    else float32 (the reference binds the float overload first)."""
    for a in args:
        if isinstance(a, PartitionedArray) and a.dtype in (torch.float32, torch.float64):
            return a.dtype
    for a in args:
        if isinstance(a, np.float64) or (isinstance(a, torch.Tensor) and a.dtype == torch.float64):
            return torch.float64
    return torch.float32


def _empty(flow_direction, dtype):
    return torch.empty(flow_direction.shape, dtype=dtype, device=flow_direction.data.device)


def d8_flow_direction(elevation):
    """value_policies::d8_flow_direction (uint8 D8 codes) from a float32 or float64 elevation array."""
    if elevation.dtype not in (torch.float32, torch.float64):
        raise TypeError("elevation must be float32 or float64")
    out = _empty(elevation, torch.uint8)
    L = _lib.lib()
    fn = L.lue_gpu_d8_flow_direction_f32 if elevation.dtype == torch.float32 else L.lue_gpu_d8_flow_direction_f64
    _lib.check(fn(elevation.data.data_ptr(), elevation.shape[0], elevation.shape[1], out.data_ptr(),
                  _stream(elevation.data)))
    return PartitionedArray(out, elevation.partition_shape)


def inflow_count(flow_direction, value_policies=True):
    t = flow_direction.topology()
    out = _empty(flow_direction, torch.uint8)
    _lib.check(_lib.lib().lue_gpu_inflow_count_u8(t.handle, int(value_policies), out.data_ptr(),
                                                  _stream(flow_direction.data)))
    return PartitionedArray(out, flow_direction.partition_shape)


def accu_info(flow_direction):
    """value_policies::accu_info: the class of every cell in the reference's partitioned flow accumulation
    (uint8: 11 ridge, 12 intra-partition stream, 13 partition output, 14 partition input, 15 partition
    input-output, 16 inter-partition stream, 17 sink, 255 no-data) for the array's partition shape."""
    t = flow_direction.topology()
    out = _empty(flow_direction, torch.uint8)
    _lib.check(_lib.lib().lue_gpu_accu_info_u8(t.handle, out.data_ptr(), _stream(flow_direction.data)))
    return PartitionedArray(out, flow_direction.partition_shape)


def partial_accu(flow_direction, inflow, nr_steps, order_dependent=False):
    """value_policies::partial_accu(flow_direction, inflow, nr_steps): per cell the number of the stream of
    the partitioned walk that reached it last, NaN above nr_steps (float32 for a float or numpy.float32
    inflow scalar, float64 for numpy.float64; the reference does not use the inflow's value).  With
    order_dependent=True also returns a uint8 array that is 1 where the reference's result depends on
    the order in which its inter-partition messages are delivered."""
    if isinstance(inflow, PartitionedArray):
        raise TypeError("partial_accu: inflow must be a scalar")
    dtype = torch.float64 if isinstance(inflow, np.float64) else torch.float32
    t = flow_direction.topology()
    out = _empty(flow_direction, dtype)
    od = _empty(flow_direction, torch.uint8) if order_dependent else None
    fn = _lib.lib().lue_gpu_partial_accu_f64 if dtype == torch.float64 else _lib.lib().lue_gpu_partial_accu_f32
    _lib.check(fn(t.handle, int(nr_steps), out.data_ptr(), None if od is None else od.data_ptr(),
                  _stream(flow_direction.data)))
    res = PartitionedArray(out, flow_direction.partition_shape)
    return (res, PartitionedArray(od, flow_direction.partition_shape)) if order_dependent else res


def downstream_level(flow_direction):
    t = flow_direction.topology()
    out = _empty(flow_direction, torch.int32)
    _lib.check(_lib.lib().lue_gpu_downstream_level_i32(t.handle, out.data_ptr(), _stream(flow_direction.data)))
    return PartitionedArray(out, flow_direction.partition_shape)


def accu(flow_direction, inflow):
    _check_partitioning(flow_direction, inflow)
    dtype = _material_dtype(inflow)
    t = flow_direction.topology()
    p, s, keep = _raster_or_scalar(inflow, flow_direction.shape, dtype, "inflow")
    out = _empty(flow_direction, dtype)
    fn = _lib.lib().lue_gpu_accu_f32 if dtype == torch.float32 else _lib.lib().lue_gpu_accu_f64
    _lib.check(fn(t.handle, p, s, out.data_ptr(), _stream(flow_direction.data)))
    del keep
    return PartitionedArray(out, flow_direction.partition_shape)


def _two_output(fn32, fn64, flow_direction, inflow, other, name):
    _check_partitioning(flow_direction, inflow, other)
    dtype = _material_dtype(inflow, other)
    t = flow_direction.topology()
    p0, s0, k0 = _raster_or_scalar(inflow, flow_direction.shape, dtype, "inflow")
    p1, s1, k1 = _raster_or_scalar(other, flow_direction.shape, dtype, name)
    flux, state = _empty(flow_direction, dtype), _empty(flow_direction, dtype)
    fn = fn32 if dtype == torch.float32 else fn64
    _lib.check(fn(t.handle, p0, s0, p1, s1, flux.data_ptr(), state.data_ptr(), _stream(flow_direction.data)))
    del k0, k1
    ps = flow_direction.partition_shape
    return PartitionedArray(flux, ps), PartitionedArray(state, ps)


def accu_threshold(flow_direction, inflow, threshold):
    L = _lib.lib()
    return _two_output(L.lue_gpu_accu_threshold_f32, L.lue_gpu_accu_threshold_f64, flow_direction, inflow,
                       threshold, "threshold")


def accu_fraction(flow_direction, inflow, fraction):
    L = _lib.lib()
    return _two_output(L.lue_gpu_accu_fraction_f32, L.lue_gpu_accu_fraction_f64, flow_direction, inflow,
                       fraction, "fraction")


def accu_capacity(flow_direction, inflow, capacity):
    """value_policies::accu_capacity: (outflow, remainder); what flows on is capped at the capacity."""
    L = _lib.lib()
    return _two_output(L.lue_gpu_accu_capacity_f32, L.lue_gpu_accu_capacity_f64, flow_direction, inflow, capacity,
                       "capacity")


def accu_trigger(flow_direction, inflow, trigger):
    """value_policies::accu_trigger: (outflow, remainder); the total flows on once it reaches the trigger."""
    L = _lib.lib()
    return _two_output(L.lue_gpu_accu_trigger_f32, L.lue_gpu_accu_trigger_f64, flow_direction, inflow, trigger,
                       "trigger")


def _one_hop(fn32, fn64, flow_direction, material, name):
    if not isinstance(material, PartitionedArray):
        raise TypeError(f"{name}: material must be a PartitionedArray")
    if material.shape != flow_direction.shape:
        raise _lib.LueGpuError(2, f"{name}: shape {material.shape} differs from flow direction shape "
                                  f"{flow_direction.shape}")
    _check_partitioning(flow_direction, material)
    if material.dtype not in (torch.float32, torch.float64):
        raise TypeError(f"{name}: material must be float32 or float64")
    out = _empty(flow_direction, material.dtype)
    fn = fn32 if material.dtype == torch.float32 else fn64
    fd = flow_direction.data
    _lib.check(fn(fd.data_ptr(), fd.shape[0], fd.shape[1], material.data.data_ptr(), out.data_ptr(), _stream(fd)))
    return PartitionedArray(out, flow_direction.partition_shape)


def upstream(flow_direction, material):
    """value_policies::upstream: per cell the sum of the material of the neighbours draining into it."""
    L = _lib.lib()
    return _one_hop(L.lue_gpu_upstream_f32, L.lue_gpu_upstream_f64, flow_direction, material, "upstream")


def downstream(flow_direction, material):
    """value_policies::downstream: per cell the material of its downstream cell."""
    L = _lib.lib()
    return _one_hop(L.lue_gpu_downstream_f32, L.lue_gpu_downstream_f64, flow_direction, material, "downstream")


def downstream_distance(flow_direction, cell_size, dtype=torch.float32):
    """downstream_distance: the length of each cell's step to its downstream cell."""
    if dtype not in (torch.float32, torch.float64):
        raise TypeError("downstream_distance: dtype must be float32 or float64")
    out = _empty(flow_direction, dtype)
    L = _lib.lib()
    fn = L.lue_gpu_downstream_distance_f32 if dtype == torch.float32 else L.lue_gpu_downstream_distance_f64
    fd = flow_direction.data
    _lib.check(fn(fd.data_ptr(), fd.shape[0], fd.shape[1], float(cell_size), out.data_ptr(), _stream(fd)))
    return PartitionedArray(out, flow_direction.partition_shape)


def kinematic_wave(flow_direction, current_outflow, inflow, alpha, beta, time_step_duration, channel_length):
    """One time step.  A float32 current outflow raster (or a numpy.float32 scalar one) selects the
    reference's float instantiation: every input as float32, float32 discharge out.  Otherwise the
    discharge is float64; float32 inflow/alpha rasters with scalar beta and channel length then take the
    mixed-precision entry point (exact float32 -> float64 promotion per cell)."""
    _check_partitioning(flow_direction, current_outflow, inflow, alpha, beta, channel_length)
    t = flow_direction.topology()
    shape = flow_direction.shape
    if ((isinstance(current_outflow, PartitionedArray) and current_outflow.dtype == torch.float32) or
            isinstance(current_outflow, np.float32)):
        out = _empty(flow_direction, torch.float32)
        args = [_raster_or_scalar(x, shape, torch.float32, name) for x, name in (
            (current_outflow, "current_outflow"), (inflow, "inflow"), (alpha, "alpha"), (beta, "beta"),
            (channel_length, "channel_length"))]
        (pq, sq, _), (pl, sl, _), (pa, sa, _), (pb, sb, _), (pd, sd, _) = args
        _lib.check(_lib.lib().lue_gpu_kinematic_wave_f32(t.handle, pq, sq, pl, sl, pa, sa, pb, sb,
                                                         float(time_step_duration), pd, sd, out.data_ptr(),
                                                         _stream(flow_direction.data)))
        del args
        return PartitionedArray(out, flow_direction.partition_shape)
    out = _empty(flow_direction, torch.float64)
    L = _lib.lib()
    stream = _stream(flow_direction.data)
    f32_in = (isinstance(inflow, PartitionedArray) and inflow.dtype == torch.float32 and
              (not isinstance(alpha, PartitionedArray) or alpha.dtype == torch.float32) and
              not isinstance(beta, PartitionedArray) and not isinstance(channel_length, PartitionedArray))
    pq, sq, kq = _raster_or_scalar(current_outflow, shape, torch.float64, "current_outflow")
    if f32_in:
        pl, sl, kl = _raster_or_scalar(inflow, shape, torch.float32, "inflow")
        pa, sa, ka = _raster_or_scalar(alpha, shape, torch.float32, "alpha")
        _lib.check(L.lue_gpu_kinematic_wave_f64_f32in(t.handle, pq, sq, pl, sl, pa, sa, float(beta),
                                                      float(time_step_duration), float(channel_length),
                                                      out.data_ptr(), stream))
    else:
        pl, sl, kl = _raster_or_scalar(inflow, shape, torch.float64, "inflow")
        pa, sa, ka = _raster_or_scalar(alpha, shape, torch.float64, "alpha")
        pb, sb, kb = _raster_or_scalar(beta, shape, torch.float64, "beta")
        pd, sd, kd = _raster_or_scalar(channel_length, shape, torch.float64, "channel_length")
        _lib.check(L.lue_gpu_kinematic_wave_f64(t.handle, pq, sq, pl, sl, pa, sa, pb, sb,
                                                float(time_step_duration), pd, sd, out.data_ptr(), stream))
        del kb, kd
    del kq, kl, ka
    return PartitionedArray(out, flow_direction.partition_shape)


def kinematic_wave_steps(flow_direction, current_outflow, inflow, alpha, beta, time_step_duration, channel_length,
                         steps):
    """`steps` kinematic_wave time steps in one call (float64 discharge; float32 inflow and alpha rasters or
    scalars; scalar beta and channel length), equal to calling kinematic_wave `steps` times."""
    _check_partitioning(flow_direction, current_outflow, inflow, alpha)
    t = flow_direction.topology()
    shape = flow_direction.shape
    out = _empty(flow_direction, torch.float64)
    pq, sq, kq = _raster_or_scalar(current_outflow, shape, torch.float64, "current_outflow")
    if pq is None:
        kq = torch.full(shape, sq, dtype=torch.float64, device=flow_direction.data.device)
        pq = kq.data_ptr()
    pl, sl, kl = _raster_or_scalar(inflow, shape, torch.float32, "inflow")
    pa, sa, ka = _raster_or_scalar(alpha, shape, torch.float32, "alpha")
    _lib.check(_lib.lib().lue_gpu_kinematic_wave_steps_f64_f32in(
        t.handle, pq, pl, sl, pa, sa, float(beta), float(time_step_duration), float(channel_length), int(steps),
        out.data_ptr(), _stream(flow_direction.data)))
    del kq, kl, ka
    return PartitionedArray(out, flow_direction.partition_shape)


def autotune_stage_schedule(flow_direction, call, repeats=1):
    """Autotunes the stage engine's schedule of `flow_direction`'s topology for `call`, a callable without
    arguments that issues one routing call over `flow_direction` (for example
    ``lambda: accu_threshold(fd, material, threshold)``) on torch's current stream.  The native tuner
    (lue_gpu_autotune_stage_schedule) times it with CUDA events for candidate stage caps, publication
    intervals and CTA sizes, keeps the fastest schedule on the topology and returns it as
    {cap, threads, publish_every, ms}.  Results do not depend on the schedule."""
    t = flow_direction.topology()
    errors = []

    def trampoline(handle, user, stream):
        try:
            call()
            return 0
        except _lib.LueGpuError as e:
            errors.append(e)
            return e.status
        except Exception as e:  # noqa: BLE001  (re-raised below, after the native tuner returns)
            errors.append(e)
            return 1

    cb = _lib.STAGE_CALL(trampoline)
    best = _lib.StageSchedule()
    status = _lib.lib().lue_gpu_autotune_stage_schedule(t.handle, cb, None, int(repeats),
                                                        _stream(flow_direction.data), ctypes.byref(best))
    if errors and not isinstance(errors[0], _lib.LueGpuError):
        raise errors[0]
    _lib.check(status)
    return best.as_dict()
