"""Batched ensembles: many kinematic-wave instances (catchment x scenario) in one launch per time step.

Every (catchment, scenario) instance is placed in one "atlas" raster, separated from its neighbours by a
one-cell border of no-data flow direction (255).  Flow never crosses that border: a cell whose flow
leaves its catchment now drains into a no-data cell, which ends the path exactly as leaving the array
does (no cell downstream waits for a no-data cell, and its own output is NaN).  So each instance's
result in the atlas is the result it gets alone, and one topology plus one kinematic_wave launch per
time step covers the whole ensemble.  The time steps are captured into one CUDA graph.

The unbatched form (one topology and one launch per instance and step) is timed on a sample of the
instances for comparison.
"""
import concurrent.futures as cf
import math
import os
import time

import numpy as np

from . import synthetic

BORDER = 1


def catchment_sides(n, lo, hi, seed):
    """Square catchment sides drawn log-uniformly from [lo, hi] (rounded to multiples of 8)."""
    rng = np.random.default_rng(seed)
    sides = np.exp(rng.uniform(math.log(lo), math.log(hi), n))
    return [int(max(8, round(s / 8) * 8)) for s in sides]


def build_flow_directions(sides, seed, amplitude=200.0, threads=None):
    """Seeded, depression-filled D8 grids (the same terrain pipeline as the single-raster workloads),
    built in parallel: the C generator releases the GIL."""
    threads = threads or min(os.cpu_count() or 1, 32)

    def one(i):
        s = sides[i]
        return synthetic.cached_flow_direction(s, s, seed * 10007 + i, amplitude)

    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        return list(ex.map(one, range(len(sides))))


class Atlas:
    """Shelf packing of rectangles into one raster of width `width`, each with a one-cell border."""

    def __init__(self, shapes, width=None):
        self.shapes = [tuple(s) for s in shapes]
        padded = [(h + 2 * BORDER, w + 2 * BORDER) for h, w in self.shapes]
        width = width or max(max(w for _, w in padded), int(math.sqrt(sum(h * w for h, w in padded)) * 1.05))
        order = sorted(range(len(padded)), key=lambda i: -padded[i][0])
        self.offsets = [None] * len(padded)
        x = y = shelf_h = 0
        for i in order:
            h, w = padded[i]
            if x + w > width:
                y += shelf_h
                x = shelf_h = 0
            self.offsets[i] = (y + BORDER, x + BORDER)
            x += w
            shelf_h = max(shelf_h, h)
        self.shape = (y + shelf_h, width)

    @property
    def cells(self):
        return sum(h * w for h, w in self.shapes)

    def pack(self, arrays, fill, dtype, device=None):
        import torch
        out = torch.full(self.shape, fill, dtype=dtype, device=device)
        for (r, c), a in zip(self.offsets, arrays):
            t = torch.as_tensor(a) if not isinstance(a, torch.Tensor) else a
            out[r:r + t.shape[0], c:c + t.shape[1]] = t.to(device=out.device, dtype=dtype)
        return out

    def view(self, atlas_array, i):
        r, c = self.offsets[i]
        h, w = self.shapes[i]
        return atlas_array[r:r + h, c:c + w]


def ensemble_inputs(n_catchments=64, scenarios=4, lo=512, hi=4096, seed=11, device="cuda"):
    """64 catchments (sides log-uniform in [512, 4096]) x 4 rain scenarios (multiplier U[0.5, 2])."""
    import torch
    sides = catchment_sides(n_catchments, lo, hi, seed)
    fds = build_flow_directions(sides, seed)
    rng = np.random.default_rng(seed + 1)
    inst = []
    for ci, (s, fd) in enumerate(zip(sides, fds)):
        base_rain = synthetic.rain_blobs(s, s, np.random.default_rng(seed * 31 + ci), n_blobs=6)
        alpha = (1.0 + 4.0 * np.random.default_rng(seed * 37 + ci).random((s, s), dtype=np.float32)).astype(np.float32)
        for k in range(scenarios):
            mult = np.float32(rng.uniform(0.5, 2.0))
            inst.append(dict(catchment=ci, scenario=k, flow_direction=fd, lateral=base_rain * mult, alpha=alpha,
                             q0_seed=int(rng.integers(1 << 31))))
    return inst


def run_batched(inst, steps, device="cuda", graph=True, partition=(1024, 1024), waves=False, autotune_steps=0):
    """All instances in one atlas.  waves=False: one kinematic_wave launch per step, the steps captured
    in one CUDA graph (graph=True) or launched in a loop; waves=True: all steps in one
    kinematic_wave_steps call (the stage engine's pipelined steps).  autotune_steps > 0 (waves=True):
    first autotune the stage schedule of the atlas on a call of that many steps, then time `steps`.
    Returns (seconds for `steps` steps, atlas, final discharge atlas tensor, topology stats); with
    autotune_steps, the stats carry the schedule (`stage_schedule`) and the tuning time (`tuning_s`)."""
    import torch

    from . import framework as lfr
    atlas = Atlas([i["flow_direction"].shape for i in inst])
    fd = atlas.pack([i["flow_direction"] for i in inst], 255, torch.uint8, device)
    lat = atlas.pack([i["lateral"] for i in inst], 0.0, torch.float32, device)
    alpha = atlas.pack([i["alpha"] for i in inst], 1.0, torch.float32, device)
    q0 = atlas.pack([torch.from_numpy(np.random.default_rng(i["q0_seed"]).random(i["flow_direction"].shape))
                     for i in inst], 0.0, torch.float64, device)
    ps = (min(partition[0], atlas.shape[0]), min(partition[1], atlas.shape[1]))
    fdA = lfr.PartitionedArray(fd, ps)
    latA, alphaA = lfr.PartitionedArray(lat, ps), lfr.PartitionedArray(alpha, ps)
    topo = fdA.topology()
    bufs = [lfr.PartitionedArray(q0.clone(), ps), lfr.PartitionedArray(torch.empty_like(q0), ps)]

    def step_into(src, dst):
        from . import _lib
        L = _lib.lib()
        stream = torch.cuda.current_stream(fd.device).cuda_stream
        _lib.check(L.lue_gpu_kinematic_wave_f64_f32in(topo.handle, src.data.data_ptr(), 0.0, lat.data_ptr(), 0.0,
                                                      alpha.data_ptr(), 0.0, 0.6, 3600.0, 100.0, dst.data.data_ptr(),
                                                      stream))

    torch.cuda.synchronize()
    if waves:
        from . import _lib
        L = _lib.lib()
        out = torch.empty_like(q0)
        stream = torch.cuda.current_stream(fd.device)
        # first call builds the level order and the history planes (not timed)
        _lib.check(L.lue_gpu_kinematic_wave_steps_f64_f32in(topo.handle, q0.data_ptr(), lat.data_ptr(), 0.0,
                                                            alpha.data_ptr(), 0.0, 0.6, 3600.0, 100.0, steps,
                                                            out.data_ptr(), stream.cuda_stream))
        torch.cuda.synchronize()
        stats = topo.stats()
        if autotune_steps > 0:
            def short_call():
                _lib.check(L.lue_gpu_kinematic_wave_steps_f64_f32in(
                    topo.handle, q0.data_ptr(), lat.data_ptr(), 0.0, alpha.data_ptr(), 0.0, 0.6, 3600.0, 100.0,
                    autotune_steps, out.data_ptr(), stream.cuda_stream))
            t0 = time.perf_counter()
            best = lfr.autotune_stage_schedule(fdA, short_call)
            stats["tuning_s"] = round(time.perf_counter() - t0, 2)
            stats["stage_schedule"] = {k: best[k] for k in ("cap", "threads", "publish_every")}
            # the full call once with the chosen schedule (a new cap rebuilds the stages and the history)
            _lib.check(L.lue_gpu_kinematic_wave_steps_f64_f32in(topo.handle, q0.data_ptr(), lat.data_ptr(), 0.0,
                                                                alpha.data_ptr(), 0.0, 0.6, 3600.0, 100.0, steps,
                                                                out.data_ptr(), stream.cuda_stream))
            torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        _lib.check(L.lue_gpu_kinematic_wave_steps_f64_f32in(topo.handle, q0.data_ptr(), lat.data_ptr(), 0.0,
                                                            alpha.data_ptr(), 0.0, 0.6, 3600.0, 100.0, steps,
                                                            out.data_ptr(), stream.cuda_stream))
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1000.0, atlas, out, stats
    if graph:
        s = torch.cuda.Stream(device)
        s.wait_stream(torch.cuda.current_stream(device))
        with torch.cuda.stream(s):
            step_into(bufs[0], bufs[1])  # warm-up outside capture
        torch.cuda.current_stream(device).wait_stream(s)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        bufs[0].data.copy_(q0)
        with torch.cuda.graph(g):
            for t in range(steps):
                step_into(bufs[t % 2], bufs[(t + 1) % 2])
        bufs[0].data.copy_(q0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        g.replay()
        e1.record()
        torch.cuda.synchronize()
        secs = e0.elapsed_time(e1) / 1000.0
    else:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for t in range(steps):
            step_into(bufs[t % 2], bufs[(t + 1) % 2])
        e1.record()
        torch.cuda.synchronize()
        secs = e0.elapsed_time(e1) / 1000.0
    return secs, atlas, bufs[steps % 2].data, topo.stats()


def run_unbatched(inst, steps, sample, device="cuda"):
    """One topology and one kinematic_wave launch per instance and step, on `sample` instances.
    Returns (seconds, cells of the sample, final discharges of the sample)."""
    import torch

    from . import framework as lfr
    results, cells = [], 0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for i in inst[:sample]:
        fd = lfr.from_numpy(i["flow_direction"], device=device)
        q = lfr.from_numpy(np.random.default_rng(i["q0_seed"]).random(i["flow_direction"].shape), device=device)
        lat, alpha = lfr.from_numpy(i["lateral"], device=device), lfr.from_numpy(i["alpha"], device=device)
        for _ in range(steps):
            q = lfr.kinematic_wave(fd, q, lat, alpha, 0.6, 3600.0, 100.0)
        results.append(q.data)
        cells += i["flow_direction"].size
    torch.cuda.synchronize()
    return time.perf_counter() - t0, cells, results


def run_plain_resident(inst, steps, device="cuda"):
    """The plain drop-in at its best, for comparison with the atlas: one resident topology per catchment
    (built before the timed region and shared by its scenarios), device-resident inputs, and one
    kinematic_wave_steps call per instance (all `steps` steps in that call), timed with CUDA events on
    the launching stream.  Returns (seconds, cells, final discharges by instance)."""
    import torch

    from . import _lib
    from . import framework as lfr
    L = _lib.lib()
    fds, prepared = {}, []
    for i in inst:
        c = i["catchment"]
        if c not in fds:
            fds[c] = lfr.from_numpy(i["flow_direction"], device=device)
            fds[c].topology()
        q0 = torch.from_numpy(np.random.default_rng(i["q0_seed"]).random(i["flow_direction"].shape)).to(device)
        lat = torch.from_numpy(i["lateral"]).to(device)
        alpha = torch.from_numpy(i["alpha"]).to(device)
        prepared.append((fds[c].topology(), q0, lat, alpha, torch.empty_like(q0)))
    stream = torch.cuda.current_stream(torch.device(device))

    def call(p):
        topo, q0, lat, alpha, out = p
        _lib.check(L.lue_gpu_kinematic_wave_steps_f64_f32in(topo.handle, q0.data_ptr(), lat.data_ptr(), 0.0,
                                                            alpha.data_ptr(), 0.0, 0.6, 3600.0, 100.0, steps,
                                                            out.data_ptr(), stream.cuda_stream))

    for p in prepared:  # first calls build each topology's stages and history (not timed)
        call(p)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for p in prepared:
        call(p)
    e1.record(stream)
    torch.cuda.synchronize()
    cells = sum(i["flow_direction"].size for i in inst)
    return e0.elapsed_time(e1) / 1000.0, cells, [p[4] for p in prepared]
