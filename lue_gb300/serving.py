"""Serving: a request loop over a pool of resident flow topologies, with continuous batching.

Requests are accu (float32 material) and multi-step kinematic_wave (float64 discharge) solves on grids
from a pool whose flow topologies (inflow counts, downstream levels, tile structures) are built once and
stay on the device.  The loop:

- queues requests as they arrive (a Poisson stream in the benchmark);
- admits the oldest waiting request as soon as a slot (CUDA stream) is free and its device memory
  (inputs, outputs, per-request scratch) fits, so requests that arrive while others run start while
  those are still on the GPU, and their kernels overlap.  "Fits" is checked against two figures at
  every admission: the server's budget less the estimates of the admitted requests, and the HBM free
  right now (cudaMemGetInfo plus what torch's caching allocator holds unused) less a reserve.  A request
  whose estimate exceeds the whole budget is never admitted: it completes at once with an error;
- runs each request on its own stream with its own topology handle (a clone that shares the grid's
  resident topology and has its own scratch), copies the result back to pinned host memory, and
  completes it when its event has fired.

Latency is measured from arrival to completion on the host clock.  The same requests can be run one at
a time through the plain drop-in path (topology built per call, as the reference recomputes inflow
counts on every call) for comparison, or alone to check that results do not depend on the mix.
"""
import collections
import time
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Request:
    rid: int
    kind: str                 # "accu" or "kinematic_wave"
    grid: int
    arrival: float            # seconds after the start of the run
    steps: int = 1
    inputs: dict = field(default_factory=dict)
    result: object = None
    start: float = None
    done: float = None
    error: str = None

    @property
    def latency(self):
        return None if self.done is None else self.done - self.arrival


def make_requests(pool_shapes, rate, duration, kw_fraction=0.5, kw_steps=24, seed=0):
    """Poisson arrivals at `rate` per second for `duration` seconds; each request draws a grid uniformly
    from the pool and is a `kw_steps`-step kinematic_wave solve with probability `kw_fraction`, else an
    accu.  Each request carries a seed; its input fields are generated on the device from that seed when
    it is admitted (material lognormal(0, 1) float32; discharge U[0, 1) float64, lateral inflow U[0, 5e-5)
    m3/s/m float32, alpha U[1, 5) float32), so a request's inputs are the same alone and in any mix."""
    rng = np.random.default_rng(seed)
    reqs, t, rid = [], 0.0, 0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        g = int(rng.integers(len(pool_shapes)))
        kind = "kinematic_wave" if rng.random() < kw_fraction else "accu"
        steps = kw_steps if kind == "kinematic_wave" else 1
        reqs.append(Request(rid, kind, g, t, steps, dict(seed=int(rng.integers(1 << 62)))))
        rid += 1
    return reqs


def device_inputs(r, shape, device, stream=None):
    """The request's input fields, generated on `device` (on the current stream) from its seed."""
    import torch
    gen = torch.Generator(device=device)
    gen.manual_seed(r.inputs["seed"])
    if r.kind == "accu":
        m = torch.empty(shape, dtype=torch.float32, device=device)
        m.log_normal_(0.0, 1.0, generator=gen)
        return {"material": m}
    q = torch.rand(shape, dtype=torch.float64, device=device, generator=gen)
    lat = torch.rand(shape, dtype=torch.float32, device=device, generator=gen) * 5e-5
    al = 1.0 + 4.0 * torch.rand(shape, dtype=torch.float32, device=device, generator=gen)
    return {"discharge": q, "lateral": lat, "alpha": al}


class Server:
    RESERVE_BYTES = 256 << 20  # kept free for the stage buffers that grow inside a call

    def __init__(self, pool_fds, slots=8, hbm_fraction=0.5, device="cuda"):
        import torch

        from . import framework as lfr
        self.torch, self.lfr, self.device = torch, lfr, torch.device(device)
        self.grids = [lfr.from_numpy(fd, device=self.device) for fd in pool_fds]
        self.topologies = [g.topology() for g in self.grids]
        # everything a request would otherwise build or allocate on its first call: the stage
        # structures of each grid, one handle (scratch) per grid, and pinned result buffers.  Many
        # requests run at once, so the stage engine takes its stages in about the order in which their
        # inputs become ready (fewer CTAs waiting on others while other requests need the SMs).
        self.free_clones = collections.defaultdict(list)
        for g, t in enumerate(self.topologies):
            t.set_stage_order("earliest")
            t.prepare()
            self.free_clones[g].append(t.clone())
        self._warm_pinned(slots)
        self.streams = [torch.cuda.Stream(self.device) for _ in range(slots)]
        free, _ = torch.cuda.mem_get_info(self.device)
        self.budget = int(free * hbm_fraction)
        self.in_use = 0
        torch.cuda.synchronize(self.device)

    def _warm_pinned(self, slots):
        """Fills the pinned host allocator's cache (sizes rounded up to powers of two) with enough result
        buffers of each size class for the concurrent requests."""
        torch = self.torch
        sizes = set()
        for g in self.grids:
            n = int(np.prod(g.shape))
            for b in (4 * n, 8 * n):
                sizes.add(1 << (b - 1).bit_length())
        per_class = max(1, slots // 4)
        held = [torch.empty(s, dtype=torch.uint8, pin_memory=True) for s in sorted(sizes) for _ in range(per_class)]
        del held

    def free_bytes(self):
        """Device memory a new request can use now: free HBM plus torch's cached, unallocated blocks."""
        torch = self.torch
        free, _ = torch.cuda.mem_get_info(self.device)
        cached = torch.cuda.memory_reserved(self.device) - torch.cuda.memory_allocated(self.device)
        return free + max(0, cached)

    def admissible(self, r, busy):
        """None if request r may start now; else why not ("wait", or "never" when its estimate exceeds
        the whole budget).  With nothing running (busy False) a request within the budget starts."""
        need = self.bytes_needed(r)
        if need > self.budget:
            return "never"
        if busy and (self.in_use + need > self.budget or need > self.free_bytes() - self.RESERVE_BYTES):
            return "wait"
        return None

    def cells(self, r):
        return int(np.prod(self.grids[r.grid].shape))

    def bytes_needed(self, r):
        n = self.cells(r)
        if r.kind == "accu":
            return n * (4 + 4 + 16)            # material, outflow, scratch
        # discharge in/out, inputs, scratch, history planes (at most 64, see kinematic_wave_steps.cu)
        return n * (8 + 4 + 4 + 8 + 16 + 8 * min(max(r.steps - 1, 0), 64))

    def _topology(self, g):
        lst = self.free_clones[g]
        return lst.pop() if lst else self.topologies[g].clone()

    def _launch(self, r, stream, keep_results=True):
        torch = self.torch
        from . import _lib
        L = _lib.lib()
        fd = self.grids[r.grid]
        topo = self._topology(r.grid)
        with torch.cuda.stream(stream):
            x = device_inputs(r, fd.shape, self.device)
            if r.kind == "accu":
                out = torch.empty(fd.shape, dtype=torch.float32, device=self.device)
                _lib.check(L.lue_gpu_accu_f32(topo.handle, x["material"].data_ptr(), 0.0, out.data_ptr(),
                                              stream.cuda_stream))
            else:
                out = torch.empty(fd.shape, dtype=torch.float64, device=self.device)
                _lib.check(L.lue_gpu_kinematic_wave_steps_f64_f32in(
                    topo.handle, x["discharge"].data_ptr(), x["lateral"].data_ptr(), 0.0, x["alpha"].data_ptr(), 0.0,
                    0.6, 3600.0, 100.0, r.steps, out.data_ptr(), stream.cuda_stream))
            # the result goes back to host memory: part of every request's latency
            host = torch.empty(out.shape, dtype=out.dtype, pin_memory=True)
            host.copy_(out, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(stream)
        return dict(req=r, topo=topo, event=ev, host=host, keep=(x, out), stream=stream)

    def run(self, requests, realtime=True, keep_results=True):
        """Serve `requests` (sorted by arrival).  With realtime=False every request is available at
        time zero (a closed-loop stress run).  Returns the summary dict."""
        torch = self.torch
        pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
        waiting, active = collections.deque(), []
        free_streams = list(self.streams)
        t0 = time.perf_counter()
        done = 0
        self.max_active = 0
        while done < len(requests):
            now = time.perf_counter() - t0
            while pending and (not realtime or pending[0].arrival <= now):
                waiting.append(pending.popleft())
            still = []
            for a in active:
                if a["event"].query():
                    r = a["req"]
                    r.done = time.perf_counter() - t0
                    if keep_results:
                        r.result = a["host"].numpy()
                    self.free_clones[r.grid].append(a["topo"])
                    self.in_use -= self.bytes_needed(r)
                    free_streams.append(a["stream"])
                    done += 1
                else:
                    still.append(a)
            active = still
            while waiting and free_streams:
                r = waiting[0]
                why = self.admissible(r, bool(active))
                if why == "never":  # larger than the whole budget: completes at once, with an error
                    waiting.popleft()
                    r.start = r.done = time.perf_counter() - t0
                    r.error = "request needs more device memory than the server's budget"
                    done += 1
                    continue
                if why == "wait":
                    break  # admission by free HBM: wait for running requests to finish
                waiting.popleft()
                self.in_use += self.bytes_needed(r)
                r.start = time.perf_counter() - t0
                active.append(self._launch(r, free_streams.pop(), keep_results))
                self.max_active = max(self.max_active, len(active))
            if not active and not waiting and pending and realtime:
                time.sleep(max(0.0, min(pending[0].arrival - (time.perf_counter() - t0), 0.001)))
            else:
                time.sleep(0.0001)
        wall = time.perf_counter() - t0
        torch.cuda.synchronize(self.device)
        return summarize(requests, wall, self)


def summarize(requests, wall, server):
    served = [r for r in requests if r.error is None]
    lat = np.array([r.latency for r in served]) if served else np.zeros(1)
    cell_steps = sum(int(np.prod(server.grids[r.grid].shape)) * r.steps for r in served)
    return {"requests": len(requests), "rejected": len(requests) - len(served),
            "max_concurrent": getattr(server, "max_active", 1),
            "p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_ms": float(lat.mean() * 1e3),
            "wall_s": wall, "mcells_per_s": cell_steps / wall / 1e6,
            "accu": sum(r.kind == "accu" for r in requests),
            "kinematic_wave": sum(r.kind == "kinematic_wave" for r in requests)}


def run_sequential_plain(server, requests, keep_results=True):
    """Reference-style: one request at a time, in arrival order, each through the plain drop-in path
    (the flow topology is built for every call, then one kinematic_wave call per time step; one stream,
    no overlap).  The result is read back to host memory, as in Server.run."""
    torch, lfr = server.torch, server.lfr
    t0 = time.perf_counter()
    for r in sorted(requests, key=lambda r: r.arrival):
        now = time.perf_counter() - t0
        if r.arrival > now:
            time.sleep(r.arrival - now)
        r.start = time.perf_counter() - t0
        fd = lfr.PartitionedArray(server.grids[r.grid].data)  # fresh array: no cached topology
        x = device_inputs(r, fd.shape, server.device)
        if r.kind == "accu":
            out = lfr.accu(fd, lfr.PartitionedArray(x["material"])).data
        else:
            q = lfr.PartitionedArray(x["discharge"])
            lat, al = lfr.PartitionedArray(x["lateral"]), lfr.PartitionedArray(x["alpha"])
            for _ in range(r.steps):
                q = lfr.kinematic_wave(fd, q, lat, al, 0.6, 3600.0, 100.0)
            out = q.data
        res = out.cpu().numpy()
        r.done = time.perf_counter() - t0
        if keep_results:
            r.result = res
        fd.topology().close()
    return summarize(requests, time.perf_counter() - t0, server)


def run_sequential_resident(server, requests, keep_results=True):
    """The plain drop-in at its best: one request at a time, in arrival order, on the server's resident
    topology of its grid (no build per call) with all kinematic-wave steps in one
    kinematic_wave_steps call; one stream, no overlap; the result read back to host memory, as in
    Server.run."""
    torch = server.torch
    from . import _lib
    L = _lib.lib()
    stream = torch.cuda.current_stream(server.device)
    t0 = time.perf_counter()
    for r in sorted(requests, key=lambda r: r.arrival):
        now = time.perf_counter() - t0
        if r.arrival > now:
            time.sleep(r.arrival - now)
        r.start = time.perf_counter() - t0
        fd = server.grids[r.grid]
        topo = server.topologies[r.grid]
        x = device_inputs(r, fd.shape, server.device)
        if r.kind == "accu":
            out = torch.empty(fd.shape, dtype=torch.float32, device=server.device)
            _lib.check(L.lue_gpu_accu_f32(topo.handle, x["material"].data_ptr(), 0.0, out.data_ptr(),
                                          stream.cuda_stream))
        else:
            out = torch.empty(fd.shape, dtype=torch.float64, device=server.device)
            _lib.check(L.lue_gpu_kinematic_wave_steps_f64_f32in(
                topo.handle, x["discharge"].data_ptr(), x["lateral"].data_ptr(), 0.0, x["alpha"].data_ptr(), 0.0,
                0.6, 3600.0, 100.0, r.steps, out.data_ptr(), stream.cuda_stream))
        res = out.cpu().numpy()
        r.done = time.perf_counter() - t0
        if keep_results:
            r.result = res
    return summarize(requests, time.perf_counter() - t0, server)


def pool_shapes(n=128, lo=256, hi=8192, seed=21):
    from .ensemble import catchment_sides
    return [(s, s) for s in catchment_sides(n, lo, hi, seed)]


def build_pool(shapes, seed=21, amplitude=200.0):
    from .ensemble import build_flow_directions
    return build_flow_directions([s[0] for s in shapes], seed, amplitude)
