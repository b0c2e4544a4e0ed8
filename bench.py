#!/usr/bin/env python3
"""Benchmark of the flow-routing hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (default ``accu_16k``): accu over a 16384 x 16384 D8 raster (268,435,456 cells) built from a
seeded fBm DEM (amplitude 200 m, 1 % tilt to the south, Priority-Flood+epsilon filled, the reference's
D8 rule), float32 lognormal(0, 1) material, partitions 2048 x 2048.  A step is one accu pass over the
whole raster.  The flow topology is built once (timed and reported separately) and stays resident, as
for a model that routes many inputs over one flow-direction raster.

Reported (one JSON line, rank 0):
  value      Mcells/s of the device-resident step (inputs in HBM), K steps timed with CUDA events on
             the launching stream between barriers + synchronize; max over ranks.
  e2e        the same metric through the public API (lue_gb300.framework.from_numpy -> accu, which calls
             the C ABI -> to_numpy_async) with host buffers: per step the float32 material goes
             host->device from a pinned numpy array and the outflow comes back device->host into one.
  roofline   algorithmic bytes (fd 1 + material 4 + outflow 4 = 9 B/cell) / mean step time against the
             measured HBM copy bandwidth; traffic from the committed ncu summary when present.
  cpu_baseline  the CPU oracle (a restatement of the reference's partitioned ridge walk, threaded
             one task per partition) on the whole raster, one pass, rank 0 only.
  accuracy   the GPU results of the timed run against the float64 oracle on the same inputs: accu and
             accu_threshold on the whole 16384^2 raster (float32 tolerance 1e-5), and the 100-step
             kinematic wave on the whole 8192^2 raster against 100 single-step float64-solve calls and on
             rows 0-1023 against 100 oracle steps (float64 tolerance 1e-9).
  extra.accu_threshold  accu_threshold over the same raster and material (threshold uniform [0, 0.5)):
             the path engine, and the stage engine with its default and its autotuned schedule.
  extra.kinematic_wave  kinematic_wave steps over the 8192 x 8192 workload (float64 discharge).

--impl reference times the reference algorithm on the CPU (the oracle port, every host core), since
the reference (HPX + Boost) cannot be built here; each step is one accu pass over the workload's whole
raster.  Multi-GPU (torchrun): each rank routes its own replica of the workload; no
collective is involved (replicas only; scaling "weak").
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

ACCU_BYTES_PER_CELL = 9      # fd 1 + material 4 + outflow 4
KW_BYTES_PER_CELL = 25       # fd 1 + Q_cur 8 + lateral 4 + alpha 4 + Q_new 8
THRESHOLD_BYTES_PER_CELL = 17  # fd 1 + material 4 + threshold 4 + flux 4 + state 4
METRIC = "accu Mcells/s (16384^2 D8 raster, float32 material)"  # the headline metric, on accu_16k


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_value(key, kernel):
    """The numbers of a committed ncu summary line '<key> <kernel> <v1> <v2> ...' (None if absent)."""
    d = os.path.join(ROOT, "profiles")
    if not os.path.isdir(d):
        return None
    for name in sorted(os.listdir(d)):
        if not name.endswith((".md", ".txt")):
            continue
        for line in open(os.path.join(d, name)):
            parts = line.strip().strip("`").split()
            if len(parts) >= 3 and parts[0] == key and parts[1] == kernel:
                return [float(x) for x in parts[2:]], name
    return None


def profile_traffic(kernel):
    """Per-launch DRAM bytes of `kernel` from a committed ncu summary line
    'traffic_per_launch <kernel> <bytes> <units_per_launch>'; scaled to a launch of this workload."""
    d = os.path.join(ROOT, "profiles")
    if not os.path.isdir(d):
        return None
    for name in sorted(os.listdir(d)):
        if not name.endswith((".md", ".txt")):
            continue
        for line in open(os.path.join(d, name)):
            parts = line.strip().strip("`").split()
            if len(parts) == 4 and parts[0] == "traffic_per_launch" and parts[1] == kernel:
                return float(parts[2]), float(parts[3])
    return None


class ClockSampler:
    """nvidia-smi SM clock / throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def outlet_mask(fd):
    """Cells whose flow leaves the array or stops (sinks): where all routed material ends up."""
    import torch
    lut_dr = torch.zeros(256, dtype=torch.int32, device=fd.device)
    lut_dc = torch.zeros(256, dtype=torch.int32, device=fd.device)
    for code, (dr, dc) in {7: (-1, -1), 8: (-1, 0), 9: (-1, 1), 4: (0, -1), 6: (0, 1), 1: (1, -1), 2: (1, 0),
                           3: (1, 1)}.items():
        lut_dr[code], lut_dc[code] = dr, dc
    rows, cols = fd.shape
    idx = fd.long()
    rr = torch.arange(rows, device=fd.device, dtype=torch.int32)[:, None] + lut_dr[idx]
    cc = torch.arange(cols, device=fd.device, dtype=torch.int32)[None, :] + lut_dc[idx]
    sink = (lut_dr[idx] == 0) & (lut_dc[idx] == 0) & (fd != 255)
    off = (rr < 0) | (rr >= rows) | (cc < 0) | (cc >= cols)
    return sink | off


def cpu_sample(inputs, partition):
    """The CPU arm's workload: the whole raster and material of the GPU workload, same partitioning."""
    fd = np.ascontiguousarray(inputs["flow_direction"])
    m = np.ascontiguousarray(inputs["material"])
    return fd, m, (min(partition[0], fd.shape[0]), min(partition[1], fd.shape[1]))


def run_cpu_accu(fd, m, partition, nthreads):
    from oracle import oracle
    t0 = time.perf_counter()
    oracle.accu(fd, m, partition, dtype=np.float32, nthreads=nthreads)
    return time.perf_counter() - t0


def best_cpu_partition(fd, m, nominal, nthreads):
    """The partition shape at which the CPU port of the reference's algorithm runs fastest on the
    raster, from a small sweep (one pass each) over the workload's partition shape and square shapes of
    1024, 2048 and 4096 cells, as a user of the reference would pick it.  Returns (shape,
    {shape: seconds})."""
    rows, cols = fd.shape
    cands = {(min(nominal[0], rows), min(nominal[1], cols))}
    cands.update((min(s, rows), min(s, cols)) for s in (1024, 2048, 4096))
    times = {c: run_cpu_accu(fd, m, c, nthreads) for c in sorted(cands)}
    best = min(times, key=times.get)
    return best, times


def rel_error_device(got, want, floor):
    """Max and mean of |got - want| / max(|want|, floor) (tests/parity.py) over the cells where want is
    not NaN, computed on the device in float64; `got` a device tensor, `want` a float64 numpy array of
    the same shape.  NaN positions must be identical (else ValueError)."""
    import torch
    g = got.reshape(-1)
    w_host = torch.from_numpy(np.ascontiguousarray(want).reshape(-1))
    mx, total, count = 0.0, 0.0, 0
    chunk = 1 << 26
    for k in range(0, g.numel(), chunk):
        gd = g[k:k + chunk].double()
        wd = w_host[k:k + chunk].to(g.device, non_blocking=False)
        nan_g, nan_w = torch.isnan(gd), torch.isnan(wd)
        if not torch.equal(nan_g, nan_w):
            raise ValueError(f"no-data positions differ ({int((nan_g != nan_w).sum())} cells)")
        ok = ~nan_w
        e = (gd[ok] - wd[ok]).abs() / wd[ok].abs().clamp_min(floor)
        if e.numel():
            mx = max(mx, float(e.max()))
            total += float(e.sum())
            count += e.numel()
    return mx, (total / count if count else 0.0)


def accuracy_full_raster(inputs, ps, accu_out, thr_holder, nthreads):
    """C2's results on the whole raster against the float64 oracle (oracle/lue_oracle.c, threaded) on the
    same inputs: the accu output of the last timed step, and the accu_threshold flux and state of the
    threshold leg.  Relative error with the float32 floor of tests/parity.py; tolerance 1e-5."""
    from oracle import oracle
    from tests import parity
    fd, m = inputs["flow_direction"], inputs["material"]
    m64 = m.astype(np.float64)
    out = {"against": "oracle/lue_oracle.c in float64, whole raster", "floor": parity.FLOOR32,
           "tolerance": parity.RTOL32, "cores": nthreads}
    t0 = time.perf_counter()
    want = oracle.accu(fd, m64, ps, dtype=np.float64, nthreads=nthreads)
    out["oracle_accu_s"] = round(time.perf_counter() - t0, 2)
    mx, mean = rel_error_device(accu_out, want, parity.FLOOR32)
    del want
    out["accu"] = {"max_rel_err": mx, "mean_rel_err": mean}
    if thr_holder.get("flux") is not None:
        thr = thr_holder["threshold"]
        t0 = time.perf_counter()
        wf, ws = oracle.accu_threshold(fd, m64, thr.astype(np.float64), ps, dtype=np.float64, nthreads=nthreads)
        out["oracle_accu_threshold_s"] = round(time.perf_counter() - t0, 2)
        for name, g, w in (("accu_threshold_flux", thr_holder["flux"], wf),
                           ("accu_threshold_state", thr_holder["state"], ws)):
            mx, mean = rel_error_device(g, w, parity.FLOOR32)
            out[name] = {"max_rel_err": mx, "mean_rel_err": mean}
        del wf, ws
    out["within_tolerance"] = all(v["max_rel_err"] <= parity.RTOL32 for k, v in out.items()
                                  if isinstance(v, dict) and "max_rel_err" in v)
    return out


def workload_inputs(name):
    from lue_gb300 import synthetic
    w = synthetic.WORKLOADS[name]
    inputs = synthetic.accu_inputs(w["rows"], w["cols"], w["seed"], w["amplitude"])
    return w, inputs


def bench_reference(args, world, rank):
    """CPU reference arm: the oracle port of the reference's algorithm on every host core."""
    if rank != 0:
        return
    w, inputs = workload_inputs(args.workload)
    fd, m, ps = cpu_sample(inputs, w["partition"])
    nthreads = os.cpu_count() or 1
    ps, sweep = best_cpu_partition(fd, m, ps, nthreads)
    for _ in range(args.warmup):
        run_cpu_accu(fd, m, ps, nthreads)
    times = [run_cpu_accu(fd, m, ps, nthreads) for _ in range(args.steps)]
    total = sum(times)
    value = fd.size * args.steps / total / 1e6
    sample = (f"accu over the whole {w['rows']}x{w['cols']} raster per step (partitions {ps[0]}x{ps[1]}, the "
              f"fastest of a sweep: " + ", ".join(f"{a}x{b} {t * 1000:.0f} ms" for (a, b), t in sweep.items())
              + ")")
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3),
        "unit": "Mcells/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * total / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded fBm DEM, lognormal material)",
        "config": {"workload": args.workload, "rows": w["rows"], "cols": w["cols"],
                   "partition_shape": list(w["partition"]), "cpu_partition_shape": list(ps),
                   "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": round(value, 3), "unit": "Mcells/s", "cores": nthreads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 3), "unit": "Mcells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference (HPX + Boost) not buildable offline; oracle/lue_oracle.c restates its partitioned "
                "ridge walk, one thread task per partition",
    }
    print(json.dumps(line), flush=True)


def bench_ours(args, world, rank, local):
    import torch

    from lue_gb300 import framework as lfr

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w, inputs = workload_inputs(args.workload)
    rows, cols, ps = w["rows"], w["cols"], w["partition"]
    n = rows * cols
    stream = torch.cuda.current_stream(dev)

    # resident inputs
    fd_d = lfr.from_numpy(inputs["flow_direction"], ps, device=dev)
    m_d = lfr.from_numpy(inputs["material"], ps, device=dev)
    torch.cuda.synchronize()

    t0 = time.perf_counter()
    topo = fd_d.topology()
    torch.cuda.synchronize()
    topology_ms = 1000 * (time.perf_counter() - t0)
    stats = topo.stats()

    from lue_gb300 import _lib
    engine = "tiles" if stats.get("tile_exits", 0) > 0 else "walk"
    out = None
    for _ in range(args.warmup):
        out = lfr.accu(fd_d, m_d)
    torch.cuda.synchronize()
    launches0 = _lib.lib().lue_gpu_kernel_launches()

    # timed, device-resident
    sampler = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    sampler.start()
    time.sleep(0.3)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    ev[0].record(stream)
    for k in range(args.steps):
        out = lfr.accu(fd_d, m_d)
        ev[k + 1].record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    launches = _lib.lib().lue_gpu_kernel_launches() - launches0
    barrier(world)
    step_ms = [ev[k].elapsed_time(ev[k + 1]) for k in range(args.steps)]
    total_s = max_over_ranks(sum(step_ms) / 1000.0, world)
    value = world * n * args.steps / total_s / 1e6

    # mass balance: the material reaching outlets and sinks equals the material put in
    mask = outlet_mask(fd_d.data)
    total_in = float(m_d.data.double().sum())
    total_out = float(out.data.double()[mask].sum())
    del mask

    # end to end through the public API with host buffers (lue_gb300.framework: from_numpy -> accu ->
    # to_numpy_async; accu is the C ABI's lue_gpu_accu_f32): every step the float32 material goes
    # host->device from a pinned numpy array, accu runs, and the outflow comes back device->host into a
    # pinned numpy array.  Three streams overlap the upload of step k+1 and the download of step k-1 with
    # the routing of step k; arrays made on one stream and used on another are recorded on it.
    e2e_steps = max(3, min(args.steps, 20))
    m_np = lfr.pinned_empty((rows, cols), np.float32)
    m_np[...] = inputs["material"]
    out_np = [lfr.pinned_empty((rows, cols), np.float32) for _ in range(2)]
    s_in, s_c, s_out = (torch.cuda.Stream(dev) for _ in range(3))

    def e2e_trial():
        torch.cuda.synchronize()
        barrier(world)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(s_in)
        s_c.wait_event(e0)
        s_out.wait_event(e0)
        for k in range(e2e_steps):
            with torch.cuda.stream(s_in):
                md = lfr.from_numpy(m_np, ps, device=dev)
                ev_in = torch.cuda.Event()
                ev_in.record(s_in)
            s_c.wait_event(ev_in)
            with torch.cuda.stream(s_c):
                md.data.record_stream(s_c)
                o = lfr.accu(fd_d, md)
                ev_c = torch.cuda.Event()
                ev_c.record(s_c)
            s_out.wait_event(ev_c)
            with torch.cuda.stream(s_out):
                o.data.record_stream(s_out)
                lfr.to_numpy_async(o, out_np[k % 2])
        e1.record(s_out)
        torch.cuda.synchronize()
        return max_over_ranks(e0.elapsed_time(e1) / 1000.0, world)

    def link_trial():
        """The same bytes moved without the routing: per step the material host->device on one stream and
        an outflow-sized buffer device->host on another, at the same time (the host link's capacity for
        this step's traffic)."""
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(s_in)
        s_out.wait_event(e0)
        for k in range(e2e_steps):
            with torch.cuda.stream(s_in):
                md = lfr.from_numpy(m_np, ps, device=dev)
            with torch.cuda.stream(s_out):
                torch.from_numpy(out_np[k % 2]).copy_(out.data, non_blocking=True)
            del md
        s_in.wait_stream(s_out)
        e1.record(s_in)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1000.0

    # The host memory and its link are shared with the other jobs of the machine: five trials, the
    # median is the value, the fastest is reported beside it
    e2e_trials = [e2e_trial() for _ in range(5)]
    link_s = min(link_trial() for _ in range(3))
    e2e_s = statistics.median(e2e_trials)
    e2e_value = world * n * e2e_steps / e2e_s / 1e6
    e2e_best = world * n * e2e_steps / min(e2e_trials) / 1e6
    assert np.array_equal(out_np[(e2e_steps - 1) % 2], out.data.cpu().numpy()), "end-to-end result differs"

    # roofline of the accu call (its kernels together; one call per step)
    peak, peak_kind = peaks()
    mean_step_s = statistics.mean(step_ms) / 1000.0
    achieved = ACCU_BYTES_PER_CELL * n / mean_step_s / 1e9
    tr = profile_traffic(f"accu_f32_{engine}")
    traffic = None if tr is None else round(tr[0] / tr[1] * n)

    extra = {}

    def leg(name, fn):
        try:
            extra[name] = fn(args, dev)
        except Exception as ex:  # a failing secondary leg must not hide the headline line
            extra[name] = {"error": f"{type(ex).__name__}: {ex}"}
        torch.cuda.synchronize()
        torch.cuda.empty_cache()

    thr_holder = {}
    if args.threshold_calls > 0 and rank == 0:
        leg("accu_threshold", lambda a, d: bench_threshold(a, d, fd_d, m_d, inputs, thr_holder))
    if args.kinematic_wave_steps > 0 and rank == 0:
        leg("kinematic_wave", bench_kinematic_wave)
    if not args.no_ensemble and rank == 0:
        leg("ensemble", bench_ensemble)
    if args.serve_seconds > 0 and rank == 0:
        leg("serving", bench_serving)

    if rank != 0:
        return
    cpu = None
    accuracy = None
    if world == 1 and not args.skip_cpu:
        fd_s, m_s, ps_s = cpu_sample(inputs, ps)
        nthreads = os.cpu_count() or 1
        ps_s, sweep = best_cpu_partition(fd_s, m_s, ps_s, nthreads)
        t_cpu = run_cpu_accu(fd_s, m_s, ps_s, nthreads)
        cpu = {"value": round(fd_s.size / t_cpu / 1e6, 3), "unit": "Mcells/s", "cores": nthreads, "kind": "port",
               "sample": f"accu over the whole raster ({fd_s.shape[0]}x{fd_s.shape[1]} cells, partitions "
                         f"{ps_s[0]}x{ps_s[1]}, the fastest of a sweep: "
                         + ", ".join(f"{a}x{b} {t * 1000:.0f} ms" for (a, b), t in sweep.items())
                         + "), one pass, oracle/lue_oracle.c threaded"}
    if world == 1 and not args.skip_accuracy:
        try:  # the float32 error of the GPU results on the whole raster, against the float64 oracle
            accuracy = {"accu_16k": accuracy_full_raster(inputs, ps, out.data, thr_holder, os.cpu_count() or 1)}
        except Exception as e:  # noqa: BLE001  (reported in the line, the bench itself goes on)
            accuracy = {"accu_16k": {"error": f"{type(e).__name__}: {e}"}}
        thr_holder.clear()
        kw = extra.get("kinematic_wave", {})
        if "accuracy" in kw:
            accuracy["kw_8k"] = kw["accuracy"]
    line = {
        "metric": METRIC, "value": round(value, 3),
        "unit": "Mcells/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * total_s / args.steps, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded fBm DEM, lognormal material)",
        "config": {"workload": args.workload, "rows": rows, "cols": cols, "partition_shape": list(ps),
                   "l2": "inputs larger than L2 (268 MB fd + 1 GB material per step)",
                   "topology": "resident, built once", "topology_build_ms": round(topology_ms, 2),
                   "longest_flow_path_cells": stats["max_level"] + 1, "engine": engine,
                   "tile_exits": stats.get("tile_exits", 0), "exit_forest_depth": stats.get("exit_forest_depth", 0)},
        "e2e": {"value": round(e2e_value, 3), "unit": "Mcells/s", "h2d_bytes_per_step": 4 * n,
                "d2h_bytes_per_step": 4 * n, "steps": e2e_steps,
                "best_of_trials": round(e2e_best, 3),
                "link_only_ms_per_step": round(1000 * link_s / e2e_steps, 3),
                "link_frac": round(link_s / e2e_s, 3),
                "link_note": "the step's host->device and device->host bytes moved at the same time without the "
                             "routing (best of 3); link_frac = that time / the e2e time",
                "trials_ms_per_step": [round(1000 * x / e2e_steps, 2) for x in e2e_trials],
                "timed": "median of 5 trials (value), fastest beside it",
                "path": "lue_gb300.framework.from_numpy -> accu (C ABI lue_gpu_accu_f32) -> to_numpy_async, "
                        "pinned numpy arrays",
                "overlap": "upload of step k+1 and download of step k-1 beside the routing of step k "
                           "(three streams, pinned host memory)"},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "kernel": ("accu_f32 call: k_tile_exits + exit-forest scan + k_slot_inflow + k_tile_accu" if engine == "tiles"
                                else "k_walk<RouteF32<accu>>"),
                     "timed": "whole call per step (all its kernels), CUDA events on the launching stream",
                     "peak_kind": peak_kind, "bytes_per_cell": ACCU_BYTES_PER_CELL},
        "cpu_baseline": cpu,
        "accuracy": accuracy,
        "clocks": clocks,
        "gpu_launches": int(launches),
        "mass_balance": {"material_in": total_in, "outlet_outflow": total_out,
                         "rel_err": abs(total_out - total_in) / total_in},
        "extra": extra,
    }
    print(json.dumps(line), flush=True)


def bench_threshold(args, dev, fd_d, m_d, inputs, holder):
    """C2's second operation: accu_threshold over the same raster and material, threshold float32
    uniform [0, 0.5) (seeded), on the path engine (one launch per path level), with the stage engine
    (default and autotuned schedule) timed beside it.  Mass balance: what the cells keep plus what leaves
    at outlets and sinks equals the material put in."""
    import torch

    from lue_gb300 import framework as lfr

    rows, cols = inputs["material"].shape
    n = rows * cols
    rng = np.random.default_rng(17)
    thr = lfr.PartitionedArray(torch.from_numpy(rng.random((rows, cols), dtype=np.float32) * 0.5).to(dev),
                               fd_d.partition_shape)
    stream = torch.cuda.current_stream(dev)
    t0 = time.perf_counter()
    flux, state = lfr.accu_threshold(fd_d, m_d, thr)  # builds the stages
    torch.cuda.synchronize()
    first_s = time.perf_counter() - t0
    calls = args.threshold_calls
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed():
        nonlocal flux, state
        e0.record(stream)
        for _ in range(calls):
            flux, state = lfr.accu_threshold(fd_d, m_d, thr)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1000.0 / calls

    s = timed()  # the path engine
    holder.update(flux=flux.data, state=state.data, threshold=thr.data.cpu().numpy())
    mask = outlet_mask(fd_d.data)
    total_in = float(m_d.data.double().sum())
    kept = float(state.data.double().sum())
    left = float(flux.data.double()[mask].sum())
    # the stage engine on the same call, with its default and its autotuned schedule
    stage = None
    if args.stage_compare:
        os.environ["LUE_GB300_ENGINE"] = "stage"
        try:
            t0 = time.perf_counter()
            lfr.accu_threshold(fd_d, m_d, thr)  # builds the stages
            torch.cuda.synchronize()
            stage_first = time.perf_counter() - t0
            default_schedule = fd_d.topology().stage_schedule()
            s_default = timed()
            tuned = None
            if not args.no_autotune:
                t0 = time.perf_counter()
                best = lfr.autotune_stage_schedule(fd_d, lambda: lfr.accu_threshold(fd_d, m_d, thr))
                tune_s = time.perf_counter() - t0
                tuned = {"schedule": {k: best[k] for k in ("cap", "threads", "publish_every")},
                         "tuner_ms_of_best": round(best["ms"], 3), "tuning_s": round(tune_s, 2),
                         "ms_per_call": round(1000 * timed(), 3)}
            stage = {"engine": "stage engine: 32 x 32 tiles cut into stages of at most `cap` cells by crossing "
                               "depth, one dataflow launch", "first_call_ms": round(1000 * stage_first, 2),
                     "default_schedule": {"schedule": default_schedule, "ms_per_call": round(1000 * s_default, 3)},
                     "autotuned": tuned}
        finally:
            del os.environ["LUE_GB300_ENGINE"]
    return {"workload": f"{args.workload} raster and material, threshold uniform [0, 0.5) float32 ({rows}x{cols})",
            "calls": calls, "ms_per_call": round(1000 * s, 3), "value": round(n / s / 1e6, 3), "unit": "Mcells/s",
            "roofline_frac_hbm": round(THRESHOLD_BYTES_PER_CELL * n / s / 1e9 / peaks()[0], 4),
            "bytes_per_cell": THRESHOLD_BYTES_PER_CELL,
            "first_call_ms": round(1000 * first_s, 2),
            "engine": "path engine: heavy paths of the flow forest, level by level, one float-float prefix scan "
                      "of the cells' max-plus maps per level (lue_gpu_accu_threshold_f32)",
            "stage_engine": stage,
            "mass_balance": {"material_in": total_in, "kept_plus_outlet_flux": kept + left,
                             "rel_err": abs(kept + left - total_in) / total_in}}


def bench_kinematic_wave(args, dev):
    """C3: kinematic_wave over the 8192 x 8192 workload, `steps` time steps in one call (the stage engine:
    pipelined time steps in shared-memory stages, float-float solve), next to single-step calls."""
    import torch

    from lue_gb300 import framework as lfr
    from lue_gb300 import synthetic

    w = synthetic.WORKLOADS["kw_8k"]
    d = synthetic.kinematic_wave_inputs(w["rows"], w["cols"], w["seed"], w["amplitude"])
    ps = w["partition"]
    fd = lfr.from_numpy(d["flow_direction"], ps, device=dev)
    q = lfr.from_numpy(d["discharge"], ps, device=dev)
    lat = lfr.from_numpy(d["lateral_inflow"], ps, device=dev)
    alpha = lfr.from_numpy(d["alpha"], ps, device=dev)
    fd.topology()
    n = w["rows"] * w["cols"]
    stream = torch.cuda.current_stream(dev)
    T = args.kinematic_wave_steps
    lfr.kinematic_wave_steps(fd, q, lat, alpha, 0.6, 3600.0, 100.0, T)  # builds the stages + history
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed_multi():
        e0.record(stream)
        o = lfr.kinematic_wave_steps(fd, q, lat, alpha, 0.6, 3600.0, 100.0, T)
        e1.record(stream)
        torch.cuda.synchronize()
        return o, e0.elapsed_time(e1) / 1000.0

    default_schedule = fd.topology().stage_schedule()
    out, s_multi = timed_multi()
    s_default = s_multi
    single_steps = 3
    qq = q
    e0.record(stream)
    for _ in range(single_steps):
        qq = lfr.kinematic_wave(fd, qq, lat, alpha, 0.6, 3600.0, 100.0)
    e1.record(stream)
    torch.cuda.synchronize()
    s_single = e0.elapsed_time(e1) / 1000.0 / single_steps
    tuned = None
    if not args.no_autotune:
        t0 = time.perf_counter()
        best = lfr.autotune_stage_schedule(fd, lambda: lfr.kinematic_wave_steps(fd, q, lat, alpha, 0.6, 3600.0, 100.0, T))
        tune_s = time.perf_counter() - t0
        out, s_multi = timed_multi()
        tuned = {"schedule": {k: best[k] for k in ("cap", "threads", "publish_every")},
                 "tuner_ms_of_best": round(best["ms"], 3), "tuning_s": round(tune_s, 2),
                 "ms_per_step": round(1000 * s_multi / T, 3)}
    finite = torch.isfinite(out.data)
    # compute roofline of the multi-step kernel: warp instructions per cell step (ncu, the same 8192^2 x
    # 100-step call) x cell steps per second, against the SM issue peak (4 warp instructions per cycle per
    # SM) at the maximum SM clock
    compute = None
    ipcs = profile_value("warp_instructions_per_cell_step", "k_stage_flow_kw")
    if ipcs is not None:
        props = torch.cuda.get_device_properties(dev)
        mhz = 2070.0
        path = os.path.join(ROOT, "MEASURED_PEAKS.json")
        if os.path.exists(path):
            mhz = float(json.load(open(path)).get("sm_max_mhz", mhz))
        peak_issue = props.multi_processor_count * 4 * mhz * 1e6
        achieved_issue = ipcs[0][0] * n * T / s_multi
        fma = profile_value("fma_pipe_pct", "k_stage_flow_kw")
        compute = {"bound": "instruction issue", "unit": "warp instructions/s",
                   "achieved": round(achieved_issue, 1), "peak": round(peak_issue, 1),
                   "frac": round(achieved_issue / peak_issue, 4),
                   "warp_instructions_per_cell_step": ipcs[0][0],
                   "fma_pipe_pct_of_active": fma[0][0] if fma else None,
                   "peak_note": f"{props.multi_processor_count} SMs x 4 warp instructions per cycle at {mhz:g} MHz",
                   "source": ipcs[1]}
    accuracy = None
    if not args.skip_accuracy:
        try:
            accuracy = kinematic_wave_accuracy(args, dev, d, ps, fd, q, lat, alpha, out, T)
        except Exception as e:  # noqa: BLE001  (reported in the line, the bench itself goes on)
            accuracy = {"error": f"{type(e).__name__}: {e}"}
    return {"workload": "kw_8k (8192x8192, float64 discharge, float32 rain and alpha, beta 0.6, dt 3600 s, dx 100 m)",
            "accuracy": accuracy,
            "steps": T, "ms_per_step": round(1000 * s_multi / T, 3),
            "value": round(n * T / s_multi / 1e6, 3), "unit": "Mcells/s",
            "compute_roofline": compute,
            "default_schedule": {"schedule": default_schedule, "ms_per_step": round(1000 * s_default / T, 3)},
            "autotuned": tuned,
            "timed_schedule": "autotuned (lue_gpu_autotune_stage_schedule)" if tuned else "default",
            "single_step_call_ms": round(1000 * s_single, 3),
            "single_step_call_mcells_per_s": round(n / s_single / 1e6, 3),
            "engine": "stage engine, pipelined steps, float-float solve in y = Q^(1/5) "
                      "(lue_gpu_kinematic_wave_steps_f64_f32in)",
            "roofline_note": "all steps run in one call with the discharge in shared memory between steps: the "
                             "kernel is bound by instruction issue, not HBM, so its roofline is the issue rate",
            "single_step_roofline_frac_hbm": round(KW_BYTES_PER_CELL * n / s_single / 1e9 / peaks()[0], 4),
            "longest_flow_path_cells": fd.topology().stats()["max_level"] + 1,
            "outflow_finite_cells": int(finite.sum())}


def kinematic_wave_accuracy(args, dev, d, ps, fd, q, lat, alpha, out, T, band_rows=1024):
    """C3's result against float64 references, tolerance 1e-9 relative (floor 1e-12):
    - the whole 8192^2 raster: the timed T-step call (stage engine, float-float solve) against T
      single-step calls with the reference-faithful float64 solve (LUE_GB300_KW_SOLVE=reference);
    - rows 0..band_rows-1 of the same inputs (flow leaving the band is dropped, as at the array edge):
      one T-step call on the band's own topology against T sequential steps of the float64 oracle
      (oracle/lue_oracle.c, threaded)."""
    import torch

    from lue_gb300 import framework as lfr
    from oracle import oracle
    from tests import parity
    res = {"tolerance": parity.RTOL64, "floor": parity.FLOOR64, "steps": T}
    os.environ["LUE_GB300_KW_SOLVE"] = "reference"
    try:
        qq = q
        t0 = time.perf_counter()
        for _ in range(T):
            qq = lfr.kinematic_wave(fd, qq, lat, alpha, 0.6, 3600.0, 100.0)
        torch.cuda.synchronize()
        secs = time.perf_counter() - t0
    finally:
        del os.environ["LUE_GB300_KW_SOLVE"]
    mx, mean = rel_error_device(out.data, qq.data.cpu().numpy(), parity.FLOOR64)
    res["whole_raster_vs_single_step_float64_calls"] = {"max_rel_err": mx, "mean_rel_err": mean,
                                                        "reference_calls_s": round(secs, 2)}
    del qq
    band = {k: np.ascontiguousarray(d[k][:band_rows]) for k in ("flow_direction", "discharge", "lateral_inflow",
                                                                "alpha")}
    bps = (min(ps[0], band_rows), ps[1])
    fdb = lfr.from_numpy(band["flow_direction"], bps, device=dev)
    got = lfr.kinematic_wave_steps(fdb, lfr.from_numpy(band["discharge"], bps, device=dev),
                                   lfr.from_numpy(band["lateral_inflow"], bps, device=dev),
                                   lfr.from_numpy(band["alpha"], bps, device=dev), 0.6, 3600.0, 100.0, T)
    want = band["discharge"]
    lat64, al64 = band["lateral_inflow"].astype(np.float64), band["alpha"].astype(np.float64)
    t0 = time.perf_counter()
    nthreads = os.cpu_count() or 1
    for _ in range(T):
        want = oracle.kinematic_wave(band["flow_direction"], want, lat64, al64, 0.6, 3600.0, 100.0, bps,
                                     dtype=np.float64, nthreads=nthreads)
    mx, mean = rel_error_device(got.data, want, parity.FLOOR64)
    res[f"rows_0_{band_rows - 1}_vs_oracle"] = {"max_rel_err": mx, "mean_rel_err": mean,
                                                "oracle_s": round(time.perf_counter() - t0, 2)}
    fdb.topology().close()
    res["within_tolerance"] = all(v["max_rel_err"] <= parity.RTOL64 for v in res.values()
                                  if isinstance(v, dict) and "max_rel_err" in v)
    return res


def bench_ensemble(args, dev):
    """C4: 256 kinematic-wave instances (64 catchments x 4 rain scenarios), 48 steps, batched in one
    atlas (one launch per step in a CUDA graph, or all steps as level waves) against one launch per
    instance and step (timed on a sample of instances)."""
    from lue_gb300 import ensemble
    inst = ensemble.ensemble_inputs(n_catchments=64, scenarios=4, lo=512, hi=4096, seed=11)
    cells = sum(i["flow_direction"].size for i in inst)
    steps = 48
    s_graph, atlas, _, stats = ensemble.run_batched(inst, steps, device=dev, graph=True)
    s_waves, _, _, _ = ensemble.run_batched(inst, steps, device=dev, waves=True)
    tuned = None
    if not args.no_autotune:
        s_tuned, _, _, tstats = ensemble.run_batched(inst, steps, device=dev, waves=True, autotune_steps=4)
        tuned = {"schedule": tstats["stage_schedule"], "tuned_on": "a 4-step call of the same atlas",
                 "tuning_s": tstats["tuning_s"], "batched_waves_s": round(s_tuned, 3),
                 "batched_waves_mcells_per_s": round(cells * steps / s_tuned / 1e6, 3)}
    s_plain, cells_plain, _ = ensemble.run_plain_resident(inst, steps, device=dev)
    sample = 8
    s_alone, cells_alone, _ = ensemble.run_unbatched(inst, steps, sample, device=dev)
    return {"workload": "64 catchments (sides log-uniform 512-4096, depression-filled D8) x 4 rain scenarios, "
                        "48 kinematic-wave steps", "instances": len(inst), "cells_per_step": cells,
            "atlas_shape": list(atlas.shape), "longest_flow_path_cells": stats["max_level"] + 1,
            "batched_graph_mcells_per_s": round(cells * steps / s_graph / 1e6, 3),
            "batched_graph_s": round(s_graph, 3),
            "batched_waves_mcells_per_s": round(cells * steps / s_waves / 1e6, 3),
            "batched_waves_s": round(s_waves, 3),
            "batched_waves_autotuned": tuned,
            "plain_resident_per_instance_mcells_per_s": round(cells_plain * steps / s_plain / 1e6, 3),
            "plain_resident_per_instance_s": round(s_plain, 3),
            "plain_resident_note": "every instance alone through the drop-in at its best: resident topology "
                                   "per catchment, device-resident inputs, one kinematic_wave_steps call of all "
                                   "48 steps per instance, CUDA events",
            "one_launch_per_instance_mcells_per_s": round(cells_alone * steps / s_alone / 1e6, 3),
            "one_launch_per_instance_sample": f"first {sample} instances, topology built per instance"}


def bench_serving(args, dev):
    """C5: Poisson stream (200 req/s) of accu and 24-step kinematic_wave requests over a pool of 128
    resident D8 grids (sides log-uniform 256-8192); p50/p99 latency, and the same requests served one at a
    time through the plain drop-in path (topology per call) for comparison."""
    import copy

    from lue_gb300 import serving
    shapes = serving.pool_shapes(n=128, lo=256, hi=8192, seed=21)
    pool = serving.build_pool(shapes, seed=21)
    server = serving.Server(pool, slots=16, device=dev)
    reqs = serving.make_requests(shapes, rate=200.0, duration=args.serve_seconds, kw_steps=24, seed=5)
    # warm-up: one request per kind on the smallest grid (clones, history planes)
    server.run(copy.deepcopy(reqs[:4]), realtime=False, keep_results=False)
    served = server.run(copy.deepcopy(reqs), realtime=True, keep_results=False)
    k = min(len(reqs), args.serve_sequential)
    sub = copy.deepcopy(reqs[:k])
    for r in sub:
        r.arrival = 0.0
    seq = serving.run_sequential_plain(server, sub, keep_results=False)
    sub3 = copy.deepcopy(reqs[:k])
    for r in sub3:
        r.arrival = 0.0
    seq_resident = serving.run_sequential_resident(server, sub3, keep_results=False)
    sub2 = copy.deepcopy(reqs[:k])
    for r in sub2:
        r.arrival = 0.0
    batched_sub = server.run(sub2, realtime=False, keep_results=False)
    return {"workload": "Poisson 200 req/s, 50 % accu (float32) / 50 % 24-step kinematic_wave (float64), "
                        "128-grid pool, sides log-uniform 256-8192", "seconds_of_arrivals": args.serve_seconds,
            "served": served,
            "same_requests_closed_loop": {"first_k": k, "continuous_batching": batched_sub,
                                          "sequential_resident_calls": seq_resident,
                                          "sequential_plain_calls": seq}}


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="accu_16k")
    ap.add_argument("--kinematic-wave-steps", type=int, default=100)
    ap.add_argument("--threshold-calls", type=int, default=3)
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--serve-seconds", type=float, default=2.0)
    ap.add_argument("--serve-sequential", type=int, default=32)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-accuracy", action="store_true",
                    help="do not compare the results with the float64 oracle on the whole raster")
    ap.add_argument("--no-autotune", action="store_true", help="time the stage legs with the default schedule only")
    ap.add_argument("--no-stage-compare", dest="stage_compare", action="store_false",
                    help="do not time accu_threshold on the stage engine beside the path engine")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_init(args)
    if args.impl == "reference":
        bench_reference(args, world, rank)
    else:
        bench_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
