"""Seeded synthetic inputs for the flow-routing workloads.

The terrain pipeline (fBm gradient-noise DEM on a south-tilted plane, Priority-Flood+epsilon depression
filling, the reference's D8 rule) runs in C (csrc/synthetic.c, built into liblue_synth.so); the
material, threshold, fraction, discharge, rainfall and alpha fields are drawn with numpy's PCG64 from
the same seed.  Identical seeds give identical bytes on x86-64 and aarch64; ``sha256`` records them.

Workloads (the reference publishes no benchmark data, so these stand in for it):

- ``accu_1k``: 1024 x 1024 in 256 x 256 partitions, amplitude 50 m, material U[0, 1).
- ``accu_16k``: 16384 x 16384, amplitude 200 m, material lognormal(0, 1), threshold U[0, 0.5),
  fraction U[0, 1].
- ``kw_8k``: 8192 x 8192, amplitude 200 m, discharge U[0, 1] m3/s (float64), lateral inflow from
  seeded Gaussian rain blobs of 0-20 mm/h (float32), alpha U[1, 5] (float32), beta 0.6, dt 3600 s,
  channel length 100 m.
"""
import ctypes
import hashlib
import os

import numpy as np

from . import _build

CELL_SIZE = 10.0      # metres per cell
TILT = 0.01           # 1 % towards the south edge
OCTAVES = 10


def _lib():
    L = ctypes.CDLL(_build.synth_library())
    i64, p, d, i32, u64 = ctypes.c_int64, ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_uint64
    L.lue_synth_dem.argtypes = [i64, i64, u64, d, d, d, d, i32, i32, p]
    L.lue_synth_fill.argtypes = [i64, i64, p]
    L.lue_synth_d8.argtypes = [i64, i64, p, i32, p]
    L.lue_synth_validate.argtypes = [i64, i64, p, p]
    return L


def dem(rows, cols, seed, amplitude, wavelength=None, nthreads=None):
    """Float64 DEM: fBm of gradient noise (amplitude metres) on a plane tilted towards the south."""
    L = _lib()
    z = np.empty((rows, cols), np.float64)
    wl = float(wavelength if wavelength is not None else max(rows, cols) / 4)
    nt = nthreads or min(os.cpu_count() or 1, 64)
    rc = L.lue_synth_dem(rows, cols, seed, float(amplitude), CELL_SIZE, TILT, wl, OCTAVES, nt, z.ctypes.data)
    if rc:
        raise RuntimeError(f"lue_synth_dem failed ({rc})")
    return z


def fill(z):
    """Priority-Flood+epsilon depression filling, in place."""
    rc = _lib().lue_synth_fill(z.shape[0], z.shape[1], z.ctypes.data)
    if rc:
        raise RuntimeError(f"lue_synth_fill failed ({rc})")
    return z


def d8(z, nthreads=None):
    fd = np.empty(z.shape, np.uint8)
    nt = nthreads or min(os.cpu_count() or 1, 64)
    _lib().lue_synth_d8(z.shape[0], z.shape[1], np.ascontiguousarray(z).ctypes.data, nt, fd.ctypes.data)
    return fd


def validate(fd):
    """dict(cycle_cells, interior_sinks, into_no_data, longest_path, edge_outlets)."""
    s = np.zeros(5, np.int64)
    fd = np.ascontiguousarray(fd, dtype=np.uint8)
    rc = _lib().lue_synth_validate(fd.shape[0], fd.shape[1], fd.ctypes.data, s.ctypes.data)
    if rc:
        raise RuntimeError(f"lue_synth_validate failed ({rc})")
    return dict(cycle_cells=int(s[0]), interior_sinks=int(s[1]), into_no_data=int(s[2]),
                longest_path=int(s[3]), edge_outlets=int(s[4]))


def flow_direction(rows, cols, seed, amplitude, wavelength=None):
    z = dem(rows, cols, seed, amplitude, wavelength)
    fill(z)
    return d8(z)


def sha256(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def _cache_path(key):
    d = os.environ.get("LUE_GB300_CACHE", os.path.join("/tmp", "lue_gb300_cache"))
    os.makedirs(d, exist_ok=True)
    return os.path.join(d, key + ".npy")


def cached_flow_direction(rows, cols, seed, amplitude, wavelength=None):
    """flow_direction(), memoised on disk (the 16384^2 terrain takes about a minute to build)."""
    key = f"fd_v1_{rows}x{cols}_s{seed}_a{amplitude:g}_w{wavelength or 0:g}"
    path = _cache_path(key)
    if os.path.exists(path):
        try:
            return np.load(path)
        except Exception:
            pass
    fd = flow_direction(rows, cols, seed, amplitude, wavelength)
    tmp = path + f".tmp{os.getpid()}.npy"
    np.save(tmp, fd)
    os.replace(tmp, path)
    return fd


def rain_blobs(rows, cols, rng, n_blobs=24, max_mm_per_h=20.0):
    """Float32 lateral inflow in m^3/s per metre of channel from Gaussian rain blobs of 0-20 mm/h.

    Rain intensity i [mm/h] over a cell of CELL_SIZE^2 m^2 gives i / 1000 / 3600 * CELL_SIZE^2 m^3/s;
    per metre of channel (the reference's lateral inflow unit, m^3/s/m) that is divided by CELL_SIZE.
    """
    r = np.arange(rows, dtype=np.float32)[:, None]
    c = np.arange(cols, dtype=np.float32)[None, :]
    i = np.zeros((rows, cols), np.float32)
    for _ in range(n_blobs):
        r0, c0 = rng.uniform(0, rows), rng.uniform(0, cols)
        s = rng.uniform(0.05, 0.25) * max(rows, cols)
        peak = rng.uniform(0.2, 1.0) * max_mm_per_h
        i += (peak * np.exp(-(((r - r0) ** 2) + ((c - c0) ** 2)) / (2 * s * s))).astype(np.float32)
    np.minimum(i, max_mm_per_h, out=i)
    factor = np.float32(CELL_SIZE * CELL_SIZE / 1000.0 / 3600.0 / CELL_SIZE)
    return (i * factor).astype(np.float32)


WORKLOADS = {
    "accu_1k": dict(rows=1024, cols=1024, partition=(256, 256), amplitude=50.0, seed=1),
    "accu_16k": dict(rows=16384, cols=16384, partition=(2048, 2048), amplitude=200.0, seed=2),
    "accu_8k": dict(rows=8192, cols=8192, partition=(1024, 1024), amplitude=200.0, seed=4),
    "kw_8k": dict(rows=8192, cols=8192, partition=(1024, 1024), amplitude=200.0, seed=3),
}


def accu_inputs(rows, cols, seed, amplitude, distribution="lognormal", cached=True, **_):
    """flow direction + float32 material (+ threshold, fraction) for an accu workload."""
    fd = (cached_flow_direction if cached else flow_direction)(rows, cols, seed, amplitude)
    rng = np.random.default_rng(seed + 1000)
    if distribution == "uniform":
        material = rng.random((rows, cols), dtype=np.float32)
    else:
        material = rng.lognormal(0.0, 1.0, (rows, cols)).astype(np.float32)
    threshold = (rng.random((rows, cols), dtype=np.float32) * np.float32(0.5)).astype(np.float32)
    fraction = rng.random((rows, cols), dtype=np.float32)
    return dict(flow_direction=fd, material=material, threshold=threshold, fraction=fraction)


def kinematic_wave_inputs(rows, cols, seed, amplitude, cached=True, **_):
    fd = (cached_flow_direction if cached else flow_direction)(rows, cols, seed, amplitude)
    rng = np.random.default_rng(seed + 2000)
    discharge = rng.random((rows, cols))  # float64 U[0, 1)
    lateral = rain_blobs(rows, cols, rng)
    alpha = (np.float32(1.0) + np.float32(4.0) * rng.random((rows, cols), dtype=np.float32)).astype(np.float32)
    return dict(flow_direction=fd, discharge=discharge, lateral_inflow=lateral, alpha=alpha, beta=0.6,
                time_step_duration=3600.0, channel_length=100.0)


def dem_device(rows, cols, seed, amplitude, wavelength=None, octaves=8, device="cuda"):
    """Float32 fBm DEM generated on the GPU with torch (hashed-gradient noise, quintic fade, octaves at
    halving wavelength and amplitude) on the same south-tilted plane as dem().  It is not bit-identical to
    dem(); it serves the pools of many grids (ensembles, serving), whose D8 rasters come from
    lue_gpu_d8_flow_direction without depression filling, so they keep interior sinks (pits)."""
    import torch

    wl = float(wavelength if wavelength is not None else max(rows, cols) / 4)
    r = torch.arange(rows, device=device, dtype=torch.float64)[:, None]
    c = torch.arange(cols, device=device, dtype=torch.float64)[None, :]
    gx = torch.tensor([np.cos(k * np.pi / 8) for k in range(16)], device=device, dtype=torch.float64)
    gy = torch.tensor([np.sin(k * np.pi / 8) for k in range(16)], device=device, dtype=torch.float64)
    m1, m2 = 0x632BE59BD9B4E019, 0x9E3779B97F4A7C15 - (1 << 64)

    def grad(ix, iy, s, dx, dy):
        h = ix * m1 + iy * m2 + s
        h = h ^ (h >> 29)
        h = h * (0xBF58476D1CE4E5B9 - (1 << 64))
        h = h ^ (h >> 32)
        k = (h & 15)
        return gx[k] * dx + gy[k] * dy

    total = torch.zeros((rows, cols), device=device, dtype=torch.float64)
    amp, norm, lam = 1.0, 0.0, wl
    for o in range(octaves):
        x, y = c / lam, r / lam
        fx, fy = torch.floor(x), torch.floor(y)
        ix, iy = fx.to(torch.int64), fy.to(torch.int64)
        dx, dy = x - fx, y - fy
        s = seed * 1000003 + o * 7919
        n00 = grad(ix, iy, s, dx, dy)
        n10 = grad(ix + 1, iy, s, dx - 1, dy)
        n01 = grad(ix, iy + 1, s, dx, dy - 1)
        n11 = grad(ix + 1, iy + 1, s, dx - 1, dy - 1)
        u = dx * dx * dx * (dx * (dx * 6 - 15) + 10)
        v = dy * dy * dy * (dy * (dy * 6 - 15) + 10)
        a = n00 + u * (n10 - n00)
        b = n01 + u * (n11 - n01)
        total += amp * (a + v * (b - a))
        norm += amp
        amp *= 0.5
        lam *= 0.5
    base = (rows - 1 - r) * CELL_SIZE * TILT + amplitude + 1.0
    return (base + amplitude * total / norm).to(torch.float32)
