"""The path engine (float32 accu_threshold, accu_fraction and accu_capacity on acyclic rasters): outflows
along the heavy paths of the flow forest from prefix scans of the cell rules' maps, level by level.

It is the default engine of these three operations, so the reference's known-answer cases
(test_gpu_golden.py) and the synthetic parity tests (test_gpu_parity.py) run through it too.  Here:
parity against the float64 oracle and against the walk engine on rasters with no-data holes, NaN and
negative material, ragged shapes and long flow paths; scalar overloads; +inf material (the walk engine
redoes the call); repeated calls and clones giving the same bits; mass balance.
"""
import numpy as np
import pytest

from lue_gb300 import synthetic
from oracle import oracle
from tests import parity

pytestmark = pytest.mark.gpu

OPS = ("threshold", "fraction", "capacity")


@pytest.fixture(scope="module")
def lfr():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from lue_gb300 import framework
    return framework


def _raster(rows, cols, seed, amplitude=40.0, holes=0.0, wavelength=None):
    fd = synthetic.flow_direction(rows, cols, seed, amplitude, wavelength=wavelength or max(rows, cols) / 2).copy()
    rng = np.random.default_rng(seed)
    if holes:
        fd[rng.random(fd.shape) < holes] = 255
    return fd, rng


def _ops(lfr, op):
    if op == "threshold":
        return lfr.accu_threshold, oracle.accu_threshold
    if op == "fraction":
        return lfr.accu_fraction, oracle.accu_fraction
    return lfr.accu_capacity, oracle.accu_capacity


def _other(rng, shape, op, scale=None):
    """Threshold U[0, 0.5), fraction U[0, 1) with a few values above 1 (outside the domain), capacity
    U[0, 3)."""
    if op == "fraction":
        b = rng.random(shape).astype(np.float32)
        b[rng.random(shape) < 0.0005] = 1.5
        return b
    return (rng.random(shape) * (scale or (0.5 if op == "threshold" else 3.0))).astype(np.float32)


def _run(lfr, op, fd, m, b, ps, engine=None, monkeypatch=None):
    gpu, _ = _ops(lfr, op)
    if engine:
        monkeypatch.setenv("LUE_GB300_ENGINE", engine)
    a = lfr.from_numpy(fd, ps)
    mb = m if np.isscalar(m) else lfr.from_numpy(m, ps)
    bb = b if np.isscalar(b) else lfr.from_numpy(b, ps)
    got = [lfr.to_numpy(x) for x in gpu(a, mb, bb)]
    if engine:
        monkeypatch.delenv("LUE_GB300_ENGINE")
    return got


@pytest.mark.parametrize("shape", [(1024, 1024), (333, 777), (65, 31), (1, 300), (300, 1)])
@pytest.mark.parametrize("op", OPS)
def test_path_engine_against_oracle_and_walk_engine(lfr, monkeypatch, shape, op):
    fd, rng = _raster(*shape, seed=71, holes=0.001)
    m = rng.lognormal(0.0, 1.0, shape).astype(np.float32)
    m[rng.random(shape) < 0.001] = np.nan
    m[rng.random(shape) < 0.001] = -1.0
    b = _other(rng, shape, op)
    b[rng.random(shape) < 0.0005] = np.nan
    ps = (min(256, shape[0]), min(256, shape[1]))
    got = _run(lfr, op, fd, m, b, ps)
    _, cpu = _ops(lfr, op)
    want = cpu(fd, m.astype(np.float64), b.astype(np.float64), ps, dtype=np.float64)
    for g, w, name in zip(got, want, ("outflow", "remainder")):
        parity.assert_close32(g, w, f"{op} {name} {shape}")
    walk = _run(lfr, op, fd, m, b, ps, engine="walk", monkeypatch=monkeypatch)
    for g, w in zip(got, walk):
        parity.assert_close32(g, w.astype(np.float64), f"{op} against the walk engine")


@pytest.mark.parametrize("op", OPS)
def test_long_paths_and_mass_balance(lfr, op):
    """A 2048^2 raster with long main channels (low-frequency terrain, amplitude 200 m): many path levels
    and paths of thousands of cells, each cut across many CTAs of the scan."""
    fd, rng = _raster(2048, 2048, seed=73, amplitude=200.0, wavelength=2048)
    m = rng.lognormal(0.0, 1.0, fd.shape).astype(np.float32)
    b = _other(rng, fd.shape, op, scale=0.5 if op == "threshold" else 50.0)
    if op == "fraction":
        b = np.minimum(b, 1.0).astype(np.float32)
    out, rem = _run(lfr, op, fd, m, b, (512, 512))
    _, cpu = _ops(lfr, op)
    wo, wr = cpu(fd, m.astype(np.float64), b.astype(np.float64), (512, 512), dtype=np.float64)
    parity.assert_close32(out, wo, f"{op} outflow")
    parity.assert_close32(rem, wr, f"{op} remainder")
    # what the cells keep plus what leaves the raster at outlets and sinks is the material put in
    rows, cols = fd.shape
    r, c = np.indices(fd.shape)
    dr = np.select([np.isin(fd, (7, 8, 9)), np.isin(fd, (1, 2, 3))], [-1, 1], 0)
    dc = np.select([np.isin(fd, (7, 4, 1)), np.isin(fd, (9, 6, 3))], [-1, 1], 0)
    leaves = ((dr == 0) & (dc == 0)) | (r + dr < 0) | (r + dr >= rows) | (c + dc < 0) | (c + dc >= cols)
    total = m.astype(np.float64).sum()
    kept = rem.astype(np.float64).sum() + out.astype(np.float64)[leaves].sum()
    assert abs(kept - total) <= 1e-5 * total


@pytest.mark.parametrize("op", OPS)
def test_scalar_overloads(lfr, op):
    fd, rng = _raster(200, 260, seed=75, holes=0.002)
    m = rng.lognormal(0.0, 1.0, fd.shape).astype(np.float32)
    b = (rng.random(fd.shape) * 0.5).astype(np.float32)
    _, cpu = _ops(lfr, op)
    for mm, bb in ((m, np.float32(0.3)), (np.float32(0.7), b), (np.float32(0.7), np.float32(0.3))):
        got = _run(lfr, op, fd, mm, bb, fd.shape)
        m64 = float(mm) if np.isscalar(mm) else mm.astype(np.float64)
        b64 = float(bb) if np.isscalar(bb) else bb.astype(np.float64)
        want = cpu(fd, m64, b64, fd.shape, dtype=np.float64)
        for g, w in zip(got, want):
            parity.assert_close32(g, w, f"{op} scalar overload")


@pytest.mark.parametrize("op", OPS)
def test_infinite_material_is_redone_by_the_walk_engine(lfr, monkeypatch, op):
    fd, rng = _raster(150, 170, seed=77)
    m = rng.lognormal(0.0, 1.0, fd.shape).astype(np.float32)
    m[40, 50] = np.inf
    b = (rng.random(fd.shape) * 0.5).astype(np.float32)
    got = _run(lfr, op, fd, m, b, fd.shape)
    walk = _run(lfr, op, fd, m, b, fd.shape, engine="walk", monkeypatch=monkeypatch)
    for g, w in zip(got, walk):
        assert np.array_equal(g, w, equal_nan=True)


def test_repeated_calls_and_clones_give_the_same_bits(lfr):
    import torch
    fd, rng = _raster(700, 600, seed=79, holes=0.001)
    m = lfr.from_numpy(rng.lognormal(0.0, 1.0, fd.shape).astype(np.float32))
    b = lfr.from_numpy((rng.random(fd.shape) * 0.5).astype(np.float32))
    a = lfr.from_numpy(fd)
    first = [lfr.to_numpy(x) for x in lfr.accu_threshold(a, m, b)]
    again = [lfr.to_numpy(x) for x in lfr.accu_threshold(a, m, b)]
    clone = a.topology().clone()
    a._topology, original = clone, a._topology
    cloned = [lfr.to_numpy(x) for x in lfr.accu_threshold(a, m, b)]
    a._topology = original
    clone.close()
    torch.cuda.synchronize()
    for x, y, z in zip(first, again, cloned):
        assert np.array_equal(x, y, equal_nan=True)
        assert np.array_equal(x, z, equal_nan=True)


def test_prepare_builds_the_paths(lfr):
    fd, rng = _raster(300, 300, seed=81)
    m = rng.lognormal(0.0, 1.0, fd.shape).astype(np.float32)
    a = lfr.from_numpy(fd)
    before = a.topology().stats()["device_bytes"]
    a.topology().prepare()
    assert a.topology().stats()["device_bytes"] > before
    out, rem = lfr.accu_threshold(a, lfr.from_numpy(m), 0.25)
    wo, wr = oracle.accu_threshold(fd, m.astype(np.float64), 0.25, fd.shape, dtype=np.float64)
    parity.assert_close32(lfr.to_numpy(out), wo, "outflow after prepare")
    parity.assert_close32(lfr.to_numpy(rem), wr, "remainder after prepare")


@pytest.mark.parametrize("op", OPS)
def test_look_back_scan_on_every_level(lfr, monkeypatch, op):
    """LUE_GB300_PATH_FREE_LONGEST=0 sends every level through the decoupled look-back scan (used on
    levels of long paths), here on a raster of short ones with no-data holes and NaN material."""
    monkeypatch.setenv("LUE_GB300_PATH_FREE_LONGEST", "0")
    fd, rng = _raster(700, 900, seed=83, holes=0.001)
    m = rng.lognormal(0.0, 1.0, fd.shape).astype(np.float32)
    m[rng.random(fd.shape) < 0.001] = np.nan
    b = _other(rng, fd.shape, op)
    got = _run(lfr, op, fd, m, b, (256, 256))
    _, cpu = _ops(lfr, op)
    want = cpu(fd, m.astype(np.float64), b.astype(np.float64), (256, 256), dtype=np.float64)
    for g, w, name in zip(got, want, ("outflow", "remainder")):
        parity.assert_close32(g, w, f"{op} {name}, look-back on every level")


def test_look_back_waits_that_give_up_are_redone_by_the_walk_engine(lfr, monkeypatch):
    """Every wait of the look-back gives up at once (LUE_GB300_PATH_POLLS=0): the kernel sets the redo
    flag, the walk engine redoes the call, and the results are the walk engine's bit for bit."""
    fd, rng = _raster(500, 600, seed=85, holes=0.001)
    m = rng.lognormal(0.0, 1.0, fd.shape).astype(np.float32)
    b = _other(rng, fd.shape, "threshold")
    monkeypatch.setenv("LUE_GB300_PATH_FREE_LONGEST", "0")
    monkeypatch.setenv("LUE_GB300_PATH_POLLS", "0")
    got = _run(lfr, "threshold", fd, m, b, fd.shape)
    monkeypatch.delenv("LUE_GB300_PATH_FREE_LONGEST")
    monkeypatch.delenv("LUE_GB300_PATH_POLLS")
    walk = _run(lfr, "threshold", fd, m, b, fd.shape, engine="walk", monkeypatch=monkeypatch)
    for g, w in zip(got, walk):
        assert np.array_equal(g, w, equal_nan=True)
    again = _run(lfr, "threshold", fd, m, b, fd.shape)  # the next call is a normal one
    for g, w in zip(again, walk):
        parity.assert_close32(g, w.astype(np.float64), "after a call that gave up")
