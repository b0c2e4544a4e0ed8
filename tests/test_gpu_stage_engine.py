"""The stage engine (accu_threshold, accu_fraction, float64 accu and kinematic_wave on acyclic rasters)
against the walk engine and the oracle.

The stage engine applies the same cell rules with the same float-float (float32) or float64 upstream
sums, in the same neighbour order, as the walk engine, so one-step results agree bit for bit.  The
multi-step kinematic wave uses a float-float solve; it is checked against the float64 oracle.  Results
do not depend on the largest stage (LUE_GB300_STAGE_CAP, read when a topology builds its stages): only
where an upstream outflow is read from changes.  LUE_GB300_ENGINE=walk selects the walk engine for a call.
"""
import os

import numpy as np
import pytest

from lue_gb300 import synthetic
from oracle import oracle
from tests import parity

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _stage_engine(monkeypatch):
    """accu_threshold and accu_capacity (float32) run on the path engine by default; these tests are about
    the stage engine."""
    monkeypatch.setenv("LUE_GB300_ENGINE", "stage")


@pytest.fixture(scope="module")
def lfr():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from lue_gb300 import framework
    return framework


class _env:
    def __init__(self, **kv):
        self.kv = kv

    def __enter__(self):
        self.old = {k: os.environ.get(k) for k in self.kv}
        os.environ.update(self.kv)

    def __exit__(self, *exc):
        for k, v in self.old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def _raster(rows, cols, seed, amplitude=40.0, holes=0.0):
    fd = synthetic.flow_direction(rows, cols, seed, amplitude, wavelength=max(rows, cols) / 2).copy()
    rng = np.random.default_rng(seed)
    if holes:
        fd[rng.random(fd.shape) < holes] = 255
    return fd, rng


@pytest.mark.parametrize("shape", [(1024, 1024), (333, 777), (65, 31), (1, 300)])
@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_threshold_and_fraction_equal_walk_engine(lfr, shape, dtype):
    fd, rng = _raster(*shape, seed=31, holes=0.001)
    m = rng.lognormal(0.0, 1.0, shape).astype(dtype)
    m[rng.random(shape) < 0.001] = np.nan
    m[rng.random(shape) < 0.001] = -1.0
    thr = (rng.random(shape) * 0.5).astype(dtype)
    frac = rng.random(shape).astype(dtype)
    ps = (min(256, shape[0]), min(256, shape[1]))
    a = lfr.from_numpy(fd, ps)
    md, td, fdd = lfr.from_numpy(m, ps), lfr.from_numpy(thr, ps), lfr.from_numpy(frac, ps)
    for op, b, name in ((lfr.accu_threshold, td, "threshold"), (lfr.accu_fraction, fdd, "fraction")):
        stage = [lfr.to_numpy(x) for x in op(a, md, b)]
        with _env(LUE_GB300_ENGINE="walk"):
            walk = [lfr.to_numpy(x) for x in op(a, md, b)]
        for s_, w_ in zip(stage, walk):
            assert np.array_equal(s_, w_, equal_nan=True), name
        ref = getattr(oracle, "accu_" + name)(fd, m.astype(np.float64), (thr if name == "threshold" else frac)
                                              .astype(np.float64), ps, dtype=np.float64)
        check = parity.assert_close32 if dtype == np.float32 else parity.assert_close64
        check(stage[0], ref[0], f"{name} flux")
        check(stage[1], ref[1], f"{name} state")


def test_accu_f64_equals_walk_engine(lfr):
    fd, rng = _raster(700, 900, seed=5, holes=0.0005)
    m = rng.random(fd.shape)
    a = lfr.from_numpy(fd)
    md = lfr.from_numpy(m)
    stage = lfr.to_numpy(lfr.accu(a, md))
    with _env(LUE_GB300_ENGINE="walk"):
        walk = lfr.to_numpy(lfr.accu(a, md))
    assert np.array_equal(stage, walk, equal_nan=True)
    parity.assert_close64(stage, oracle.accu(fd, m, (700, 900), dtype=np.float64), "accu f64")


def _kw(rows, cols, seed):
    d = synthetic.kinematic_wave_inputs(rows, cols, seed, amplitude=40.0)
    return d


def test_kinematic_wave_single_step_against_walk_engine(lfr):
    """float32 lateral inflow and alpha with beta = 3/5: the stage engine's float-float solve in
    y = Q^(1/5) against the walk engine's float64 solve (~1e-13); float64 rasters: the same float64 solve
    on both engines, bit for bit."""
    d = _kw(300, 500, 9)
    fd = d["flow_direction"].copy()
    fd[7, 11] = 255
    a = lfr.from_numpy(fd)
    for lat, alpha, exact in ((d["lateral_inflow"], d["alpha"], False),
                              (d["lateral_inflow"].astype(np.float64), d["alpha"].astype(np.float64), True)):
        args = (lfr.from_numpy(d["discharge"]), lfr.from_numpy(lat), lfr.from_numpy(alpha), 0.6, 3600.0, 100.0)
        stage = lfr.to_numpy(lfr.kinematic_wave(a, *args))
        with _env(LUE_GB300_ENGINE="walk"):
            walk = lfr.to_numpy(lfr.kinematic_wave(a, *args))
        if exact:
            assert np.array_equal(stage, walk, equal_nan=True)
        else:
            assert np.array_equal(np.isnan(stage), np.isnan(walk))
            assert parity.rel_error(stage, walk, parity.FLOOR64)[0] <= 1e-12
        want = oracle.kinematic_wave(fd, d["discharge"], lat.astype(np.float64), alpha.astype(np.float64), 0.6,
                                     3600.0, 100.0, fd.shape, dtype=np.float64)
        parity.assert_close64(stage, want, "kinematic_wave one step")


@pytest.mark.parametrize("cap", ["1", "7", "64", "256"])
def test_kinematic_wave_steps_stage_caps(lfr, cap):
    """Stages of at most 1, 7, 64 or 256 cells give the oracle's discharge after 12 steps."""
    d = _kw(257, 390, 4)
    fd = d["flow_direction"]
    a = lfr.from_numpy(fd)
    lat, alpha, q0 = (lfr.from_numpy(d[k]) for k in ("lateral_inflow", "alpha", "discharge"))
    with _env(LUE_GB300_STAGE_CAP=cap):
        got = lfr.to_numpy(lfr.kinematic_wave_steps(a, q0, lat, alpha, 0.6, 3600.0, 100.0, 12))
    q = d["discharge"]
    for _ in range(12):
        q = oracle.kinematic_wave(fd, q, d["lateral_inflow"].astype(np.float64), d["alpha"].astype(np.float64),
                                  0.6, 3600.0, 100.0, fd.shape, dtype=np.float64)
    parity.assert_close64(got, q, f"kinematic_wave_steps, stages of at most {cap} cells")


def test_kinematic_wave_steps_zero_and_no_data(lfr):
    """Cells without water, cells whose discharge starts at 0 (the reference's DBL_MIN start), NaN
    lateral inflow and no-data flow directions."""
    d = _kw(200, 260, 12)
    fd = d["flow_direction"].copy()
    rng = np.random.default_rng(3)
    fd[rng.random(fd.shape) < 0.002] = 255
    q0 = d["discharge"].copy()
    q0[rng.random(fd.shape) < 0.05] = 0.0
    lat = d["lateral_inflow"].copy()
    lat[rng.random(fd.shape) < 0.05] = 0.0
    lat[rng.random(fd.shape) < 0.001] = np.nan
    a = lfr.from_numpy(fd)
    got = lfr.to_numpy(lfr.kinematic_wave_steps(a, lfr.from_numpy(q0), lfr.from_numpy(lat),
                                                lfr.from_numpy(d["alpha"]), 0.6, 3600.0, 100.0, 9))
    q = q0
    for _ in range(9):
        q = oracle.kinematic_wave(fd, q, lat.astype(np.float64), d["alpha"].astype(np.float64), 0.6, 3600.0, 100.0,
                                  fd.shape, dtype=np.float64)
    parity.assert_close64(got, q, "kinematic_wave_steps with zeros and no-data")


@pytest.mark.parametrize("shape", [(1024, 1024), (333, 777), (1, 300)])
@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_capacity_and_trigger_equal_walk_engine(lfr, shape, dtype):
    fd, rng = _raster(*shape, seed=41, holes=0.001)
    m = rng.lognormal(0.0, 1.0, shape).astype(dtype)
    m[rng.random(shape) < 0.001] = np.nan
    m[rng.random(shape) < 0.001] = -1.0
    limit = (rng.random(shape) * 20.0).astype(dtype)
    ps = (min(256, shape[0]), min(256, shape[1]))
    a = lfr.from_numpy(fd, ps)
    md, ld = lfr.from_numpy(m, ps), lfr.from_numpy(limit, ps)
    for name in ("accu_capacity", "accu_trigger"):
        op = getattr(lfr, name)
        stage = [lfr.to_numpy(x) for x in op(a, md, ld)]
        with _env(LUE_GB300_ENGINE="walk"):
            walk = [lfr.to_numpy(x) for x in op(a, md, ld)]
        for s_, w_ in zip(stage, walk):
            assert np.array_equal(s_, w_, equal_nan=True), name
        ref = getattr(oracle, name)(fd, m.astype(np.float64), limit.astype(np.float64), ps, dtype=np.float64)
        check = parity.assert_close32 if dtype == np.float32 else parity.assert_close64
        check(stage[0], ref[0], f"{name} outflow")
        check(stage[1], ref[1], f"{name} remainder")


@pytest.mark.parametrize("shape", [(517, 1031), (64, 32), (1, 77), (77, 1)])
@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_upstream_downstream_distance_against_oracle(lfr, shape, dtype):
    import torch
    fd, rng = _raster(*shape, seed=19, holes=0.01)
    fd = fd.copy()
    fd[rng.random(shape) < 0.005] = 5       # sinks
    m = rng.random(shape).astype(dtype)
    m[rng.random(shape) < 0.01] = np.nan
    a = lfr.from_numpy(fd)
    md = lfr.from_numpy(m)
    assert np.array_equal(lfr.to_numpy(lfr.upstream(a, md)), oracle.upstream(fd, m, dtype), equal_nan=True)
    assert np.array_equal(lfr.to_numpy(lfr.downstream(a, md)), oracle.downstream(fd, m, dtype), equal_nan=True)
    tdt = torch.float32 if dtype == np.float32 else torch.float64
    got = lfr.to_numpy(lfr.downstream_distance(a, 2.5, tdt))
    assert np.array_equal(got, oracle.downstream_distance(fd, 2.5, dtype), equal_nan=True)


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_results_do_not_depend_on_the_stage_cap(lfr, dtype):
    """Stages of at most 1, 32, 128 (default) or 256 cells: the same cells, rules and sums in the same
    neighbour order, so the same bits."""
    fd, rng = _raster(1536, 700, seed=77, holes=0.0005)
    m = rng.lognormal(0.0, 1.0, fd.shape).astype(dtype)
    thr = (rng.random(fd.shape) * 0.5).astype(dtype)
    ps = (512, 350)
    md, td = lfr.from_numpy(m, ps), lfr.from_numpy(thr, ps)
    results = {}
    for cap in ("1", "32", "128", "256"):
        with _env(LUE_GB300_STAGE_CAP=cap):
            a = lfr.from_numpy(fd, ps)
            results[cap] = [lfr.to_numpy(x) for op in (lfr.accu_threshold, lfr.accu_capacity) for x in op(a, md, td)]
    for cap, got in results.items():
        for g, w in zip(got, results["128"]):
            assert np.array_equal(g, w, equal_nan=True), cap


def test_kinematic_wave_steps_do_not_depend_on_the_stage_cap(lfr):
    d = _kw(700, 900, 21)
    args = tuple(lfr.from_numpy(d[k]) for k in ("discharge", "lateral_inflow", "alpha")) + (0.6, 3600.0, 100.0, 17)
    results = {}
    for cap in ("16", "128", "256"):
        with _env(LUE_GB300_STAGE_CAP=cap):
            a = lfr.from_numpy(d["flow_direction"])
            results[cap] = lfr.to_numpy(lfr.kinematic_wave_steps(a, *args))
    for cap, got in results.items():
        assert np.array_equal(got, results["128"], equal_nan=True), cap


def test_dataflow_wait_that_gives_up_is_reported(lfr):
    """A stage whose first wait can never end (LUE_GB300_FLOW_STUCK_STAGE: it waits for a step of its own
    that it has not published) gives up after a bounded number of polls: every output of the call is NaN,
    the next call on the topology returns LUE_GPU_ETIMEDOUT, and the call after that is valid again."""
    import torch
    from lue_gb300 import _lib
    fd, rng = _raster(512, 512, seed=3)
    m = rng.random(fd.shape).astype(np.float32)
    thr = np.full(fd.shape, 0.1, np.float32)
    a = lfr.from_numpy(fd)
    md, td = lfr.from_numpy(m), lfr.from_numpy(thr)
    want = [lfr.to_numpy(x) for x in lfr.accu_threshold(a, md, td)]
    with _env(LUE_GB300_FLOW_STUCK_STAGE="0"):
        bad = [lfr.to_numpy(x) for x in lfr.accu_threshold(a, md, td)]
    torch.cuda.synchronize()
    assert all(np.isnan(x).all() for x in bad)
    with pytest.raises(_lib.LueGpuError) as e:
        lfr.accu_threshold(a, md, td)
    assert e.value.status == 5
    again = [lfr.to_numpy(x) for x in lfr.accu_threshold(a, md, td)]
    for g, w in zip(again, want):
        assert np.array_equal(g, w, equal_nan=True)
