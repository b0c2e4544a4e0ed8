"""GPU results against the CPU oracle on seeded synthetic rasters and on edge cases.

All calls go through liblue_gb300.so's C ABI (lue_gb300.framework).  Tolerances: tests/parity.py.
"""
import numpy as np
import pytest
import torch

from lue_gb300 import synthetic
from oracle import oracle
from tests import parity

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lfr():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from lue_gb300 import framework
    return framework


@pytest.fixture(scope="module")
def c1():
    """The 1024 x 1024 workload in 256 x 256 partitions: amplitude 50 m, material U[0, 1)."""
    w = synthetic.WORKLOADS["accu_1k"]
    d = synthetic.accu_inputs(w["rows"], w["cols"], w["seed"], w["amplitude"], distribution="uniform",
                              cached=False)
    d["partition"] = w["partition"]
    return d


def ragged(rows, cols, seed, amplitude=30.0):
    fd = synthetic.flow_direction(rows, cols, seed, amplitude, wavelength=max(rows, cols) / 2)
    rng = np.random.default_rng(seed)
    return fd, rng.lognormal(0.0, 1.0, (rows, cols)).astype(np.float32), rng


def test_inflow_count_and_levels_bit_exact(lfr, c1):
    fd = c1["flow_direction"]
    a = lfr.from_numpy(fd, c1["partition"])
    assert np.array_equal(lfr.to_numpy(lfr.inflow_count(a)), oracle.inflow_count(fd, c1["partition"]))
    assert np.array_equal(lfr.to_numpy(lfr.inflow_count(a, value_policies=False)),
                          oracle.inflow_count(fd, c1["partition"], value_policies=False))
    assert np.array_equal(lfr.to_numpy(lfr.downstream_level(a)), oracle.downstream_level(fd))
    s = a.topology().stats()
    v = synthetic.validate(fd)
    assert s["cycle_cells"] == 0 and s["max_level"] + 1 == v["longest_path"]
    assert s["outlet_cells"] == v["edge_outlets"]


def test_accu_f32_against_fp64_oracle(lfr, c1):
    fd, m, ps = c1["flow_direction"], c1["material"], c1["partition"]
    got = lfr.to_numpy(lfr.accu(lfr.from_numpy(fd, ps), lfr.from_numpy(m, ps)))
    want = oracle.accu(fd, m.astype(np.float64), ps, dtype=np.float64)
    parity.assert_close32(got, want, "accu_f32")
    # compensated accumulation is at least as close to float64 as the reference's float32 walk
    ref32 = oracle.accu(fd, m, ps, dtype=np.float32)
    assert parity.rel_error(got, want, parity.FLOOR32)[0] <= parity.rel_error(ref32, want, parity.FLOOR32)[0] + 1e-7


def test_accu_f64_against_fp64_oracle(lfr, c1):
    fd, m, ps = c1["flow_direction"], c1["material"].astype(np.float64), c1["partition"]
    got = lfr.to_numpy(lfr.accu(lfr.from_numpy(fd, ps), lfr.from_numpy(m, ps)))
    parity.assert_close64(got, oracle.accu(fd, m, ps, dtype=np.float64), "accu_f64")


def test_accu_scalar_inflow(lfr, c1):
    fd, ps = c1["flow_direction"], c1["partition"]
    got = lfr.to_numpy(lfr.accu(lfr.from_numpy(fd, ps), 1.0))
    want = oracle.accu(fd, 1.0, ps, dtype=np.float64)
    assert np.array_equal(got, want.astype(np.float32))  # integer counts of upstream cells: exact


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_accu_threshold_and_fraction(lfr, dtype):
    fd, m, rng = ragged(777, 1001, 11)
    thr = (rng.random(fd.shape, dtype=np.float32) * 0.5).astype(np.float32)
    frac = rng.random(fd.shape, dtype=np.float32)
    ps = (256, 300)
    a = lfr.from_numpy(fd, ps)
    check = parity.assert_close32 if dtype == np.float32 else parity.assert_close64
    for fn_gpu, fn_cpu, other in ((lfr.accu_threshold, oracle.accu_threshold, thr),
                                  (lfr.accu_fraction, oracle.accu_fraction, frac)):
        flux, state = fn_gpu(a, lfr.from_numpy(m.astype(dtype), ps), lfr.from_numpy(other.astype(dtype), ps))
        wf, ws = fn_cpu(fd, m.astype(np.float64), other.astype(np.float64), ps, dtype=np.float64)
        check(lfr.to_numpy(flux), wf, fn_gpu.__name__ + " flux")
        check(lfr.to_numpy(state), ws, fn_gpu.__name__ + " state")
    # scalar threshold / fraction overloads
    flux, state = lfr.accu_threshold(a, lfr.from_numpy(m.astype(dtype), ps), dtype(0.25))
    wf, ws = oracle.accu_threshold(fd, m.astype(np.float64), float(dtype(0.25)), ps, dtype=np.float64)
    check(lfr.to_numpy(flux), wf, "threshold scalar")


def kw_inputs(rows, cols, seed):
    d = synthetic.kinematic_wave_inputs(rows, cols, seed, 100.0, cached=False)
    return d


def test_kinematic_wave_float_instantiation_three_steps(lfr):
    """kinematic_wave for F = float: float32 discharge, lateral inflow, alpha (raster), beta and channel
    length (scalars) in, float32 out, against the oracle's float instantiation within the float32
    tolerance, three steps, with a no-data cell and negative lateral inflow (extraction)."""
    d = kw_inputs(512, 640, 6)
    fd, ps = d["flow_direction"].copy(), (128, 160)
    fd[100, 100] = 255
    lat = d["lateral_inflow"].copy()
    lat[::97, ::89] = np.float32(-2e-5)
    q = d["discharge"].astype(np.float32)
    a = lfr.from_numpy(fd, ps)
    lat_d, alpha_d = lfr.from_numpy(lat, ps), lfr.from_numpy(d["alpha"], ps)
    q_gpu = lfr.from_numpy(q, ps)
    q_cpu = q
    for step in range(3):
        q_gpu = lfr.kinematic_wave(a, q_gpu, lat_d, alpha_d, np.float32(0.6), np.float32(3600.0), np.float32(100.0))
        assert q_gpu.dtype == torch.float32
        q_cpu = oracle.kinematic_wave(fd, q_cpu, lat, d["alpha"], np.float32(0.6), np.float32(3600.0),
                                      np.float32(100.0), ps, dtype=np.float32)
        parity.assert_close32(lfr.to_numpy(q_gpu), q_cpu, f"kinematic_wave float step {step}")
        q_cpu = lfr.to_numpy(q_gpu)  # each step from the same inputs


@pytest.mark.parametrize("f32_inputs", [True, False], ids=["f32in", "f64in"])
def test_kinematic_wave_three_steps(lfr, f32_inputs):
    d = kw_inputs(512, 640, 5)
    fd, ps = d["flow_direction"], (128, 160)
    a = lfr.from_numpy(fd, ps)
    lat = d["lateral_inflow"] if f32_inputs else d["lateral_inflow"].astype(np.float64)
    alpha = d["alpha"] if f32_inputs else d["alpha"].astype(np.float64)
    q_gpu = lfr.from_numpy(d["discharge"], ps)
    q_cpu = d["discharge"]
    lat_d, alpha_d = lfr.from_numpy(lat, ps), lfr.from_numpy(alpha, ps)
    for step in range(3):
        q_gpu = lfr.kinematic_wave(a, q_gpu, lat_d, alpha_d, 0.6, 3600.0, 100.0)
        q_cpu = oracle.kinematic_wave(fd, q_cpu, lat.astype(np.float64), alpha.astype(np.float64), 0.6, 3600.0,
                                      100.0, ps, dtype=np.float64)
        parity.assert_close64(lfr.to_numpy(q_gpu), q_cpu, f"kinematic_wave step {step}")


def test_kinematic_wave_raster_beta_and_channel_length(lfr):
    d = kw_inputs(200, 300, 9)
    fd = d["flow_direction"]
    rng = np.random.default_rng(3)
    beta = rng.uniform(0.5, 0.7, fd.shape)
    dx = rng.uniform(50, 150, fd.shape)
    q0 = d["discharge"]
    q0[::17, ::13] = 0.0  # dry cells
    lat = d["lateral_inflow"].astype(np.float64)
    lat[::29, ::31] = 0.0
    got = lfr.kinematic_wave(lfr.from_numpy(fd), lfr.from_numpy(q0), lfr.from_numpy(lat),
                             lfr.from_numpy(d["alpha"].astype(np.float64)), lfr.from_numpy(beta), 900.0,
                             lfr.from_numpy(dx))
    want = oracle.kinematic_wave(fd, q0, lat, d["alpha"].astype(np.float64), beta, 900.0, dx, dtype=np.float64)
    parity.assert_close64(lfr.to_numpy(got), want, "kinematic_wave raster beta/dx")


def test_no_data_propagation(lfr):
    fd, m, rng = ragged(300, 301, 4)
    fd = fd.copy()
    fd[rng.random(fd.shape) < 0.002] = 255  # no-data flow directions (flow into them is undefined:
    m = m.copy()                              # the comparison below is with the oracle on the same input)
    m[rng.random(fd.shape) < 0.003] = np.nan
    m[rng.random(fd.shape) < 0.003] = -1.0  # outside the domain
    a = lfr.from_numpy(fd)
    got = lfr.to_numpy(lfr.accu(a, lfr.from_numpy(m)))
    want = oracle.accu(fd, m.astype(np.float64), dtype=np.float64)
    parity.assert_close32(got, want, "accu with no-data")
    assert np.isnan(got).sum() > 0


def test_all_no_data(lfr):
    fd = np.full((37, 41), 255, np.uint8)
    a = lfr.from_numpy(fd)
    assert (lfr.to_numpy(lfr.inflow_count(a)) == 255).all()
    assert np.isnan(lfr.to_numpy(lfr.accu(a, 1.0))).all()
    assert (lfr.to_numpy(lfr.downstream_level(a)) == -1).all()


def test_cycles_sinks_and_unknown_codes(lfr):
    """Cells on or below a cycle keep the sum of what entered upstream cells pushed into them (the
    reference never enters them); sinks (5) and unknown codes keep their material."""
    rng = np.random.default_rng(2)
    fd = rng.choice(np.array([1, 2, 3, 4, 6, 7, 8, 9, 5, 0, 17], np.uint8), size=(64, 48))
    fd[10, 10], fd[10, 11], fd[11, 11], fd[11, 10] = 6, 2, 4, 8  # 4-cycle
    fd[30, 5], fd[30, 6] = 6, 4  # 2-cycle
    m = rng.random(fd.shape, dtype=np.float32)
    a = lfr.from_numpy(fd)
    assert a.topology().stats()["cycle_cells"] > 0
    got = lfr.to_numpy(lfr.accu(a, lfr.from_numpy(m)))
    want = oracle.accu(fd, m.astype(np.float64), dtype=np.float64)
    parity.assert_close32(got, want, "accu with cycles")
    assert np.array_equal(lfr.to_numpy(lfr.downstream_level(a)), oracle.downstream_level(fd))
    thr = np.float32(0.3)  # the float32 entry point sees 0.3f: give the float64 oracle the same value
    flux, state = lfr.accu_threshold(a, lfr.from_numpy(m), thr)
    wf, ws = oracle.accu_threshold(fd, m.astype(np.float64), float(thr), dtype=np.float64)
    parity.assert_close32(lfr.to_numpy(flux), wf, "threshold with cycles")
    parity.assert_close32(lfr.to_numpy(state), ws, "threshold state with cycles")


@pytest.mark.parametrize("shape", [(1, 1), (1, 257), (263, 1), (3, 2)])
def test_degenerate_shapes(lfr, shape):
    rng = np.random.default_rng(sum(shape))
    fd = rng.choice(np.array([1, 2, 3, 4, 5, 6, 7, 8, 9], np.uint8), size=shape)
    m = rng.random(shape, dtype=np.float32)
    a = lfr.from_numpy(fd)
    parity.assert_close32(lfr.to_numpy(lfr.accu(a, lfr.from_numpy(m))),
                          oracle.accu(fd, m.astype(np.float64), dtype=np.float64), f"accu {shape}")
    assert np.array_equal(lfr.to_numpy(lfr.inflow_count(a)), oracle.inflow_count(fd))


def test_shape_mismatch_is_an_error(lfr):
    from lue_gb300._lib import LueGpuError
    a = lfr.from_numpy(np.full((8, 8), 6, np.uint8), (4, 4))
    with pytest.raises(LueGpuError):
        lfr.accu(a, lfr.from_numpy(np.ones((8, 9), np.float32)))
    with pytest.raises(LueGpuError):
        lfr.accu(a, lfr.from_numpy(np.ones((8, 8), np.float32), (8, 8)))
    with pytest.raises(ValueError):
        lfr.from_numpy(np.ones((8, 8), np.float32), (9, 1))


def test_repeated_calls_are_identical(lfr, c1):
    fd, m, ps = c1["flow_direction"], c1["material"], c1["partition"]
    a = lfr.from_numpy(fd, ps)
    md = lfr.from_numpy(m, ps)
    r1 = lfr.to_numpy(lfr.accu(a, md))
    r2 = lfr.to_numpy(lfr.accu(a, md))
    assert np.array_equal(r1, r2)  # the pull order is fixed: bitwise reproducible


def _accu_with_engine(lfr, a, m, engine):
    import os
    old = os.environ.get("LUE_GB300_ENGINE")
    os.environ["LUE_GB300_ENGINE"] = engine
    try:
        return lfr.to_numpy(lfr.accu(a, m))
    finally:
        if old is None:
            del os.environ["LUE_GB300_ENGINE"]
        else:
            os.environ["LUE_GB300_ENGINE"] = old


def test_tile_engine_against_walk_engine_and_oracle(lfr, c1):
    fd, m, ps = c1["flow_direction"], c1["material"], c1["partition"]
    a = lfr.from_numpy(fd, ps)
    s = a.topology().stats()
    assert s["tile_exits"] > 0 and s["exit_forest_depth"] > 1  # the tile engine is on
    md = lfr.from_numpy(m, ps)
    tiles = _accu_with_engine(lfr, a, md, "tiles")
    walk = _accu_with_engine(lfr, a, md, "walk")
    want = oracle.accu(fd, m.astype(np.float64), ps, dtype=np.float64)
    parity.assert_close32(tiles, want, "accu tiles")
    parity.assert_close32(walk, want, "accu walk")
    parity.assert_close32(tiles, walk, "tiles vs walk")


def test_tile_scan_waits_that_give_up_are_redone_by_the_walk_engine(lfr, c1, monkeypatch):
    """Every look-back wait of the exit-forest scan gives up at once (LUE_GB300_TILE_POLLS=0): the scan
    sets the redo flag, the walk engine redoes the call, and the results are the walk engine's bit for
    bit; the next call is a normal one."""
    fd, m, ps = c1["flow_direction"], c1["material"], c1["partition"]
    a = lfr.from_numpy(fd, ps)
    assert a.topology().stats()["tile_exits"] > 2 * 4096  # several scan chunks: some of them wait
    md = lfr.from_numpy(m, ps)
    normal = lfr.to_numpy(lfr.accu(a, md))
    walk = _accu_with_engine(lfr, a, md, "walk")
    assert not np.array_equal(normal, walk)  # the engines round differently: equality shows the redo
    monkeypatch.setenv("LUE_GB300_TILE_POLLS", "0")
    gave_up = lfr.to_numpy(lfr.accu(a, md))
    monkeypatch.delenv("LUE_GB300_TILE_POLLS")
    assert np.array_equal(gave_up, walk, equal_nan=True)
    assert np.array_equal(lfr.to_numpy(lfr.accu(a, md)), normal)


def test_tile_engine_ragged_with_no_data(lfr):
    fd, m, rng = ragged(777, 1001, 13)
    m = m.copy()
    m[rng.random(fd.shape) < 0.001] = np.nan
    m[rng.random(fd.shape) < 0.001] = -2.0
    fd = fd.copy()
    fd[rng.random(fd.shape) < 0.0005] = 255
    a = lfr.from_numpy(fd, (256, 300))
    assert a.topology().stats()["tile_exits"] > 0
    got = lfr.to_numpy(lfr.accu(a, lfr.from_numpy(m, (256, 300))))
    want = oracle.accu(fd, m.astype(np.float64), (256, 300), dtype=np.float64)
    parity.assert_close32(got, want, "accu tiles ragged with no-data")
    r2 = lfr.to_numpy(lfr.accu(a, lfr.from_numpy(m, (256, 300))))
    assert np.array_equal(got, r2, equal_nan=True)  # exact integer coarse sums: bitwise reproducible


def test_tile_engine_hands_infinite_material_to_the_walk_engine(lfr, c1):
    fd, m, ps = c1["flow_direction"], c1["material"].copy(), c1["partition"]
    m[100, 100] = np.inf
    m[900, 17] = np.inf
    got = lfr.to_numpy(lfr.accu(lfr.from_numpy(fd, ps), lfr.from_numpy(m, ps)))
    want = oracle.accu(fd, m.astype(np.float64), ps, dtype=np.float64)
    assert np.array_equal(np.isinf(got), np.isinf(want))
    finite = np.isfinite(want)
    parity.assert_close32(got[finite], want[finite], "accu with +inf material")


@pytest.mark.parametrize("tiny", [1e-6, 1e-14])
def test_tile_engine_wide_material_range(lfr, c1, tiny):
    """1 % of the cells carry material ~tiny next to U[0, 1) material: 1e-6 stays on the tile engine's
    64-bit fixed point, 1e-14 (a range beyond 2^43 inside a tile) is handed to the walk engine.  Either
    way the small values keep float32 precision."""
    fd, ps = c1["flow_direction"], c1["partition"]
    rng = np.random.default_rng(5)
    m = c1["material"].copy()
    small = rng.random(fd.shape) < 0.01
    m[small] = (tiny * (1.0 + rng.random(int(small.sum())))).astype(np.float32)
    got = lfr.to_numpy(lfr.accu(lfr.from_numpy(fd, ps), lfr.from_numpy(m, ps)))
    want = oracle.accu(fd, m.astype(np.float64), ps, dtype=np.float64)
    parity.assert_close32(got, want, f"accu with material down to {tiny}")
    rel = np.abs(got[small].astype(np.float64) - want[small]) / want[small]
    assert rel.max() <= parity.RTOL32, rel.max()


def test_kinematic_wave_fast_solve_matches_reference_solve(lfr):
    """The float32-Newton + float64-polish solve against the reference-faithful float64 solve."""
    import os
    d = kw_inputs(300, 400, 21)
    fd = d["flow_direction"]
    a = lfr.from_numpy(fd)
    args = (lfr.from_numpy(d["discharge"]), lfr.from_numpy(d["lateral_inflow"]), lfr.from_numpy(d["alpha"]),
            0.6, 3600.0, 100.0)
    fast = lfr.to_numpy(lfr.kinematic_wave(a, *args))
    os.environ["LUE_GB300_KW_SOLVE"] = "reference"
    try:
        ref = lfr.to_numpy(lfr.kinematic_wave(a, *args))
    finally:
        del os.environ["LUE_GB300_KW_SOLVE"]
    mx, _ = parity.rel_error(fast, ref, parity.FLOOR64)
    assert mx <= 1e-11, mx


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
def test_d8_flow_direction_against_oracle(lfr, dtype):
    """A raw fBm DEM (pits kept, so interior sinks appear) with NaN holes, at a ragged size."""
    z = synthetic.dem(517, 1031, seed=8, amplitude=40.0, wavelength=200).astype(dtype)
    rng = np.random.default_rng(8)
    z[rng.random(z.shape) < 0.002] = np.nan
    got = lfr.to_numpy(lfr.d8_flow_direction(lfr.from_numpy(z)))
    assert np.array_equal(got, oracle.d8_flow_direction(z.astype(np.float64) if dtype == np.float64 else z))


@pytest.mark.parametrize("steps", [1, 2, 7, 20])
def test_kinematic_wave_steps_equal_repeated_single_steps(lfr, steps):
    """Many steps in one call (float-float solve, state carried between steps) against one call per
    step (float64 solve, state through float64 rasters): the same roots to about 1e-13, and both within
    the float64 tolerance of the oracle."""
    d = kw_inputs(400, 333, 17)
    fd = d["flow_direction"].copy()
    fd[5, 5] = 255  # a no-data cell
    a = lfr.from_numpy(fd, (100, 111))
    lat, alpha = lfr.from_numpy(d["lateral_inflow"], (100, 111)), lfr.from_numpy(d["alpha"], (100, 111))
    q0 = lfr.from_numpy(d["discharge"], (100, 111))
    multi = lfr.to_numpy(lfr.kinematic_wave_steps(a, q0, lat, alpha, 0.6, 3600.0, 100.0, steps))
    q = q0
    for _ in range(steps):
        q = lfr.kinematic_wave(a, q, lat, alpha, 0.6, 3600.0, 100.0)
    single = lfr.to_numpy(q)
    assert np.array_equal(np.isnan(multi), np.isnan(single))
    mx, _ = parity.rel_error(multi, single, parity.FLOOR64)
    assert mx <= 1e-12, mx
    q_cpu = d["discharge"]
    for _ in range(steps):
        q_cpu = oracle.kinematic_wave(fd, q_cpu, d["lateral_inflow"].astype(np.float64),
                                      d["alpha"].astype(np.float64), 0.6, 3600.0, 100.0, (100, 111), dtype=np.float64)
    parity.assert_close64(multi, q_cpu, f"kinematic_wave_steps {steps}")
