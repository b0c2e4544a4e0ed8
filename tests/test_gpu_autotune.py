"""The stage engine's schedule (stage cap, threads per stage, steps per progress publication) and its
autotuner (lue_gpu_autotune_stage_schedule): a schedule changes how long a call takes, never its result."""
import ctypes

import numpy as np
import pytest

from lue_gb300 import _lib, synthetic

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


def _threshold_case(lfr, rows=600, cols=700, seed=41):
    fd = synthetic.flow_direction(rows, cols, seed, 40.0, wavelength=max(rows, cols) / 2)
    rng = np.random.default_rng(seed)
    m = rng.lognormal(0.0, 1.0, fd.shape).astype(np.float32)
    thr = (rng.random(fd.shape) * 0.5).astype(np.float32)
    ps = (min(256, rows), min(256, cols))
    return lfr.from_numpy(fd, ps), lfr.from_numpy(m, ps), lfr.from_numpy(thr, ps)


def _kw_case(lfr, rows=500, cols=640, seed=43):
    d = synthetic.kinematic_wave_inputs(rows, cols, seed, amplitude=40.0)
    return (lfr.from_numpy(d["flow_direction"]),) + tuple(
        lfr.from_numpy(d[k]) for k in ("discharge", "lateral_inflow", "alpha"))


def test_schedule_round_trip_and_results_do_not_depend_on_it(lfr):
    fd, m, thr = _threshold_case(lfr)
    t = fd.topology()
    want = [lfr.to_numpy(x) for x in lfr.accu_threshold(fd, m, thr)]
    for cap, threads, publish in ((64, 64, 2), (256, 32, 1), (7, 128, 8), (128, 0, 4)):
        t.set_stage_schedule(cap, threads, publish)
        assert t.stage_schedule() == {"cap": cap, "threads": threads, "publish_every": publish}
        got = [lfr.to_numpy(x) for x in lfr.accu_threshold(fd, m, thr)]
        for g, w in zip(got, want):
            assert np.array_equal(g, w, equal_nan=True), (cap, threads, publish)


def test_kinematic_wave_steps_do_not_depend_on_the_schedule(lfr):
    fd, q, lat, alpha = _kw_case(lfr)
    want = lfr.to_numpy(lfr.kinematic_wave_steps(fd, q, lat, alpha, 0.6, 3600.0, 100.0, 9))
    for cap, threads, publish in ((32, 64, 1), (256, 128, 3), (128, 32, 8)):
        fd.topology().set_stage_schedule(cap, threads, publish)
        got = lfr.to_numpy(lfr.kinematic_wave_steps(fd, q, lat, alpha, 0.6, 3600.0, 100.0, 9))
        assert np.array_equal(got, want, equal_nan=True), (cap, threads, publish)


def test_stage_order_round_trip_and_results_do_not_depend_on_it(lfr):
    """Both ticket orders (latest start, the default; earliest start, for servers) give the same bits for
    a one-step and a multi-step kinematic wave and for accu_threshold; another order is refused while
    clones share the stage structures, and a bad order is refused."""
    fd, q, lat, alpha = _kw_case(lfr)
    t = fd.topology()
    assert t.stage_order() == "latest"
    want1 = lfr.to_numpy(lfr.kinematic_wave(fd, q, lat, alpha, 0.6, 3600.0, 100.0))
    want9 = lfr.to_numpy(lfr.kinematic_wave_steps(fd, q, lat, alpha, 0.6, 3600.0, 100.0, 9))
    t.set_stage_order("earliest")
    assert t.stage_order() == "earliest"
    assert np.array_equal(lfr.to_numpy(lfr.kinematic_wave(fd, q, lat, alpha, 0.6, 3600.0, 100.0)), want1,
                          equal_nan=True)
    assert np.array_equal(lfr.to_numpy(lfr.kinematic_wave_steps(fd, q, lat, alpha, 0.6, 3600.0, 100.0, 9)), want9,
                          equal_nan=True)
    c = t.clone()
    with pytest.raises(_lib.LueGpuError) as e:
        t.set_stage_order("latest")
    assert "clone" in str(e.value)
    c.close()
    with pytest.raises(_lib.LueGpuError) as e:
        _lib.check(_lib.lib().lue_gpu_topology_set_stage_order(t.handle, 7))
    assert e.value.status == 1
    t.set_stage_order("latest")
    fdt, m, thr = _threshold_case(lfr, 300, 350, 9)
    a = [lfr.to_numpy(x) for x in lfr.accu_threshold(fdt, m, thr)]
    fdt.topology().set_stage_order("earliest")
    b = [lfr.to_numpy(x) for x in lfr.accu_threshold(fdt, m, thr)]
    for x, y in zip(a, b):
        assert np.array_equal(x, y, equal_nan=True)


def test_bad_schedules_and_cap_changes_under_clones_are_refused(lfr):
    fd, m, thr = _threshold_case(lfr, 200, 300, 5)
    t = fd.topology()
    for bad in ((300, 0, 0), (-1, 0, 0), (0, 48, 0), (0, 0, -2)):
        with pytest.raises(_lib.LueGpuError) as e:
            t.set_stage_schedule(*bad)
        assert e.value.status == 1
    t.set_stage_schedule(64, 0, 0)
    c = t.clone()
    with pytest.raises(_lib.LueGpuError) as e:
        t.set_stage_schedule(128, 0, 0)
    assert "clone" in str(e.value)
    c.set_stage_schedule(0, 64, 2)  # the handle's own launch parameters stay free
    assert c.stage_schedule() == {"cap": 64, "threads": 64, "publish_every": 2}
    c.close()
    t.set_stage_schedule(128, 0, 0)
    assert t.stage_schedule()["cap"] == 128


@pytest.mark.parametrize("op", ["accu_threshold", "kinematic_wave_steps"])
def test_autotune_keeps_the_fastest_schedule_and_the_results(lfr, op):
    if op == "accu_threshold":
        fd, m, thr = _threshold_case(lfr, 700, 800, 47)
        want = [lfr.to_numpy(x) for x in lfr.accu_threshold(fd, m, thr)]
        box = {}

        def call():
            box["out"] = lfr.accu_threshold(fd, m, thr)
    else:
        fd, q, lat, alpha = _kw_case(lfr, 600, 600, 49)
        want = [lfr.to_numpy(lfr.kinematic_wave_steps(fd, q, lat, alpha, 0.6, 3600.0, 100.0, 12))]
        box = {}

        def call():
            box["out"] = (lfr.kinematic_wave_steps(fd, q, lat, alpha, 0.6, 3600.0, 100.0, 12),)
    best = lfr.autotune_stage_schedule(fd, call, repeats=2)
    assert best["cap"] in (64, 128, 256)
    assert best["threads"] in (0, 32, 64, 128)  # 0: by the largest stage, when no fixed size was faster
    assert best["publish_every"] in (1, 2, 4, 8)
    assert best["ms"] > 0
    assert fd.topology().stage_schedule() == {k: best[k] for k in ("cap", "threads", "publish_every")}
    for g, w in zip(box["out"], want):  # the last run of the call, with some candidate schedule
        assert np.array_equal(lfr.to_numpy(g), w, equal_nan=True)
    call()  # with the chosen schedule
    for g, w in zip(box["out"], want):
        assert np.array_equal(lfr.to_numpy(g), w, equal_nan=True)


def test_autotune_stops_at_a_failing_call_and_keeps_the_schedule(lfr):
    import torch
    fd, m, thr = _threshold_case(lfr, 200, 300, 7)
    t = fd.topology()
    t.set_stage_schedule(64, 64, 2)
    L = _lib.lib()

    def failing():  # NULL outputs: the routing call returns LUE_GPU_EINVAL
        _lib.check(L.lue_gpu_accu_threshold_f32(t.handle, m.data.data_ptr(), 0.0, thr.data.data_ptr(), 0.0, None,
                                                None, torch.cuda.current_stream().cuda_stream))
    with pytest.raises(_lib.LueGpuError) as e:
        lfr.autotune_stage_schedule(fd, failing)
    assert e.value.status == 1 and "NULL output" in str(e.value)
    assert t.stage_schedule() == {"cap": 64, "threads": 64, "publish_every": 2}

    def raising():
        raise KeyError("not a routing error")
    with pytest.raises(KeyError):
        lfr.autotune_stage_schedule(fd, raising)
    assert t.stage_schedule() == {"cap": 64, "threads": 64, "publish_every": 2}
    s = _lib.StageSchedule()
    cb = _lib.STAGE_CALL(lambda handle, user, stream: 0)
    assert L.lue_gpu_autotune_stage_schedule(t.handle, cb, None, 0, None, ctypes.byref(s)) == 1
