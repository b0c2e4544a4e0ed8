"""The C++ mirror of lue::value_policies (lue_gb300/csrc/lue_gb300.hpp) on two of the reference's
known-answer cases, through a compiled example program (lue_gb300/examples/accu_example.cpp)."""
import subprocess

import numpy as np
import pytest

from tests.golden import cases as golden

pytestmark = pytest.mark.gpu


def test_cpp_mirror_known_answers():
    from lue_gb300 import _build
    exe = _build.cpp_example()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.strip().splitlines()
    accu = np.array([float(v) for v in lines[0].split()], np.float32).reshape(6, 5)
    want = [c for c in golden.load("accu") if c["name"] == "back_and_forth"][0]["expected"]["outflow_we_got"]
    assert np.array_equal(accu, golden.f32(want))
    case = [c for c in golden.load("accu_threshold") if c["name"] == "pcraster_manual_example1"][0]
    flux = np.array([float(v) for v in lines[1].split()], np.float32).reshape(5, 5)
    state = np.array([float(v) for v in lines[2].split()], np.float32).reshape(5, 5)
    assert np.array_equal(flux, golden.f32(case["expected"]["outflow_we_got"]))
    assert np.array_equal(state, golden.f32(case["expected"]["residue_we_got"]))
    # accu_capacity / accu_trigger against the reference's pcraster manual example 1 of each
    rows = [np.array([float(v) for v in lines[k].split()], np.float32).reshape(5, 5) for k in range(3, 10)]
    for op, (o, r) in (("accu_capacity", rows[0:2]), ("accu_trigger", rows[2:4])):
        case = [c for c in golden.load(op) if c["name"] == "pcraster_manual_example1"][0]
        assert np.array_equal(o, golden.f32(case["expected"]["outflow_we_got"])), op
        assert np.array_equal(r, golden.f32(case["expected"]["residue_we_got"])), op
    # upstream / downstream / downstream_distance against the oracle on the same rasters
    from oracle import oracle
    fd = golden.u8(case["flow_direction"])
    inflow = golden.f32(case["inputs"]["inflow"]["raster"]).astype(np.float32)
    assert np.array_equal(rows[4], oracle.upstream(fd, inflow, np.float32))
    assert np.array_equal(rows[5], oracle.downstream(fd, inflow, np.float32))
    # printed with %g: six significant digits
    np.testing.assert_allclose(rows[6], oracle.downstream_distance(fd, 2.0, np.float32), rtol=1e-5)
    assert lines[10] == "shape mismatch rejected"
    # accu_threshold again after the stage schedule was autotuned for it: the same flux
    assert lines[11].split() == lines[1].split()
    assert lines[12].startswith("schedule cap ")
    # partial_accu on back_and_forth against the oracle (one partition row per 3 rows: one inter-partition
    # hand-off per column, no order dependence)
    bf = [c for c in golden.load("accu") if c["name"] == "back_and_forth"][0]
    fd_bf = golden.u8(bf["flow_direction"])
    partial = np.array([float(v) for v in lines[13].split()]).reshape(6, 5)
    assert np.array_equal(partial, oracle.partial_accu(fd_bf, 1000, (3, 5)), equal_nan=True)
    # kinematic_wave<float> against the oracle's float instantiation
    q1 = np.array([float(v) for v in lines[14].split()], np.float32).reshape(5, 5)
    want = oracle.kinematic_wave(fd, inflow / np.float32(10), inflow / np.float32(1000), np.float32(1.5),
                                 np.float32(0.6), np.float32(15.0), np.float32(10.0), (5, 5), dtype=np.float32)
    from tests import parity
    parity.assert_close32(q1, want, "kinematic_wave<float>")
