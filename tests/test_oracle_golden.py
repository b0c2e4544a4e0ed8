"""Pin the CPU oracle to the reference's own known-answer tests.

Every case in tests/golden/reference_cases.json was extracted from the reference's Boost.Test sources
(source/framework/algorithm/test/{accu,accu_threshold,accu_fraction,accu_capacity,accu_trigger,
kinematic_wave,inflow_count,upstream,downstream,downstream_distance,d8_flow_direction,accu_info}_test.cpp)
by tests/golden/extract_reference_cases.py.  The comparison rules restate the reference's
test helpers (source/framework/test/include/lue/framework/test/compare.hpp):

- ``check_arrays_are_equal``: element-wise equality, NaN == NaN (compare.hpp:52-100);
- ``check_arrays_are_close``: Boost ``tt::tolerance(1e-6)``, a relative tolerance that must hold with
  respect to both operands; when one operand is exactly zero the other must be smaller than the
  tolerance in absolute value (compare.hpp:102-116, 210-219).
"""
import math

import numpy as np
import pytest

from oracle import oracle
from tests.golden import cases as golden


def boost_close(a, b, tol=1e-6):
    if math.isnan(a) or math.isnan(b):
        return math.isnan(a) and math.isnan(b)
    if a == 0.0 or b == 0.0:
        return abs(a if b == 0.0 else b) <= tol
    d = abs(a - b)
    return d <= tol * abs(a) and d <= tol * abs(b)


def assert_matches(got, want, how, tol=1e-6):
    got = np.asarray(got, dtype=np.float64)
    want = np.asarray(want, dtype=np.float64)
    assert got.shape == want.shape
    if how == "equal":
        same = (got == want) | (np.isnan(got) & np.isnan(want))
        assert same.all(), f"differ at {np.argwhere(~same)[:5].tolist()}:\n got {got}\n want {want}"
    else:
        bad = [(i, j) for i in range(got.shape[0]) for j in range(got.shape[1])
               if not boost_close(got[i, j], want[i, j], tol)]
        assert not bad, f"not close at {bad[:5]}:\n got {got}\n want {want}"


def run_case(c, dtype):
    fd = golden.u8(c["flow_direction"])
    ps = c["partition_shape"]
    ins = c["inputs"]
    op = c["op"]
    if op == "accu":
        return {"outflow_we_got": oracle.accu(fd, golden.arg(ins["inflow"], dtype), ps, dtype)}
    if op == "accu_threshold":
        flux, state = oracle.accu_threshold(fd, golden.arg(ins["inflow"], dtype),
                                            golden.arg(ins["threshold"], dtype), ps, dtype)
        return {"outflow_we_got": flux, "residue_we_got": state}
    if op == "accu_fraction":
        flux, state = oracle.accu_fraction(fd, golden.arg(ins["inflow"], dtype),
                                           golden.arg(ins["fraction"], dtype), ps, dtype)
        return {"outflow_we_got": flux, "residue_we_got": state}
    if op in ("accu_capacity", "accu_trigger"):
        other = "capacity" if op == "accu_capacity" else "trigger"
        out, rem = getattr(oracle, op)(fd, golden.arg(ins["inflow"], dtype), golden.arg(ins[other], dtype), ps,
                                       dtype)
        return {"outflow_we_got": out, "residue_we_got": rem}
    if op in ("upstream", "downstream"):
        return {"material_we_got": getattr(oracle, op)(fd, golden.arg(ins["material"], dtype), dtype)}
    if op == "kinematic_wave":
        a = [golden.arg(ins[k], dtype) for k in ("current_outflow", "inflow", "alpha", "beta",
                                                  "time_step_duration", "channel_length")]
        return {"outflow_we_got": oracle.kinematic_wave(fd, *a, partition_shape=ps, dtype=dtype)}
    raise AssertionError(op)


ROUTING = [c for c in golden.load() if c["op"] in ("accu", "accu_threshold", "accu_fraction", "kinematic_wave",
                                                   "accu_capacity", "accu_trigger", "upstream", "downstream")]


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
@pytest.mark.parametrize("case", ROUTING, ids=[golden.case_id(c) for c in ROUTING])
def test_routing_case(case, dtype):
    got = run_case(case, dtype)
    if case["compare"] == "all_positive":
        assert (got["outflow_we_got"] > 0).all()
        return
    for name, want in case["expected"].items():
        assert_matches(got[name], golden.f32(want), case["compare"])


COUNTS = golden.load("inflow_count")


@pytest.mark.parametrize("case", COUNTS, ids=[golden.case_id(c) for c in COUNTS])
def test_inflow_count_case(case):
    fd = golden.u8(case["flow_direction"])
    got = oracle.inflow_count(fd, case["partition_shape"], value_policies=case["no_data_policy"])
    want = golden.u8(case["expected"]["inflow_count"])
    assert (got == want).all(), f"\n got {got}\n want {want}"


SCALAR = golden.load("iterate_to_new_discharge")


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
@pytest.mark.parametrize("case", SCALAR, ids=[f"{golden.case_id(c)}#{i}" for i, c in enumerate(SCALAR)])
def test_iterate_to_new_discharge(case, dtype):
    a = case["args"]
    got = oracle.iterate_to_new_discharge(a["upstream_discharge"], a["current_outflow"], a["lateral_inflow"],
                                          a["alpha"], a["beta"], a["time_step_duration"], a["channel_length"],
                                          dtype=dtype)
    assert boost_close(got, case["expected"])
    assert got >= 0


def test_partitioning_does_not_change_accu_of_ones():
    """Same raster in one partition and in 3x3 partitions: identical counts and integer-valued sums."""
    c = [c for c in ROUTING if c["name"] == "spiral_in_case" and c["op"] == "accu"][0]
    fd = golden.u8(c["flow_direction"])
    one = oracle.accu(fd, 1.0, None)
    many = oracle.accu(fd, 1.0, (3, 3))
    assert (one == many).all()


def test_threaded_oracle_matches_single_threaded():
    rng = np.random.default_rng(7)
    c = [c for c in ROUTING if c["name"] == "merging_streams_case_01" and c["op"] == "accu"][0]
    fd = golden.u8(c["flow_direction"])
    ext = rng.random(fd.shape, dtype=np.float32)
    a = oracle.accu(fd, ext, (3, 3), nthreads=1)
    b = oracle.accu(fd, ext, (3, 3), nthreads=4)
    np.testing.assert_allclose(a, b, rtol=1e-6, equal_nan=True)


D8_CASES = golden.load("d8_flow_direction")


@pytest.mark.parametrize("case", D8_CASES, ids=[f"{golden.case_id(c)}#{i}" for i, c in enumerate(D8_CASES)])
def test_d8_flow_direction_case(case):
    z = golden.arg({"raster": case["elevation"]}, np.float32)
    got = oracle.d8_flow_direction(z)
    assert (got == np.array(case["expected"]["flow_direction"], np.uint8)).all(), got


DISTANCE = golden.load("downstream_distance")


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
@pytest.mark.parametrize("case", DISTANCE, ids=[golden.case_id(c) for c in DISTANCE])
def test_downstream_distance_case(case, dtype):
    got = oracle.downstream_distance(golden.u8(case["flow_direction"]), case["cell_size"], dtype)
    assert_matches(got, golden.f32(case["expected"]["distance"]), "close")


INFO = golden.load("accu_info")


@pytest.mark.parametrize("case", INFO, ids=[golden.case_id(c) for c in INFO])
def test_accu_info_case(case):
    got = oracle.accu_info(golden.u8(case["flow_direction"]), case["partition_shape"])
    want = golden.u8(case["expected"]["class_we_got"])
    assert (got == want).all(), f"\n got {got}\n want {want}"


def test_fixture_is_what_the_extractor_reads_from_the_reference_sources(tmp_path):
    """tests/golden/reference_cases.json is exactly what tests/golden/extract_reference_cases.py writes from
    the reference's test sources, where LUE_REFERENCE names their root (the fixture travels without them)."""
    import json
    import os
    import subprocess
    import sys

    from tests.golden import extract_reference_cases as extract
    ref = extract.DEFAULT_REFERENCE
    if not ref or not os.path.isdir(os.path.join(ref, extract.TEST_DIR)):
        pytest.skip("reference sources not given (LUE_REFERENCE)")
    here = os.path.dirname(os.path.abspath(__file__))
    out = tmp_path / "cases.json"
    subprocess.run([sys.executable, os.path.join(here, "golden", "extract_reference_cases.py"), "--reference", ref,
                    "--out", str(out)], check=True, capture_output=True)
    with open(out) as fh:
        fresh = json.load(fh)
    with open(os.path.join(here, "golden", "reference_cases.json")) as fh:
        committed = json.load(fh)
    assert fresh == committed
