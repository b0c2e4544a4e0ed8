"""The reference's known-answer cases through the C ABI on the GPU.

Same cases and comparison rules as tests/test_oracle_golden.py (which pins the oracle), now run by
liblue_gb300.so via lue_gb300.framework.  float32 cases run the float32 entry points; the
kinematic-wave cases run the float64 entry point (the reference's double instantiation).
"""
import numpy as np
import pytest

from tests.golden import cases as golden
from tests.test_oracle_golden import assert_matches, boost_close

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lfr():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from lue_gb300 import framework
    return framework


def run_case(lfr, c, dtype):
    ps = c["partition_shape"]
    fd = lfr.from_numpy(golden.u8(c["flow_direction"]), ps)
    ins = c["inputs"]

    def arg(name):
        v = golden.arg(ins[name], dtype)
        return lfr.from_numpy(v, ps) if isinstance(v, np.ndarray) else v

    op = c["op"]
    if op == "accu":
        return {"outflow_we_got": lfr.to_numpy(lfr.accu(fd, arg("inflow")))}
    if op in ("accu_threshold", "accu_fraction"):
        fn = lfr.accu_threshold if op == "accu_threshold" else lfr.accu_fraction
        other = "threshold" if op == "accu_threshold" else "fraction"
        flux, state = fn(fd, arg("inflow"), arg(other))
        return {"outflow_we_got": lfr.to_numpy(flux), "residue_we_got": lfr.to_numpy(state)}
    if op in ("accu_capacity", "accu_trigger"):
        fn = getattr(lfr, op)
        out, rem = fn(fd, arg("inflow"), arg("capacity" if op == "accu_capacity" else "trigger"))
        return {"outflow_we_got": lfr.to_numpy(out), "residue_we_got": lfr.to_numpy(rem)}
    if op in ("upstream", "downstream"):
        m = lfr.from_numpy(np.asarray(golden.arg(ins["material"], dtype)), ps)
        return {"material_we_got": lfr.to_numpy(getattr(lfr, op)(fd, m))}
    if op == "kinematic_wave":
        out = lfr.kinematic_wave(fd, *[arg(k) for k in ("current_outflow", "inflow", "alpha", "beta",
                                                          "time_step_duration", "channel_length")])
        return {"outflow_we_got": lfr.to_numpy(out)}
    raise AssertionError(op)


ROUTING = [c for c in golden.load() if c["op"] in ("accu", "accu_threshold", "accu_fraction", "accu_capacity",
                                                   "accu_trigger", "upstream", "downstream")]
KW = golden.load("kinematic_wave")


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
@pytest.mark.parametrize("case", ROUTING, ids=[golden.case_id(c) for c in ROUTING])
def test_routing_case(lfr, case, dtype):
    got = run_case(lfr, case, dtype)
    for name, want in case["expected"].items():
        assert got[name].dtype == dtype
        assert_matches(got[name], golden.f32(want), case["compare"])


@pytest.mark.parametrize("case", KW, ids=[golden.case_id(c) for c in KW])
def test_kinematic_wave_case(lfr, case):
    got = run_case(lfr, case, np.float64)["outflow_we_got"]
    if case["compare"] == "all_positive":
        assert (got > 0).all()
    else:
        assert_matches(got, golden.f32(case["expected"]["outflow_we_got"]), case["compare"])


@pytest.mark.parametrize("case", KW, ids=[golden.case_id(c) for c in KW])
def test_kinematic_wave_case_float_instantiation(lfr, case):
    """The same cases through the float instantiation (every raster float32, float Newton with 14-bit
    stopping): float32 out, within the cases' own relative tolerance of the reference's values."""
    got = run_case(lfr, case, np.float32)["outflow_we_got"]
    assert got.dtype == np.float32
    if case["compare"] == "all_positive":
        assert (got > 0).all()
    else:
        assert_matches(got, golden.f32(case["expected"]["outflow_we_got"]), case["compare"])


COUNTS = golden.load("inflow_count")


@pytest.mark.parametrize("case", COUNTS, ids=[golden.case_id(c) for c in COUNTS])
def test_inflow_count_case(lfr, case):
    fd = lfr.from_numpy(golden.u8(case["flow_direction"]), case["partition_shape"])
    got = lfr.to_numpy(lfr.inflow_count(fd, value_policies=case["no_data_policy"]))
    want = golden.u8(case["expected"]["inflow_count"])
    assert (got == want).all(), f"\n got {got}\n want {want}"


def test_scalar_kw_cases_through_a_one_cell_raster(lfr):
    """iterate_to_new_discharge cases (kinematic_wave_test.cpp:200-313) as 1x1 rasters with the
    upstream discharge fed by a 1x2 raster whose first cell drains east into the second."""
    for c in golden.load("iterate_to_new_discharge"):
        a = c["args"]
        if a["lateral_inflow"] < 0 or a["current_outflow"] < 0:
            continue  # negative lateral inflow is outside the value-policy domain: NaN by design
        fd = lfr.from_numpy(np.array([[5]], np.uint8))
        got = lfr.to_numpy(lfr.kinematic_wave(fd, a["current_outflow"], a["lateral_inflow"], a["alpha"],
                                              a["beta"], a["time_step_duration"], a["channel_length"]))[0, 0]
        if a["upstream_discharge"] == 0:
            assert boost_close(got, c["expected"])


D8_CASES = golden.load("d8_flow_direction")


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
@pytest.mark.parametrize("case", D8_CASES, ids=[f"{golden.case_id(c)}#{i}" for i, c in enumerate(D8_CASES)])
def test_d8_flow_direction_case(lfr, case, dtype):
    z = golden.arg({"raster": case["elevation"]}, dtype)
    got = lfr.to_numpy(lfr.d8_flow_direction(lfr.from_numpy(z)))
    assert (got == np.array(case["expected"]["flow_direction"], np.uint8)).all(), got


DISTANCE = golden.load("downstream_distance")


@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
@pytest.mark.parametrize("case", DISTANCE, ids=[golden.case_id(c) for c in DISTANCE])
def test_downstream_distance_case(lfr, case, dtype):
    import torch
    fd = lfr.from_numpy(golden.u8(case["flow_direction"]), case["partition_shape"])
    got = lfr.to_numpy(lfr.downstream_distance(fd, case["cell_size"],
                                               torch.float32 if dtype == np.float32 else torch.float64))
    assert got.dtype == dtype
    assert_matches(got, golden.f32(case["expected"]["distance"]), "close")


INFO = golden.load("accu_info")


@pytest.mark.parametrize("case", INFO, ids=[golden.case_id(c) for c in INFO])
def test_accu_info_case(lfr, case):
    fd = golden.u8(case["flow_direction"])
    got = lfr.to_numpy(lfr.accu_info(lfr.from_numpy(fd, case["partition_shape"])))
    want = golden.u8(case["expected"]["class_we_got"])
    assert (got == want).all(), f"\n got {got}\n want {want}"
