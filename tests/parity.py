"""Error metrics shared by the parity tests and bench.py.

Tolerances (stated once, used everywhere):

- integer outputs (inflow counts, downstream levels): bit-exact;
- float32 accumulation (accu, accu_threshold, accu_fraction): max relative error <= 1e-5 against the
  float64 oracle, with relative error |gpu - oracle| / max(|oracle|, FLOOR32) and FLOOR32 = 1e-3
  (material is O(1) per cell, so the floor only matters for values that are essentially zero);
- float64 discharge (kinematic_wave): max relative error <= 1e-9 against the float64 oracle, floor 1e-12;
- NaN (no-data) positions identical.
"""
import numpy as np

RTOL32 = 1e-5
FLOOR32 = 1e-3
RTOL64 = 1e-9
FLOOR64 = 1e-12


def rel_error(got, want, floor):
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    nan_g, nan_w = np.isnan(got), np.isnan(want)
    if not np.array_equal(nan_g, nan_w):
        bad = np.argwhere(nan_g != nan_w)
        raise AssertionError(f"no-data positions differ at {bad[:5].tolist()} ({len(bad)} cells)")
    ok = ~nan_w
    if not ok.any():
        return 0.0, 0.0
    err = np.abs(got[ok] - want[ok]) / np.maximum(np.abs(want[ok]), floor)
    return float(err.max()), float(err.mean())


def assert_close32(got, want, what=""):
    mx, mean = rel_error(got, want, FLOOR32)
    assert mx <= RTOL32, f"{what}: max relative error {mx:.3e} > {RTOL32} (mean {mean:.3e})"
    return mx, mean


def assert_close64(got, want, what=""):
    mx, mean = rel_error(got, want, FLOOR64)
    assert mx <= RTOL64, f"{what}: max relative error {mx:.3e} > {RTOL64} (mean {mean:.3e})"
    return mx, mean
