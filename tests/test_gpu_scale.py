"""Parity at the sizes the benchmark numbers are quoted on.

- kw_8k (8192 x 8192, float64 discharge, float32 rain and alpha, beta 0.6, dt 3600 s, dx 100 m): rows
  0-2047 (2048 x 8192 cells; flow leaving the band is dropped, as at the array edge) routed 100 steps in
  one kinematic_wave_steps call (stage engine, float-float solve carried between steps along paths of
  thousands of cells) against 100 sequential steps of the float64 oracle, within 1e-9 relative.
- The batched ensemble's multi-step atlas call against every instance run alone through the drop-in
  (its own resident topology, one kinematic_wave_steps call) and through single-step float64 calls.
"""
import os

import numpy as np
import pytest

from lue_gb300 import ensemble, synthetic
from oracle import oracle
from tests import parity

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lfr():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from lue_gb300 import framework
    return framework


def test_kw_8k_band_100_steps_against_oracle(lfr):
    w = synthetic.WORKLOADS["kw_8k"]
    d = synthetic.kinematic_wave_inputs(w["rows"], w["cols"], w["seed"], w["amplitude"])
    rows = 2048
    fd = np.ascontiguousarray(d["flow_direction"][:rows])
    q0 = np.ascontiguousarray(d["discharge"][:rows])
    lat = np.ascontiguousarray(d["lateral_inflow"][:rows])
    alpha = np.ascontiguousarray(d["alpha"][:rows])
    ps = (1024, 1024)
    steps = 100
    a = lfr.from_numpy(fd, ps)
    got = lfr.to_numpy(lfr.kinematic_wave_steps(a, lfr.from_numpy(q0, ps), lfr.from_numpy(lat, ps),
                                                lfr.from_numpy(alpha, ps), 0.6, 3600.0, 100.0, steps))
    assert a.topology().stats()["max_level"] > 2000  # long channels inside the band
    want = q0
    lat64, al64 = lat.astype(np.float64), alpha.astype(np.float64)
    for _ in range(steps):
        want = oracle.kinematic_wave(fd, want, lat64, al64, 0.6, 3600.0, 100.0, ps, dtype=np.float64,
                                     nthreads=os.cpu_count() or 1)
    parity.assert_close64(got, want, "kinematic_wave_steps, kw_8k rows 0-2047, 100 steps")


def test_multi_step_atlas_equals_each_instance_alone(lfr):
    """The measured batched form (all steps of all instances in one kinematic_wave_steps call on the
    atlas) against each instance alone: its own resident topology and one kinematic_wave_steps call
    (stages differ, so equal to about 1e-13, not bit for bit), and single-step float64 calls."""
    import torch
    inst = ensemble.ensemble_inputs(n_catchments=4, scenarios=2, lo=96, hi=400, seed=13)
    steps = 12
    _, atlas, q, _ = ensemble.run_batched(inst, steps, waves=True)
    _, _, plain = ensemble.run_plain_resident(inst, steps)
    _, _, single = ensemble.run_unbatched(inst, steps, sample=len(inst))
    for i in range(len(inst)):
        got = atlas.view(q, i).cpu().numpy()
        alone = plain[i].cpu().numpy()
        assert np.array_equal(np.isnan(got), np.isnan(alone)), i
        assert parity.rel_error(got, alone, parity.FLOOR64)[0] <= 1e-12, i
        assert parity.rel_error(got, single[i].cpu().numpy(), parity.FLOOR64)[0] <= 1e-12, i
    torch.cuda.synchronize()
