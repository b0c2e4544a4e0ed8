"""Runs one stage-engine operation on a seeded synthetic raster, timed with CUDA events: the workload
that the stage-engine profiles are taken on.

    python -m lue_gb300.examples.stage_workload SIDE OPERATION [CALLS]

SIDE: raster side (cells); OPERATION: ``accu`` (the tile engine, float32 lognormal(0, 1) material),
``threshold`` (accu_threshold, float32 lognormal(0, 1) material, uniform [0, 0.5) thresholds) or ``kwN``
(kinematic_wave_steps with N steps; ``kw1`` is one kinematic_wave call), beta 0.6,
dt 3600 s, dx 100 m, float64 discharge, float32 rain and alpha); CALLS: calls, the last one timed
(default 4).  Inputs come from ``lue_gb300.synthetic.kinematic_wave_inputs(SIDE, SIDE, 5, 200.0)``.
"""
import sys

import numpy as np
import torch

from lue_gb300 import framework as lfr
from lue_gb300 import synthetic


def main(argv):
    side, op = int(argv[1]), argv[2]
    calls = int(argv[3]) if len(argv) > 3 else 4
    d = synthetic.kinematic_wave_inputs(side, side, 5, 200.0)
    fd = lfr.from_numpy(d["flow_direction"])
    q, lat, alpha = (lfr.from_numpy(d[k]) for k in ("discharge", "lateral_inflow", "alpha"))
    rng = np.random.default_rng(1)
    material = lfr.from_numpy(rng.lognormal(0.0, 1.0, d["flow_direction"].shape).astype(np.float32))
    threshold = lfr.from_numpy((rng.random(d["flow_direction"].shape) * 0.5).astype(np.float32))
    if op == "accu":
        def fn():
            return lfr.accu(fd, material)
    elif op == "threshold":
        def fn():
            return lfr.accu_threshold(fd, material, threshold)
    elif op == "kw1":
        def fn():
            return lfr.kinematic_wave(fd, q, lat, alpha, 0.6, 3600.0, 100.0)
    elif op.startswith("kw"):
        steps = int(op[2:])

        def fn():
            return lfr.kinematic_wave_steps(fd, q, lat, alpha, 0.6, 3600.0, 100.0, steps)
    else:
        raise SystemExit(f"unknown operation {op!r}")
    for _ in range(calls - 1):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    fn()
    e1.record()
    torch.cuda.synchronize()
    print(f"{op} {side}x{side}: {e0.elapsed_time(e1):.3f} ms")


if __name__ == "__main__":
    main(sys.argv)
