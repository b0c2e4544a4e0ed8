"""Batched ensembles: atlas packing (CPU) and batched-vs-alone results (GPU)."""
import numpy as np
import pytest

from lue_gb300 import ensemble, synthetic


def test_atlas_packs_without_overlap_and_with_borders():
    rng = np.random.default_rng(0)
    shapes = [(int(h), int(w)) for h, w in rng.integers(5, 60, size=(40, 2))]
    a = ensemble.Atlas(shapes)
    occ = np.zeros(a.shape, np.int32)
    for (r, c), (h, w) in zip(a.offsets, shapes):
        assert r >= 1 and c >= 1 and r + h + 1 <= a.shape[0] and c + w + 1 <= a.shape[1]
        occ[r - 1:r + h + 1, c - 1:c + w + 1] += 1  # instance plus its one-cell border
    assert occ.max() == 1
    assert a.cells == sum(h * w for h, w in shapes)


def test_catchment_sides_are_log_uniform_and_seeded():
    s1 = ensemble.catchment_sides(64, 512, 4096, 3)
    assert s1 == ensemble.catchment_sides(64, 512, 4096, 3)
    assert min(s1) >= 512 - 8 and max(s1) <= 4096 + 8 and all(s % 8 == 0 for s in s1)


@pytest.mark.gpu
def test_batched_results_equal_each_instance_alone():
    import torch
    assert torch.cuda.is_available()
    inst = ensemble.ensemble_inputs(n_catchments=3, scenarios=2, lo=64, hi=200, seed=5)
    secs, atlas, q, stats = ensemble.run_batched(inst, steps=4)
    _, _, alone = ensemble.run_unbatched(inst, steps=4, sample=len(inst))
    for i, qa in enumerate(alone):
        got = atlas.view(q, i).cpu().numpy()
        assert np.array_equal(got, qa.cpu().numpy()), i  # same kernels, same inputs: bitwise equal


@pytest.mark.gpu
def test_autotuned_multi_step_atlas_equals_the_default_schedule():
    """The batched multi-step call with the stage schedule autotuned on a shorter call gives the same bits
    as with the default schedule."""
    import torch
    assert torch.cuda.is_available()
    inst = ensemble.ensemble_inputs(n_catchments=3, scenarios=2, lo=64, hi=200, seed=7)
    _, atlas, q_default, _ = ensemble.run_batched(inst, steps=6, waves=True)
    _, _, q_tuned, stats = ensemble.run_batched(inst, steps=6, waves=True, autotune_steps=2)
    assert stats["stage_schedule"]["cap"] in (64, 128, 256)
    assert np.array_equal(q_default.cpu().numpy(), q_tuned.cpu().numpy(), equal_nan=True)  # NaN: atlas borders
