"""Serving loop: continuous batching over resident topologies; each result equals the same request
served alone, bit for bit, and the plain one-call-per-step path to ~1e-13."""
import copy

import numpy as np
import pytest

from lue_gb300 import serving


def test_requests_are_seeded_poisson_arrivals():
    shapes = [(64, 64), (128, 96)]
    a = serving.make_requests(shapes, rate=200, duration=0.5, seed=3)
    b = serving.make_requests(shapes, rate=200, duration=0.5, seed=3)
    assert [r.arrival for r in a] == [r.arrival for r in b]
    assert 50 < len(a) < 160
    assert all(x.arrival < y.arrival for x, y in zip(a, a[1:]))
    assert {r.kind for r in a} == {"accu", "kinematic_wave"}


@pytest.mark.gpu
def test_results_in_the_mix_equal_results_alone():
    import torch
    assert torch.cuda.is_available()
    shapes = serving.pool_shapes(n=6, lo=64, hi=320, seed=4)
    pool = serving.build_pool(shapes, seed=4)
    server = serving.Server(pool, slots=6)
    reqs = serving.make_requests(shapes, rate=400, duration=0.1, kw_steps=5, seed=9)
    assert len(reqs) >= 10
    mixed = copy.deepcopy(reqs)
    summary = server.run(mixed, realtime=False)  # everything queued at once: maximal overlap
    assert summary["max_concurrent"] > 1
    for r in reqs:  # each request alone, on a fresh server state
        single = copy.deepcopy(r)
        single.arrival = 0.0
        server.run([single], realtime=False)
        m = [x for x in mixed if x.rid == r.rid][0]
        assert np.array_equal(m.result, single.result, equal_nan=True), r.rid
    # the plain path: a topology per request and one kinematic_wave call per step (float64 solve); the
    # served path runs the steps in one call (float-float solve): equal accu results, and discharge equal
    # to ~1e-13 (well inside the float64 tolerance against the oracle)
    from tests import parity
    plain = copy.deepcopy(reqs)
    serving.run_sequential_plain(server, plain)
    for m, p in zip(sorted(mixed, key=lambda x: x.rid), sorted(plain, key=lambda x: x.rid)):
        if m.kind == "accu":
            assert np.array_equal(m.result, p.result, equal_nan=True), m.rid
        else:
            assert np.array_equal(np.isnan(m.result), np.isnan(p.result)), m.rid
            assert parity.rel_error(m.result, p.result, parity.FLOOR64)[0] <= 1e-12, m.rid


@pytest.mark.gpu
def test_admission_waits_for_memory_and_rejects_requests_above_the_budget():
    """A request that does not fit beside the running ones waits until they finish; one that exceeds the
    whole budget is never admitted; low free HBM (a fake of the free-memory query) holds requests back."""
    import torch
    assert torch.cuda.is_available()
    shapes = [(64, 64), (256, 256)]
    pool = serving.build_pool(shapes, seed=4)
    server = serving.Server(pool, slots=4)
    small = serving.Request(0, "accu", 0, 0.0, 1, dict(seed=1))
    big = serving.Request(1, "kinematic_wave", 1, 0.0, 5, dict(seed=2))
    server.budget = server.bytes_needed(small) + server.bytes_needed(big) - 1  # not both at once
    server.in_use = server.bytes_needed(small)  # as if the small request were running
    assert server.admissible(big, busy=True) == "wait"
    assert server.admissible(big, busy=False) is None
    server.in_use = 0
    summary = server.run([small, big], realtime=False)
    assert summary["rejected"] == 0 and summary["max_concurrent"] == 1
    assert big.start >= small.done and big.result is not None
    server.budget = 1 << 40
    server.free_bytes = lambda: server.RESERVE_BYTES  # nothing free beyond the reserve
    assert server.admissible(small, busy=True) == "wait"
    assert server.admissible(small, busy=False) is None
    del server.free_bytes
    server.budget = server.bytes_needed(big) - 1
    too_big = serving.Request(2, "kinematic_wave", 1, 0.0, 5, dict(seed=3))
    summary = server.run([too_big], realtime=False)
    assert summary["rejected"] == 1 and too_big.error and too_big.result is None
