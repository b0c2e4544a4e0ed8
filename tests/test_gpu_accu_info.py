"""accu_info on the GPU against the oracle's restatement of the reference's event sequence.

The oracle takes inter-partition arrivals in FIFO order, one order the reference's channels may deliver.
At a partition input cell whose upstream cells in its own partition also wait for other partitions the
reference's class depends on that order; the GPU classes such a cell as if material from another
partition arrived last.  Those cells (found here from the flow directions) are compared with that rule;
every other cell must equal the oracle.
"""
import numpy as np
import pytest

from lue_gb300 import synthetic
from oracle import oracle

pytestmark = pytest.mark.gpu

OFF = {7: (-1, -1), 8: (-1, 0), 9: (-1, 1), 4: (0, -1), 6: (0, 1), 1: (1, -1), 2: (1, 0), 3: (1, 1)}


@pytest.fixture(scope="module")
def lfr():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from lue_gb300 import framework
    return framework


def ambiguous_inputs(fd, ps):
    """Partition input cells with an in-partition upstream cell that depends on another partition."""
    rows, cols = fd.shape
    nr, nc = rows // ps[0], cols // ps[1]
    pr = np.minimum(np.arange(rows) // ps[0], nr - 1)
    pc = np.minimum(np.arange(cols) // ps[1], nc - 1)
    part = pr[:, None] * nc + pc[None, :]
    down = -np.ones(fd.shape, np.int64)
    for code, (dr, dc) in OFF.items():
        r, c = np.nonzero(fd == code)
        ok = (r + dr >= 0) & (r + dr < rows) & (c + dc >= 0) & (c + dc < cols)
        down[r[ok], c[ok]] = (r[ok] + dr) * cols + (c[ok] + dc)
    flat_part = part.ravel()
    flat_down = down.ravel()
    valid = fd.ravel() != 255
    src = np.nonzero((flat_down >= 0) & valid)[0]
    dst = flat_down[src]
    keep = valid[dst]
    src, dst = src[keep], dst[keep]
    cross = flat_part[src] != flat_part[dst]
    inp = np.zeros(fd.size, bool)
    inp[dst[cross]] = True
    # dep: upstream-first propagation inside partitions (Kahn order over all edges)
    indeg = np.bincount(dst, minlength=fd.size)
    dep = inp.copy()
    order = list(np.nonzero(valid & (indeg == 0))[0])
    succ = -np.ones(fd.size, np.int64)
    succ[src] = dst
    i = 0
    while i < len(order):
        u = order[i]
        i += 1
        d = succ[u]
        if d >= 0:
            if flat_part[d] == flat_part[u] and dep[u]:
                dep[d] = True
            indeg[d] -= 1
            if indeg[d] == 0:
                order.append(d)
    amb = np.zeros(fd.size, bool)
    same = ~cross
    amb[dst[same & dep[src]]] = True
    return (amb & inp).reshape(fd.shape)


@pytest.mark.parametrize("seed", range(6))
def test_accu_info_against_oracle(lfr, seed):
    rng = np.random.default_rng(seed)
    rows, cols = int(rng.integers(40, 300)), int(rng.integers(40, 300))
    fd = synthetic.flow_direction(rows, cols, 100 + seed, 40.0, wavelength=max(rows, cols) / 2).copy()
    fd[rng.random(fd.shape) < 0.01] = 5  # sinks
    fd[rng.random(fd.shape) < 0.005] = 0  # unknown codes: sinks too
    for ps in ((rows, cols), (max(1, rows // 3), max(1, cols // 4)), (17, 23)):
        got = lfr.to_numpy(lfr.accu_info(lfr.from_numpy(fd, ps)))
        want = oracle.accu_info(fd, ps)
        amb = ambiguous_inputs(fd, ps)
        assert (got[~amb] == want[~amb]).all(), (ps, np.argwhere((got != want) & ~amb)[:5])
        assert np.isin(got[amb], (14, 15)).all()


def test_accu_info_no_data_and_one_partition(lfr):
    """Outside no-data cells the classes of a single partition are ridge, intra stream, sink or output."""
    fd = synthetic.flow_direction(120, 90, 7, 40.0, wavelength=60).copy()
    fd[:, :3] = 255
    fd[:, 3][np.isin(fd[:, 3], (7, 4, 1))] = 5  # no flow into no-data (the reference leaves that undefined)
    got = lfr.to_numpy(lfr.accu_info(lfr.from_numpy(fd)))
    assert (got[:, :3] == 255).all()
    assert np.isin(got[:, 3:], (11, 12, 13, 17)).all()
    assert (got == oracle.accu_info(fd, fd.shape)).all()
