"""partial_accu: the oracle's restatement of the reference's event sequence (CPU) and the GPU rule against
it (GPU) on every cell whose value does not depend on the order of inter-partition delivery.

The reference has no test of partial_accu (only its definition, ALG/definition/partial_accu.hpp, and its
Python binding), so the oracle is pinned to a case worked out by hand from the hooks:
ALG/definition/partial_accu.hpp:71-83 (a ridge takes the partition's stream counter, which then goes up
by one), :86-109 (a value from another partition: the larger one), :112-120 (+1 on the partition input
cell after its walk), :129-165 (leave_cell copies the value downstream; above nr_steps: NaN).
"""
import numpy as np
import pytest

from lue_gb300 import synthetic
from oracle import oracle

NAN = np.nan


def test_oracle_hand_worked_case():
    """4 x 3, everything flows south, partitions of 2 rows: partition 0's ridges (row 0) are streams 0, 1,
    2 and row 1 copies them; row 2 (partition 1's input cells) takes the arriving values, its walks copy
    them into row 3, then row 2 goes up by one."""
    fd = np.full((4, 3), 2, np.uint8)
    want = np.array([[0, 1, 2], [0, 1, 2], [1, 2, 3], [0, 1, 2]], np.float64)
    for order in (0, 1):
        assert np.array_equal(oracle.partial_accu(fd, 100, (2, 3), order), want)
    # nr_steps 1: a ridge keeps its number; a copy above 1 is NaN, and NaN flows on; the +1 is not checked
    want1 = np.array([[0, 1, 2], [0, 1, NAN], [1, 2, NAN], [0, 1, NAN]])
    assert np.array_equal(oracle.partial_accu(fd, 1, (2, 3)), want1, equal_nan=True)
    # one partition: every column is one stream; nr_steps below 0 counts as 0
    assert np.array_equal(oracle.partial_accu(fd, 100, (4, 3)), np.tile([0.0, 1.0, 2.0], (4, 1)))
    assert np.array_equal(oracle.partial_accu(fd, -5, (4, 3)), np.array([[0, 1, 2]] + [[0, NAN, NAN]] * 3),
                          equal_nan=True)


def test_oracle_confluence_takes_the_last_walk_and_no_data_is_nan():
    """One partition, 2 x 3: (0,0) flows SE and (0,2) flows SW into (1,1), a sink; (0,1) is no-data.  The
    ridges are streams 0 and 1 (row-major); the walk of stream 1 arrives last at the confluence."""
    fd = np.array([[3, 255, 1], [5, 5, 5]], np.uint8)
    got = oracle.partial_accu(fd, 10, (2, 3))
    assert np.array_equal(got, np.array([[0, NAN, 1], [2, 1, 3]]), equal_nan=True)


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", [np.float32, np.float64], ids=["f32", "f64"])
@pytest.mark.parametrize("shape,partition,nr_steps", [
    ((300, 257), (300, 257), 10 ** 9),
    ((300, 257), (64, 64), 10 ** 9),
    ((300, 257), (50, 37), 10 ** 9),
    ((300, 257), (128, 100), 400),
    ((129, 1031), (40, 200), 10 ** 9),
])
def test_gpu_against_oracle_on_order_independent_cells(dtype, shape, partition, nr_steps):
    import torch
    assert torch.cuda.is_available()
    from lue_gb300 import framework as lfr
    fd = synthetic.flow_direction(shape[0], shape[1], seed=3, amplitude=30.0, wavelength=150)
    fd[np.random.default_rng(5).random(fd.shape) < 0.003] = 255  # no-data cells
    a = lfr.from_numpy(fd, partition)
    got, od = lfr.partial_accu(a, np.float32(0) if dtype == np.float32 else np.float64(0), nr_steps,
                               order_dependent=True)
    got, od = lfr.to_numpy(got), lfr.to_numpy(od).astype(bool)
    assert got.dtype == dtype
    fifo = oracle.partial_accu(fd, nr_steps, partition, order=0)
    other = oracle.partial_accu(fd, nr_steps, partition, order=1)
    differ = ~((fifo == other) | (np.isnan(fifo) & np.isnan(other)))
    assert not (differ & ~od).any(), "a cell whose value depends on the delivery order is not flagged"
    keep = ~od
    assert np.array_equal(got[keep], fifo[keep].astype(dtype), equal_nan=True)
    excluded = od.mean()
    print(f"partial_accu {shape} in {partition}: {100 * excluded:.2f} % of cells order-dependent")
    assert excluded < 0.10  # 6.8 % at the smallest partitions here (50 x 37), none for one partition
    if partition == shape:
        assert not od.any()  # one partition: no inter-partition messages


@pytest.mark.gpu
def test_gpu_hand_worked_cases():
    import torch
    assert torch.cuda.is_available()
    from lue_gb300 import framework as lfr
    fd = np.full((4, 3), 2, np.uint8)
    got = lfr.to_numpy(lfr.partial_accu(lfr.from_numpy(fd, (2, 3)), 0.0, 100))
    assert np.array_equal(got, np.array([[0, 1, 2], [0, 1, 2], [1, 2, 3], [0, 1, 2]], np.float32))
    got = lfr.to_numpy(lfr.partial_accu(lfr.from_numpy(fd, (2, 3)), 0.0, 1))
    assert np.array_equal(got, np.array([[0, 1, 2], [0, 1, NAN], [1, 2, NAN], [0, 1, NAN]], np.float32),
                          equal_nan=True)
    fd = np.array([[3, 255, 1], [5, 5, 5]], np.uint8)
    got = lfr.to_numpy(lfr.partial_accu(lfr.from_numpy(fd, (2, 3)), np.float64(0), 10))
    assert np.array_equal(got, np.array([[0, NAN, 1], [2, 1, 3]]), equal_nan=True)


@pytest.mark.gpu
def test_gpu_cycle_cells_keep_what_was_pushed():
    """A 2 x 2 flow cycle (E, S / N, W) fed by one ridge: the reference never enters the cycle; the cell
    the ridge's walk reaches keeps the ridge's value, the others 0."""
    import torch
    assert torch.cuda.is_available()
    from lue_gb300 import framework as lfr
    fd = np.array([[6, 2, 5], [8, 4, 4]], np.uint8)  # (0,0)->(0,1)->(1,1)->(1,0)->(0,0); (1,2) W into (1,1)
    want = oracle.partial_accu(fd, 10, (2, 3))
    got = lfr.to_numpy(lfr.partial_accu(lfr.from_numpy(fd, (2, 3)), np.float64(0), 10))
    assert np.array_equal(got, want, equal_nan=True)
