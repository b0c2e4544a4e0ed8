"""The numpy boundary (lue.framework.from_numpy / to_numpy, source/framework/python/source/numpy/
{from_numpy,to_numpy}.cpp): no-data mapping on the device, pinned staging, stream-ordered copies."""
import numpy as np
import pytest

from tests.golden import cases as golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lfr():
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    from lue_gb300 import framework
    return framework


@pytest.mark.parametrize("dtype,no_data,device_no_data", [
    (np.float32, -999.0, np.nan), (np.float64, -1.0e30, np.nan), (np.uint8, 0, 255),
    (np.int32, -1, np.iinfo(np.int32).min), (np.int64, 7, np.iinfo(np.int64).min)])
def test_round_trip_with_no_data_value(lfr, dtype, no_data, device_no_data):
    rng = np.random.default_rng(3)
    a = (rng.integers(0, 100, size=(37, 1001)) if np.issubdtype(dtype, np.integer)
         else rng.random((37, 1001)) * 10).astype(dtype)
    mask = rng.random(a.shape) < 0.05
    a[mask] = no_data
    mask = a == no_data  # values that happened to equal it too
    d = lfr.from_numpy(a, (10, 200), no_data_value=no_data)
    on_device = d.data.cpu().numpy()
    want = a.copy()
    want[mask] = device_no_data
    assert np.array_equal(on_device, want, equal_nan=True)
    back = lfr.to_numpy(d, no_data_value=no_data)
    assert back.dtype == dtype and np.array_equal(back, a)
    raw = lfr.to_numpy(d)  # without a no-data value: the element type's own no-data value comes out
    assert np.array_equal(raw, want, equal_nan=True)


def test_golden_rasters_round_trip_and_route_with_an_explicit_no_data_value(lfr):
    """The reference's back_and_forth case with its material marked -1 where no-data is wanted: routed
    after from_numpy(no_data_value=-1) it equals routing NaN material; to_numpy(no_data_value=-1)
    writes -1 back where the result is no-data."""
    from oracle import oracle
    c = [c for c in golden.load("accu") if c["name"] == "back_and_forth"][0]
    fd = golden.u8(c["flow_direction"])
    ps = tuple(c["partition_shape"])
    m = np.ones(fd.shape, np.float32)
    m[1, 2] = -1.0
    fd_d = lfr.from_numpy(fd, ps)
    assert np.array_equal(lfr.to_numpy(fd_d), fd)
    out = lfr.accu(fd_d, lfr.from_numpy(m, ps, no_data_value=-1.0))
    m_nan = m.copy()
    m_nan[1, 2] = np.nan
    want = oracle.accu(fd, m_nan.astype(np.float64), ps, dtype=np.float64)
    got = lfr.to_numpy(out, no_data_value=-1.0)
    assert np.array_equal(got[np.isnan(want)], np.full(np.isnan(want).sum(), -1.0, np.float32))
    assert np.array_equal(got[~np.isnan(want)], want[~np.isnan(want)].astype(np.float32))


def test_pinned_arrays_copy_asynchronously_on_the_current_stream(lfr):
    import torch
    rows, cols = 1024, 2048
    src = lfr.pinned_empty((rows, cols), np.float32)
    src[...] = np.arange(rows * cols, dtype=np.float32).reshape(rows, cols)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        d = lfr.from_numpy(src, (256, 256))
        out = lfr.pinned_empty((rows, cols), np.float32)
        ev = lfr.to_numpy_async(d, out)
    ev.synchronize()
    assert np.array_equal(out, src)
    with pytest.raises(ValueError):
        lfr.to_numpy_async(d, np.empty((rows, cols), np.float32))  # pageable: refused
    with pytest.raises(TypeError):
        lfr.from_numpy(np.zeros((4, 4), np.float16))
