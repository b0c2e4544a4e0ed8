"""lue_gpu_accu_f32_noalloc: accu for callers that must not allocate device memory.

Such callers (a model step inside a host framework that owns the device memory pool, or a
latency-critical loop in which cudaMalloc/cudaFree would synchronise the device) get an entry point
whose scratch lives in a fixed device array inside the library.  This test calls it through the C ABI
twice in a row, on different rasters, and checks each result against lue_gpu_accu_f32 (the entry point
that uses a topology with its own scratch), with the float32 tolerance of the other parity tests.
The test buffers are allocated here, by the test; the entry point itself allocates nothing.

Collected last on purpose (file name), so that a run stopping at the first failure has already run
every other test.
"""
import ctypes

import numpy as np
import pytest

from tests import parity

pytestmark = pytest.mark.gpu


def _existing_accu(L, torch, fd, m, ps):
    """lue_gpu_accu_f32 through a topology (the entry point the no-alloc variant must agree with)."""
    h = ctypes.c_void_p()
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.lue_gpu_topology_create(fd.data_ptr(), fd.shape[0], fd.shape[1], ps[0], ps[1], stream, ctypes.byref(h))
    assert rc == 0, L.lue_gpu_last_error()
    out = torch.empty(fd.shape, dtype=torch.float32, device=fd.device)
    rc = L.lue_gpu_accu_f32(h, m.data_ptr(), 0.0, out.data_ptr(), stream)
    assert rc == 0, L.lue_gpu_last_error()
    torch.cuda.synchronize()
    assert L.lue_gpu_topology_destroy(h) == 0
    return out.cpu().numpy()


def _noalloc_accu(L, torch, fd, m, ps):
    out = torch.full(fd.shape, -7.0, dtype=torch.float32, device=fd.device)
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.lue_gpu_accu_f32_noalloc(fd.data_ptr(), fd.shape[0], fd.shape[1], ps[0], ps[1], m.data_ptr(), 0.0,
                                    out.data_ptr(), stream)
    assert rc == 0, L.lue_gpu_last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_noalloc_accu_matches_topology_accu_on_two_calls_in_a_row():
    import torch
    assert torch.cuda.is_available(), "GPU test needs a CUDA device"
    from lue_gb300 import _lib, synthetic

    L = _lib.lib()
    rng = np.random.default_rng(2024)
    cases = []
    # call 1: the 1024 x 1024 workload shape in 256 x 256 partitions, uniform material
    fd1 = synthetic.flow_direction(1024, 1024, seed=1, amplitude=50.0)
    cases.append((fd1, rng.random(fd1.shape, dtype=np.float32), (256, 256)))
    # call 2: exactly the documented maximum (2048 x 2048 = LUE_GPU_NOALLOC_MAX_CELLS), lognormal
    # material with no-data and out-of-domain cells
    fd2 = synthetic.flow_direction(2048, 2048, seed=9, amplitude=120.0)
    m2 = rng.lognormal(0.0, 1.0, fd2.shape).astype(np.float32)
    m2[rng.random(fd2.shape) < 1e-4] = np.nan
    m2[rng.random(fd2.shape) < 1e-4] = -1.0
    cases.append((fd2, m2, (512, 512)))
    assert fd2.size == 4194304
    for fd_np, m_np, ps in cases:
        fd = torch.from_numpy(fd_np).cuda()
        m = torch.from_numpy(m_np).cuda()
        got = _noalloc_accu(L, torch, fd, m, ps)
        want = _existing_accu(L, torch, fd, m, ps)
        parity.assert_close32(got, want, f"accu_f32_noalloc {fd_np.shape}")


def test_noalloc_rejects_rasters_above_the_fixed_scratch():
    import torch
    assert torch.cuda.is_available(), "GPU test needs a CUDA device"
    from lue_gb300 import _lib

    L = _lib.lib()
    fd = torch.zeros(1, dtype=torch.uint8, device="cuda")
    out = torch.zeros(1, dtype=torch.float32, device="cuda")
    rc = L.lue_gpu_accu_f32_noalloc(fd.data_ptr(), 2049, 2048, 1, 1, None, 1.0, out.data_ptr(), None)
    assert rc == 6  # LUE_GPU_ERANGE, before any device work
    assert b"exceed" in L.lue_gpu_last_error()
