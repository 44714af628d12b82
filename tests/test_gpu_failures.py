"""Failure paths on the GPU, made without a GPU fault.

The reference ends the process with exit() on any CUDA error and lets cuFFT
errors escape its C ABI as C++ exceptions (src/book.h:22-30, :112-121).  This
library reports a status instead and leaves the caller's buffer unchanged.
These tests make the failures on purpose in ways that fault nothing:

  * bounded waits: fc_test_set_wait_fault(limit, 1) makes the kernels with
    asynchronous copies (the pipelined x passes, the fused z pass's
    tensor-map stage) arm their barriers without issuing the copies, with a
    short limit (1e5 clock cycles, about 50 us).  Every wait runs out with
    no copy in flight, each kernel counts its timeout and returns, and the
    context stays usable;
  * allocation failure: fc_fault_inject("alloc:n") fails the n-th device
    allocation on the host, before the CUDA call.

Each test checks the status, that the caller's buffer is unchanged, and that
the next normal call on the same context gives the FP64-oracle result within
rel-L2 <= 1e-5 and max-abs <= 1e-5 * max.
"""
import numpy as np
import pytest

import fourierconvolutioncudalib_gb300 as fc

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5
MAXABS_TOL = 1e-5
SHORT_LIMIT = 100_000  # clock cycles


def _case():
    rng = np.random.default_rng(77)
    im = rng.random((64, 64, 64), dtype=np.float32)  # power-of-two axes: pipelined x passes + tensor-map z stage
    k = rng.random((7, 5, 9), dtype=np.float32)
    return im, (k / k.sum()).astype(np.float32)


def _good(out, exact):
    from oracle import oracle as orc

    assert orc.rel_l2(out, exact) <= REL_TOL
    assert orc.max_abs(out, exact) <= MAXABS_TOL * float(np.max(np.abs(exact)))


def _inplace(buf, k):
    nz, ny, nx = buf.shape
    kz, ky, kx = k.shape
    fc.convolution3DfftCUDAInPlace(buf, (nx, ny, nz), k, (kx, ky, kz), 0)


@pytest.mark.parametrize("host_io", [0, 1], ids=["copy", "direct"])
def test_expired_waits_fail_inplace_and_keep_im(cuda, fclib, orc, host_io):
    im, k = _case()
    exact = orc.conv_fp64(im, k, "centered")
    fclib.fc_set_host_io(host_io)
    try:
        buf = im.copy()
        assert fclib.fc_test_set_wait_fault(SHORT_LIMIT, 1) == fc.FC_OK
        try:
            with pytest.raises(fc.FcError) as e:
                _inplace(buf, k)
        finally:
            assert fclib.fc_test_set_wait_fault(0, 0) == fc.FC_OK
        assert e.value.status == fc.FC_ERR_TIMEOUT, e.value.message
        np.testing.assert_array_equal(buf, im)  # the caller's buffer is as it was
        _inplace(buf, k)  # the context stays usable
        _good(buf, exact)
    finally:
        fclib.fc_set_host_io(2)


def test_expired_waits_reported_for_device_entry(cuda, fclib, orc):
    import torch

    from fourierconvolutioncudalib_gb300 import device as fcd

    im, k = _case()
    img = torch.from_numpy(im).to(cuda)
    ker = torch.from_numpy(k).to(cuda)
    st = torch.cuda.current_stream().cuda_stream
    assert fclib.fc_device_wait_status(st) == fc.FC_OK
    assert fclib.fc_test_set_wait_fault(SHORT_LIMIT, 1) == fc.FC_OK
    try:
        fcd.conv3d(img, ker)
        rc = fclib.fc_device_wait_status(st)
    finally:
        assert fclib.fc_test_set_wait_fault(0, 0) == fc.FC_OK
    assert rc == fc.FC_ERR_TIMEOUT, fclib.fc_last_error().decode()
    assert fclib.fc_device_wait_status(st) == fc.FC_OK  # the counts were cleared
    out = fcd.conv3d(img, ker)
    assert fclib.fc_device_wait_status(st) == fc.FC_OK
    _good(out.cpu().numpy(), orc.conv_fp64(im, k, "centered"))


@pytest.mark.parametrize("nth", [1, 2, 3])
def test_injected_allocation_failure(cuda, fclib, orc, nth):
    im, k = _case()
    assert fclib.fc_release_device(0) == fc.FC_OK  # the next call allocates its buffers afresh
    buf = im.copy()
    assert fclib.fc_fault_inject(f"alloc:{nth}".encode()) == fc.FC_OK
    try:
        with pytest.raises(fc.FcError) as e:
            _inplace(buf, k)
    finally:
        fclib.fc_fault_inject(b"off")
    assert e.value.status == fc.FC_ERR_NOMEM
    assert "injected allocation failure" in e.value.message
    np.testing.assert_array_equal(buf, im)
    _inplace(buf, k)
    _good(buf, orc.conv_fp64(im, k, "centered"))
