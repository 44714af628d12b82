"""The allocation-free entry point, fc_conv3d_device_noalloc.

It serves callers that cannot allocate device memory when they convolve (a
framework that already holds the GPU's memory in its own pool, a real-time
loop that cannot afford cudaMalloc's synchronisation, a deployment that
forbids device allocation after start-up): all of its scratch comes from one
static device array of FC_NOALLOC_SCRATCH_BYTES.  The test calls it through
the C ABI and checks it against fc_conv3d_device, on two calls in a row with
different shapes (the shared array keeps the previous call's contents), and
checks that an oversized request is refused.

Tolerance: rel-L2 <= 1e-5 and max-abs <= 1e-5 * max|reference| against the
existing entry point (same kernels; only the twiddle tables are generated on
the device instead of the host).

This file is named to be collected last, so that a run stopping at the first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

import fourierconvolutioncudalib_gb300 as fc

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5
MAXABS_TOL = 1e-5
NOALLOC_SCRATCH_BYTES = 64 << 20  # FC_NOALLOC_SCRATCH_BYTES in include/convolution3Dfft.h


def _existing(torch, img, ker, flags=0):
    from fourierconvolutioncudalib_gb300 import device as fcd

    return fcd.conv3d(img, ker, flags=flags)


def _noalloc(torch, img, ker, flags=0):
    L = fc.lib()
    nz, ny, nx = img.shape
    kz, ky, kx = ker.shape
    out = torch.empty_like(img)
    rc = L.fc_conv3d_device_noalloc(img.data_ptr(), out.data_ptr(), fc._iarr([nx, ny, nz]), ker.data_ptr(),
                                    fc._iarr([kx, ky, kz]), int(flags), torch.cuda.current_stream().cuda_stream)
    assert rc == fc.FC_OK, L.fc_last_error().decode()
    return out


def _compare(out, ref):
    o = out.double().cpu().numpy()
    r = ref.double().cpu().numpy()
    rel = np.linalg.norm(o - r) / np.linalg.norm(r)
    mx = np.max(np.abs(o - r)) / np.max(np.abs(r))
    assert rel <= REL_TOL, rel
    assert mx <= MAXABS_TOL, mx


def test_noalloc_matches_device_entry_twice(cuda):
    import torch

    rng = np.random.default_rng(123)
    cases = [((48, 80, 128), (9, 7, 11), 0),   # power-of-two rows and z: register-resident kernels
             ((30, 44, 50), (5, 3, 7), 0),     # mixed radices: generic kernels; smaller than the first call
             ((24, 20, 30), (5, 3, 7), fc.FC_FLAG_SHIFT_COMPAT)]
    for shape, kshape, flags in cases:
        img = torch.from_numpy(rng.random(shape, dtype=np.float32)).to(cuda)
        k = rng.random(kshape, dtype=np.float32)
        ker = torch.from_numpy(k / k.sum()).to(cuda)
        ref = _existing(torch, img, ker, flags)
        got = _noalloc(torch, img, ker, flags)
        torch.cuda.synchronize()
        _compare(got, ref)


def test_noalloc_rejects_oversized(cuda):
    import torch

    L = fc.lib()
    # 512x512x128 with a 31x31x63 kernel needs ~210 MiB of scratch, beyond the static array;
    # the size check happens on the host before anything is enqueued
    dummy = torch.empty(1, device=cuda)
    rc = L.fc_conv3d_device_noalloc(dummy.data_ptr(), dummy.data_ptr(), fc._iarr([512, 512, 128]), dummy.data_ptr(),
                                    fc._iarr([31, 31, 63]), 0, torch.cuda.current_stream().cuda_stream)
    assert rc == fc.FC_ERR_NOMEM
    msg = L.fc_last_error().decode()
    assert str(NOALLOC_SCRATCH_BYTES) in msg
