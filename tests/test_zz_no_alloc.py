"""The allocation-free entry point, fc_conv3d_device_noalloc.

It serves callers that cannot allocate device memory when they convolve (a
framework that already holds the GPU's memory in its own pool, a real-time
loop that cannot afford cudaMalloc's synchronisation, a deployment that
forbids device allocation after start-up): all of its scratch comes from one
static device array of FC_NOALLOC_SCRATCH_BYTES.  The tests call it through
the C ABI and check it against fc_conv3d_device and against the FP64 oracle,
on calls in a row with different shapes (the shared array keeps the previous
call's contents); check that, once the first call has set the array up, the
calls change neither the device's free memory nor torch's allocator; and
check that an oversized request is refused.

Tolerance: rel-L2 <= 1e-5 and max-abs <= 1e-5 * max|reference| against the
existing entry point and against FP64.  The two entry points run the same
kernels; the allocation-free one generates its twiddle tables on the device
(sincospi in double precision, rounded once) on every call, the existing one
on the host once per length, so the two can differ by about an ulp there.

This file is named to be collected last, so that a run stopping at the first
failure has already run every other test.
"""
import numpy as np
import pytest

import fourierconvolutioncudalib_gb300 as fc

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5
MAXABS_TOL = 1e-5
NOALLOC_SCRATCH_BYTES = 64 << 20  # FC_NOALLOC_SCRATCH_BYTES in include/convolution3Dfft.h


def _existing(img, ker, flags=0):
    from fourierconvolutioncudalib_gb300 import device as fcd

    return fcd.conv3d(img, ker, flags=flags)


def _noalloc_into(torch, out, img, ker, flags=0):
    L = fc.lib()
    nz, ny, nx = img.shape
    kd = fc._iarr([ker.shape[2], ker.shape[1], ker.shape[0]])
    rc = L.fc_conv3d_device_noalloc(img.data_ptr(), out.data_ptr(), fc._iarr([nx, ny, nz]), ker.data_ptr(), kd,
                                    int(flags), torch.cuda.current_stream().cuda_stream)
    assert rc == fc.FC_OK, L.fc_last_error().decode()
    return out


def _compare(out, ref, what):
    o = np.asarray(out, np.float64)
    r = np.asarray(ref, np.float64)
    rel = np.linalg.norm(o - r) / np.linalg.norm(r)
    mx = np.max(np.abs(o - r)) / np.max(np.abs(r))
    assert rel <= REL_TOL, f"{what}: rel-L2 {rel:.3e}"
    assert mx <= MAXABS_TOL, f"{what}: max-abs {mx:.3e}"


def _cases(rng):
    """(image zyx, kernel, flags, FP64 placement): x = 128 with z = 48 and y = 80
    (register-resident kernels on every axis), mixed radices (generic
    kernels, a smaller call after a larger one), the reference placement, and
    an image-sized, already shifted (dense) kernel."""
    out = []
    for shape, kshape, flags, placement in (((48, 80, 128), (9, 7, 11), 0, "centered"),
                                            ((30, 44, 50), (5, 3, 7), 0, "centered"),
                                            ((24, 20, 30), (5, 3, 7), fc.FC_FLAG_SHIFT_COMPAT, "reference_inplace")):
        k = rng.random(kshape, dtype=np.float32)
        out.append((rng.random(shape, dtype=np.float32), (k / k.sum()).astype(np.float32), flags, placement))
    dense = rng.random((32, 40, 64), dtype=np.float32)
    dense /= dense.sum()
    out.append((rng.random((32, 40, 64), dtype=np.float32), dense, fc.FC_FLAG_DENSE_KERNEL, "dense"))
    return out


def test_noalloc_matches_device_entry_and_fp64(cuda, orc):
    import torch

    rng = np.random.default_rng(123)
    for im, k, flags, placement in _cases(rng):
        img = torch.from_numpy(im).to(cuda)
        ker = torch.from_numpy(k).to(cuda)
        ref = _existing(img, ker, flags)
        got = _noalloc_into(torch, torch.empty_like(img), img, ker, flags)
        torch.cuda.synchronize()
        g = got.cpu().numpy()
        _compare(g, ref.cpu().numpy(), f"{im.shape} flags {flags} vs fc_conv3d_device")
        _compare(g, orc.conv_fp64(im, k, placement), f"{im.shape} flags {flags} vs FP64")


def test_noalloc_allocates_nothing_after_setup(cuda, orc):
    """After the first call on the device (which loads the module that holds
    the static array), two calls in a row leave the device's free memory and
    torch's allocator counters unchanged, and both give the right result."""
    import torch

    rng = np.random.default_rng(7)
    im1 = rng.random((40, 64, 96), dtype=np.float32)
    im2 = rng.random((20, 36, 50), dtype=np.float32)
    k = rng.random((7, 5, 9), dtype=np.float32)
    k /= k.sum()
    i1, i2, kt = (torch.from_numpy(a).to(cuda) for a in (im1, im2, k))
    o1, o2 = torch.empty_like(i1), torch.empty_like(i2)
    _noalloc_into(torch, o1, i1, kt)  # set-up call
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    alloc0, resv0 = torch.cuda.memory_allocated(), torch.cuda.memory_reserved()
    _noalloc_into(torch, o1, i1, kt)
    _noalloc_into(torch, o2, i2, kt)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"device free memory changed by {free0 - free1} bytes"
    assert torch.cuda.memory_allocated() == alloc0 and torch.cuda.memory_reserved() == resv0
    _compare(o1.cpu().numpy(), orc.conv_fp64(im1, k, "centered"), "first of two calls vs FP64")
    _compare(o2.cpu().numpy(), orc.conv_fp64(im2, k, "centered"), "second of two calls vs FP64")


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
