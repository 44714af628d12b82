"""Subsampled-kernel convolution (convolution3DfftCUDAInPlaceSaveMemory and
fc_conv3d_subsampled_device) against the FP64 restatement of the reference's
nearest-neighbour product (src/convolution3Dfft.cu:65-125).

Tolerances: against the FP64 oracle rel-L2 <= 1e-5 and max-abs <= 1e-5 *
max|ref| (the plain path's bar: the same fp32 transforms and one product);
the host entry against the device entry rel-L2 <= 1e-6 (the same passes, the
x passes possibly on their non-pipelined form).
"""
import numpy as np
import pytest

import fourierconvolutioncudalib_gb300 as fc

pytestmark = pytest.mark.gpu

# (z, y, x) image, (kz, ky, kx) kernel: fused z pass (z of 64, 128, 20) and
# the generic z sequence (z of 37); odd kx (x Nyquist past the stored half)
# and even kx; the kernel as large as the image (r = 1); a single tap
CASES = [((64, 128, 128), (9, 7, 5)), ((128, 96, 160), (15, 9, 8)), ((37, 50, 44), (5, 7, 9)),
         ((20, 34, 221), (3, 5, 7)), ((32, 32, 32), (32, 32, 32)), ((16, 24, 30), (1, 1, 1))]


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def _case(shape, kshape):
    rng = np.random.default_rng(sum(shape) + 7 * sum(kshape))
    im = rng.random(shape).astype(np.float32)
    k = rng.random(kshape).astype(np.float32)
    return im, k / k.sum()


@pytest.fixture(params=["fast", "generic"])
def kernels(request, fclib):
    """The register-resident kernels where the lengths have them, and the
    generic kernels forced on every axis (unfused z forward, product, z inverse)."""
    fclib.fc_set_generic_kernels(1 if request.param == "generic" else 0)
    yield request.param
    fclib.fc_set_generic_kernels(0)


@pytest.mark.parametrize("shape,kshape", CASES)
def test_device_entry_vs_fp64(cuda, orc, kernels, shape, kshape):
    import torch
    from fourierconvolutioncudalib_gb300 import device as fcd

    im, k = _case(shape, kshape)
    got = fcd.conv3d_subsampled(torch.from_numpy(im).to(cuda), torch.from_numpy(k).to(cuda))
    torch.cuda.synchronize()
    g = got.cpu().numpy()
    ref = orc.subsampled_fp64(im, k)
    rel = _rel(g, ref)
    assert rel <= 1e-5, (kernels, shape, kshape, rel)
    assert np.max(np.abs(g - ref)) <= 1e-5 * np.max(np.abs(ref))


def test_single_tap_scales_the_image(cuda):
    import torch
    from fourierconvolutioncudalib_gb300 import device as fcd

    im = np.random.default_rng(3).random((24, 40, 64)).astype(np.float32)
    got = fcd.conv3d_subsampled(torch.from_numpy(im).to(cuda), torch.full((1, 1, 1), 2.0, device=cuda))
    torch.cuda.synchronize()
    assert _rel(got.cpu().numpy(), 2.0 * im) <= 1e-6


@pytest.mark.parametrize("pinned", [False, True])
def test_host_entry_matches_device_entry(cuda, orc, pinned):
    import torch
    from fourierconvolutioncudalib_gb300 import device as fcd

    shape, kshape = (64, 96, 128), (11, 9, 7)
    im, k = _case(shape, kshape)
    dev = fcd.conv3d_subsampled(torch.from_numpy(im).to(cuda), torch.from_numpy(k).to(cuda))
    torch.cuda.synchronize()
    buf = torch.from_numpy(im.copy()).pin_memory().numpy() if pinned else im.copy()
    nz, ny, nx = shape
    kz, ky, kx = kshape
    fc.convolution3DfftCUDAInPlaceSaveMemory(buf, (nx, ny, nz), k, (kx, ky, kz), 0)
    assert _rel(buf, dev.cpu().numpy()) <= 1e-6
    assert _rel(buf, orc.subsampled_fp64(im, k)) <= 1e-5


def test_in_place_and_caller_workspace(cuda, orc):
    import torch
    from fourierconvolutioncudalib_gb300 import device as fcd

    shape, kshape = (32, 64, 96), (7, 5, 9)
    im, k = _case(shape, kshape)
    x = torch.from_numpy(im).to(cuda)
    ws = torch.empty(fcd.subsampled_workspace_bytes(shape, kshape), dtype=torch.uint8, device=cuda)
    fcd.conv3d_subsampled(x, torch.from_numpy(k).to(cuda), out=x, workspace=ws)
    torch.cuda.synchronize()
    assert _rel(x.cpu().numpy(), orc.subsampled_fp64(im, k)) <= 1e-5


def test_rejects_bad_arguments(cuda):
    import torch

    L = fc.lib()
    img = torch.zeros((8, 8, 8), device=cuda)
    ker = torch.ones((3, 3, 3), device=cuda)
    small = torch.empty(256, dtype=torch.uint8, device=cuda)
    rc = L.fc_conv3d_subsampled_device(img.data_ptr(), img.data_ptr(), fc._iarr([8, 8, 8]), ker.data_ptr(),
                                       fc._iarr([3, 3, 3]), small.data_ptr(), 256, None)
    assert rc == fc.FC_ERR_NOMEM
    rc = L.fc_conv3d_subsampled_device(img.data_ptr(), img.data_ptr(), fc._iarr([8, 8, 8]), ker.data_ptr(),
                                       fc._iarr([9, 3, 3]), None, 0, None)
    assert rc == fc.FC_ERR_ARG
    im = np.ones((8, 8, 8), np.float32)
    with pytest.raises(fc.FcError):
        fc.convolution3DfftCUDAInPlaceSaveMemory(im, (8, 8, 8), np.ones((3, 3, 9), np.float32), (3, 3, 9), 0)
    assert np.all(im == 1)
