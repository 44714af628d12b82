"""The largest configurations at full size.

Through properties that hold at any size:

* a centred unit delta kernel reproduces the input (rel-L2 <= 1e-6);
* linearity: conv(a*x + y) = a*conv(x) + conv(y) (rel-L2 <= 1e-5);
* flux: with a kernel of unit sum, sum(conv(x)) = sum(x) (relative 1e-5);

on 1024x1024x256 with a 63^3 PSF (the tensor-core configuration's shapes,
fp32 path) and 64x2048x2048 (2048-long y axis, wide column tiles).  And
against an FP64 FFT convolution of the whole 1024x1024x256 configuration on
the host, for the fp32 path and both tensor-core modes.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    import torch

    a = a.double()
    b = b.double()
    return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))


@pytest.mark.parametrize("shape,kshape", [((256, 1024, 1024), (63, 63, 63)), ((64, 2048, 2048), (31, 15, 15))])
def test_full_size_properties(cuda, shape, kshape):
    import torch
    from fourierconvolutioncudalib_gb300 import device as fcd

    g = torch.Generator(device=cuda).manual_seed(7)
    x = torch.rand(shape, device=cuda, generator=g)
    y = torch.rand(shape, device=cuda, generator=g)
    k = torch.rand(kshape, device=cuda, generator=g)
    k /= k.sum()
    ws = torch.empty(fcd.workspace_bytes(shape, kshape), dtype=torch.uint8, device=cuda)
    # delta kernel at the centre: identity
    delta = torch.zeros(kshape, device=cuda)
    delta[kshape[0] // 2, kshape[1] // 2, kshape[2] // 2] = 1.0
    cx = fcd.conv3d(x, delta, workspace=ws)
    torch.cuda.synchronize()
    assert _rel(cx, x) <= 1e-6
    # linearity
    a = 0.37
    lhs = fcd.conv3d(a * x + y, k, workspace=ws)
    rhs = a * fcd.conv3d(x, k, workspace=ws)
    rhs += fcd.conv3d(y, k, workspace=ws)
    torch.cuda.synchronize()
    assert _rel(lhs, rhs) <= 1e-5
    # flux
    s_in = float(x.double().sum())
    s_out = float(fcd.conv3d(x, k, workspace=ws).double().sum())
    assert abs(s_out / s_in - 1) <= 1e-5


@pytest.mark.parametrize("mode", ["fp32", "fp16", "bf16"])
def test_c5_against_fp64(cuda, mode):
    """The tensor-core configuration at full size (1024x1024x256 spot stack,
    20000 spots, 63^3 mixture PSF) against an FP64 FFT convolution on the host
    (scipy, all cores): the fp32 path at rel-L2 <= 1e-5 and max-abs <= 1e-5*max,
    the tensor-core modes at their tolerances (fp16 2e-6 / 1e-5, bf16
    1e-5 / 5e-5)."""
    import torch

    import fourierconvolutioncudalib_gb300 as fc
    from fourierconvolutioncudalib_gb300 import device as fcd

    ref, im, k = _c5_fp64()
    flag = {"fp32": 0, "fp16": fc.FC_FLAG_TC_FP16, "bf16": fc.FC_FLAG_TC_BF16}[mode]
    tol = {"fp32": (1e-5, 1e-5), "fp16": (2e-6, 1e-5), "bf16": (1e-5, 5e-5)}[mode]
    out = fcd.conv3d(torch.from_numpy(im).to(cuda), torch.from_numpy(k).to(cuda), flags=flag)
    got = out.cpu().numpy().astype(np.float64)
    del out
    rel = np.linalg.norm((got - ref).ravel()) / np.linalg.norm(ref.ravel())
    mx = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    print(f"1024x1024x256 / 63^3 {mode}: FP64 rel-L2 {rel:.3e}, max-abs/max {mx:.3e}")
    assert rel <= tol[0] and mx <= tol[1]


_C5 = {}


def _c5_fp64():
    """FP64 convolution of the 1024x1024x256 configuration, computed once per session."""
    import os

    import scipy.fft as sfft

    from fourierconvolutioncudalib_gb300 import workloads as W

    if "ref" not in _C5:
        d = W.c5()
        im, k = d["image"], d["kernel"]
        nz, ny, nx = im.shape
        kz, ky, kx = k.shape
        pk = np.zeros(im.shape, np.float64)
        pk[np.ix_((np.arange(kz) - kz // 2) % nz, (np.arange(ky) - ky // 2) % ny, (np.arange(kx) - kx // 2) % nx)] = k
        w = os.cpu_count() or 1
        a = sfft.rfftn(im.astype(np.float64), workers=w)
        a *= sfft.rfftn(pk, workers=w)
        del pk
        _C5.update(ref=sfft.irfftn(a, s=im.shape, workers=w), im=im, k=k)
    return _C5["ref"], _C5["im"], _C5["k"]
