"""The largest configurations at full size, through properties that need no
FP64 reference of the whole volume (which would not fit a test's budget):

* a centred unit delta kernel reproduces the input (rel-L2 <= 1e-6);
* linearity: conv(a*x + y) = a*conv(x) + conv(y) (rel-L2 <= 1e-5);
* flux: with a kernel of unit sum, sum(conv(x)) = sum(x) (relative 1e-5).

1024x1024x256 with a 63^3 PSF (the tensor-core configuration's shapes, fp32
path) and 64x2048x2048 (2048-long y axis, wide column tiles).
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
