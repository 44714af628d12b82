"""The library's own 3D R2C / C2R transforms against numpy (FP64), on the
round-trip shapes of the reference's cuFFT behaviour tests
(tests/test_how_cufft_works.cu:191-711) and more.

Tolerances: forward spectrum rel-L2 <= 2e-6 against numpy.fft.rfftn in
float64; R2C -> 1/N -> C2R round trip rel-L2 <= 2e-6 (the reference's own
thresholds on sqrt(sum d^2)/N, 1e-1 .. 1e-4, are also asserted)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [  # (z, y, x)
    (13, 17, 19),   # of_prime_shape (:191-222)
    (17, 17, 17),   # of_prime_shape_symmetric (:224-253)
    (32, 16, 8),    # power_of_2 (:255-287)
    (9, 27, 3),     # power_of_3 (:289-319)
    (5, 25, 125),   # power_of_5 (:321-351)
    (7, 49, 343),   # power_of_7 (:353-384)
    (128, 128, 128),  # cube_128_shape (:386-416)
    (7, 14, 343),   # out-of-place variant shape
    (128, 512, 512), (96, 448, 384), (1, 1, 64), (2, 3, 4), (1, 1, 1), (8, 16, 4096), (4, 1024, 32), (160, 288, 320), (200, 352, 400), (12, 960, 768),
]


@pytest.fixture(params=["fast", "generic"])
def kernels(request, fclib):
    fclib.fc_set_generic_kernels(1 if request.param == "generic" else 0)
    yield request.param
    fclib.fc_set_generic_kernels(0)


@pytest.mark.parametrize("shape", SHAPES)
def test_rfft3d_and_round_trip(cuda, kernels, shape):
    import torch
    from fourierconvolutioncudalib_gb300 import device as fcd
    from oracle import oracle as orc

    rng = np.random.default_rng(int(np.prod(shape)) % 1000)
    x = rng.standard_normal(shape).astype(np.float32)
    xt = torch.from_numpy(x).to(cuda)
    spec = fcd.rfft3d(xt)
    ref = np.fft.rfftn(x.astype(np.float64))
    got = spec.cpu().numpy()
    assert got.shape == ref.shape
    err = np.linalg.norm((got - ref).ravel()) / max(np.linalg.norm(ref.ravel()), 1e-30)
    assert err <= 2e-6, f"forward rel-L2 {err:.3e}"
    back = fcd.irfft3d(spec, shape[2]).cpu().numpy() / np.float32(x.size)
    rt = orc.rel_l2(back, x)
    assert rt <= 2e-6, f"round trip rel-L2 {rt:.3e}"
    assert orc.l2norm(x, back) < 1e-4
