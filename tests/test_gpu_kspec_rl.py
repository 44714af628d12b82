"""Kernel-spectrum reuse (fc_kernel_spectrum_device + fc_conv3d_kspec_device)
and the Richardson-Lucy driver (fc_rl_deconvolve_device).

Tolerances: convolution / correlation against the FP64 oracle rel-L2 <= 1e-5
and max-abs <= 1e-5 * max|ref| (same bar as the plain path); against the
plain entry with the same kernel rel-L2 <= 1e-7 (same passes, same
arithmetic); Richardson-Lucy against the FP64 restatement rel-L2 <= 2e-5
after 10 iterations (each iteration is two convolutions and a division, so
the fp32 rounding of ~20 transforms accumulates).
"""
import numpy as np
import pytest

import fourierconvolutioncudalib_gb300 as fc

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def _case(shape, kshape, seed):
    rng = np.random.default_rng(seed)
    im = (1 + rng.random(shape)).astype(np.float32)
    k = rng.random(kshape).astype(np.float32)
    return im, k / k.sum()


@pytest.mark.parametrize("shape,kshape", [((64, 128, 128), (9, 7, 5)), ((48, 96, 160), (11, 9, 7)),
                                          ((13, 34, 221), (3, 5, 7))])
def test_kspec_conv_matches_plain_and_fp64(cuda, orc, shape, kshape):
    import torch
    from fourierconvolutioncudalib_gb300 import device as fcd

    im, k = _case(shape, kshape, sum(shape))
    img = torch.from_numpy(im).to(cuda)
    ker = torch.from_numpy(k).to(cuda)
    ks = fcd.kernel_spectrum(ker, shape)
    got = fcd.conv3d_kspec(img, ks, kshape)
    plain = fcd.conv3d(img, ker)
    torch.cuda.synchronize()
    g = got.cpu().numpy()
    ref = orc.conv_fp64(im, k, "centered")
    assert _rel(g, ref) <= 1e-5
    assert np.max(np.abs(g - ref)) <= 1e-5 * np.max(np.abs(ref))
    assert _rel(g, plain.cpu().numpy()) <= 1e-7


def test_kspec_reused_for_many_images_and_correlation(cuda, orc):
    import torch
    from fourierconvolutioncudalib_gb300 import device as fcd

    shape, kshape = (40, 64, 96), (7, 9, 5)
    _, k = _case(shape, kshape, 3)
    ker = torch.from_numpy(k).to(cuda)
    ks = fcd.kernel_spectrum(ker, shape)
    rng = np.random.default_rng(4)
    for _ in range(3):
        im = rng.random(shape).astype(np.float32)
        img = torch.from_numpy(im).to(cuda)
        conv = fcd.conv3d_kspec(img, ks, kshape)
        corr = fcd.conv3d_kspec(img, ks, kshape, correlate=True)
        torch.cuda.synchronize()
        assert _rel(conv.cpu().numpy(), orc.conv_fp64(im, k, "centered")) <= 1e-5
        cref = orc.correlate_fp64(im, k)
        assert _rel(corr.cpu().numpy(), cref) <= 1e-5
        # odd kernel edges: correlation is the convolution with the kernel flipped about its centre
        flipped = np.ascontiguousarray(k[::-1, ::-1, ::-1])
        assert _rel(cref, orc.conv_fp64(im, flipped, "centered")) <= 1e-12


def test_kspec_rejects_compat_and_small_buffer(cuda):
    import torch
    from fourierconvolutioncudalib_gb300 import device as fcd

    ker = torch.ones((3, 3, 3), device=cuda) / 27
    with pytest.raises(fc.FcError):
        fcd.kernel_spectrum(ker, (8, 8, 8), flags=fc.FC_FLAG_SHIFT_COMPAT)
    L = fcd.lib()
    small = torch.empty(256, dtype=torch.uint8, device=cuda)
    rc = L.fc_kernel_spectrum_device(ker.data_ptr(), fc._iarr([3, 3, 3]), fc._iarr([8, 8, 8]), 0, small.data_ptr(),
                                     256, None)
    assert rc == fc.FC_ERR_NOMEM


# x extents 40 and 56 run on the generic kernels, 64 and 96 on the register-resident ones
@pytest.mark.parametrize("shape,kshape", [((32, 48, 40), (9, 5, 7)), ((24, 40, 56), (5, 7, 3)),
                                          ((32, 48, 64), (9, 5, 7)), ((20, 32, 96), (5, 7, 9))])
def test_richardson_lucy_vs_fp64(cuda, orc, shape, kshape):
    import torch
    from fourierconvolutioncudalib_gb300 import device as fcd

    rng = np.random.default_rng(sum(shape))
    truth = np.zeros(shape, np.float64)
    idx = tuple(rng.integers(0, s, 60) for s in shape)
    truth[idx] = rng.uniform(50, 500, 60)
    truth += 1.0
    k = rng.random(kshape)
    k = (k / k.sum()).astype(np.float32)
    y = np.maximum(orc.conv_fp64(truth, k, "centered"), 0).astype(np.float32)
    iters = 10
    ref = orc.rl_fp64(y, k, iters)
    got = fcd.rl_deconvolve(torch.from_numpy(y).to(cuda), torch.from_numpy(k).to(cuda), iters)
    torch.cuda.synchronize()
    g = got.cpu().numpy()
    rel = _rel(g, ref)
    print(f"RL {shape} k{kshape} {iters} it: rel-L2 vs FP64 {rel:.2e}")
    assert rel <= 2e-5
    # the update conserves the observed flux (unit-sum kernel, circular, est > 0)
    assert abs(g.astype(np.float64).sum() / y.astype(np.float64).sum() - 1) <= 1e-5
    # and moves the estimate towards the truth
    assert _rel(g, truth) < _rel(y, truth)


def test_richardson_lucy_zero_iterations_keeps_estimate(cuda):
    import torch
    from fourierconvolutioncudalib_gb300 import device as fcd

    y = torch.rand((16, 16, 16), device=cuda) + 1
    x0 = torch.rand((16, 16, 16), device=cuda)
    x = fcd.rl_deconvolve(y, torch.ones((3, 3, 3), device=cuda) / 27, 0, estimate=x0.clone())
    torch.cuda.synchronize()
    assert torch.equal(x, x0)
