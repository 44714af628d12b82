"""The adjoint (differentiation) form of the convolution.

grad_image = corr(g, k) and grad_kernel = crop_K(corr(x, g)) from
fc_conv3d_adjoint_device, through a torch.autograd.Function.

Checks and tolerances:
  * the adjoint operator against FP64 FFT formulas of both gradients, for a
    given upstream gradient: rel-L2 <= 1e-5
  * the least-squares loss 0.5*||conv(x,k) - y||^2 through autograd (float32
    forward + adjoint) against FP64: rel-L2 <= 1e-4.  The residual
    conv(x,k) - y is about 100x smaller than conv(x,k), so the float32
    rounding of the forward output (~1e-7 relative, mostly a constant offset
    from the DC bin) reaches ~1e-5 relative in the residual and hence in the
    gradients; the operator itself is held to 1e-5 on the FP64 residual.
  * FP64 central differences (eps = 1e-3) of that loss at 64 random image
    and 64 random kernel coordinates: |diff| <= 1e-4 * max|grad| + 1e-4 * |fd|
  * grad_image against the reference algorithm convolving g with the
    flipped kernel (cuFFT restatement, odd kernel edges): rel-L2 <= 1e-5
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(params=["fast", "generic"])
def kernels(request, fclib):
    fclib.fc_set_generic_kernels(1 if request.param == "generic" else 0)
    yield request.param
    fclib.fc_set_generic_kernels(0)


def fp64_grads(x, k, g, orc):
    """grad_x = irfft(G * conj(P)), grad_P = irfft(conj(X) * G), grad_k = crop of grad_P."""
    P = orc.centered_padded_kernel(k, x.shape).astype(np.float64)
    ax = (0, 1, 2)
    G = np.fft.rfftn(g.astype(np.float64))
    gx = np.fft.irfftn(G * np.conj(np.fft.rfftn(P)), s=x.shape, axes=ax)
    gP = np.fft.irfftn(np.conj(np.fft.rfftn(x.astype(np.float64))) * G, s=x.shape, axes=ax)
    kz, ky, kx = k.shape
    nz, ny, nx = x.shape
    iz = (np.arange(kz) - kz // 2) % nz
    iy = (np.arange(ky) - ky // 2) % ny
    ix = (np.arange(kx) - kx // 2) % nx
    return gx, gP[np.ix_(iz, iy, ix)]


def rel(a, b):
    return float(np.linalg.norm((np.asarray(a, np.float64) - b).ravel()) / np.linalg.norm(b.ravel()))


@pytest.mark.parametrize("shape,kshape", [((24, 20, 30), (5, 3, 7)), ((32, 64, 64), (7, 7, 7)),
                                          ((16, 32, 48), (4, 6, 3)), ((13, 17, 19), (3, 5, 3))])
def test_adjoint_vs_fp64(cuda, orc, kernels, shape, kshape):
    import torch
    from fourierconvolutioncudalib_gb300 import device as fcd

    rng = np.random.default_rng(sum(shape))
    x = rng.standard_normal(shape).astype(np.float32)
    k = rng.random(kshape).astype(np.float32)
    g = rng.standard_normal(shape).astype(np.float32)
    gi, gk = fcd.conv3d_adjoint(torch.from_numpy(x).to(cuda), torch.from_numpy(k).to(cuda),
                                torch.from_numpy(g).to(cuda), kshape)
    ex, ek = fp64_grads(x, k, g, orc)
    assert rel(gi.cpu().numpy(), ex) <= 1e-5
    assert rel(gk.cpu().numpy(), ek) <= 1e-5
    # one gradient at a time
    gi2, gk2 = fcd.conv3d_adjoint(None, torch.from_numpy(k).to(cuda), torch.from_numpy(g).to(cuda), kshape,
                                  need_kernel_grad=False)
    assert gk2 is None and rel(gi2.cpu().numpy(), ex) <= 1e-5
    gi3, gk3 = fcd.conv3d_adjoint(torch.from_numpy(x).to(cuda), None, torch.from_numpy(g).to(cuda), kshape,
                                  need_image_grad=False)
    assert gi3 is None and rel(gk3.cpu().numpy(), ek) <= 1e-5


def test_autograd_least_squares_c3(cuda, orc):
    """The differentiation configuration: 256^3 image with 5000 spots, 21^3
    perturbed Gaussian kernel, y = conv(x_true, k_true) + N(0,1), x and k
    perturbed by 10 % multiplicative noise, loss 0.5*||conv(x,k) - y||^2."""
    import torch
    from fc_autograd import fourier_conv3d
    from fourierconvolutioncudalib_gb300 import workloads as W

    d = W.c3()
    x_true, k_true, x0, k0 = d["x_true"], d["k_true"], d["image"], d["kernel"]
    rng = np.random.Generator(np.random.PCG64(40))
    y = (orc.conv_fp64(x_true, k_true, "centered") + rng.standard_normal(x_true.shape)).astype(np.float32)

    xt = torch.from_numpy(x0).to(cuda).requires_grad_(True)
    kt = torch.from_numpy(k0).to(cuda).requires_grad_(True)
    yt = torch.from_numpy(y).to(cuda)
    out = fourier_conv3d(xt, kt)
    loss = 0.5 * ((out - yt) ** 2).sum()
    loss.backward()
    gx = xt.grad.cpu().numpy()
    gk = kt.grad.cpu().numpy()

    # FP64 residual and gradients
    r = orc.conv_fp64(x0, k0, "centered") - y.astype(np.float64)
    ex, ek = fp64_grads(x0, k0, r, orc)
    assert rel(gx, ex) <= 1e-4
    assert rel(gk, ek) <= 1e-4
    # the adjoint operator alone, driven by the FP64 residual
    from fourierconvolutioncudalib_gb300 import device as fcd

    gi_op, gk_op = fcd.conv3d_adjoint(torch.from_numpy(x0).to(cuda), torch.from_numpy(k0).to(cuda),
                                      torch.from_numpy(r.astype(np.float32)).to(cuda), k0.shape)
    assert rel(gi_op.cpu().numpy(), ex) <= 1e-5
    assert rel(gk_op.cpu().numpy(), ek) <= 1e-5

    # FP64 central differences, eps = 1e-3, evaluated exactly on the affected voxels:
    # L(x + e*d_i) - L(x - e*d_i) = sum_p [(r_p + e*P_{p-i})^2 - (r_p - e*P_{p-i})^2] / 2
    eps = 1e-3
    nz, ny, nx = x0.shape
    kz, ky, kx = k0.shape
    pick = np.random.default_rng(64)
    k64 = k0.astype(np.float64)
    for _ in range(64):
        i = [int(pick.integers(s)) for s in x0.shape]
        zz = (i[0] + np.arange(kz) - kz // 2) % nz
        yy = (i[1] + np.arange(ky) - ky // 2) % ny
        xx = (i[2] + np.arange(kx) - kx // 2) % nx
        rl = r[np.ix_(zz, yy, xx)]
        fd = (np.sum((rl + eps * k64) ** 2) - np.sum((rl - eps * k64) ** 2)) / 2 / (2 * eps)
        assert abs(gx[tuple(i)] - fd) <= 1e-4 * np.max(np.abs(ex)) + 1e-4 * abs(fd)
    x64 = x0.astype(np.float64)
    for _ in range(64):
        j = [int(pick.integers(s)) for s in k0.shape]
        shift = [j[0] - kz // 2, j[1] - ky // 2, j[2] - kx // 2]
        xs = np.roll(x64, shift, axis=(0, 1, 2))
        fd = (np.sum((r + eps * xs) ** 2) - np.sum((r - eps * xs) ** 2)) / 2 / (2 * eps)
        assert abs(gk[tuple(j)] - fd) <= 1e-4 * np.max(np.abs(ek)) + 1e-4 * abs(fd)


def test_grad_image_is_flipped_kernel_convolution(cuda, orc):
    """grad_image = conv(g, flip(k)) for odd kernel edges; checked against the
    reference's algorithm (cuFFT restatement) run with the flipped kernel."""
    import torch
    from baseline import refseq
    from fourierconvolutioncudalib_gb300 import device as fcd

    rng = np.random.default_rng(8)
    shape, kshape = (64, 96, 128), (7, 9, 5)
    g = rng.standard_normal(shape).astype(np.float32)
    k = rng.random(kshape).astype(np.float32)
    gi, _ = fcd.conv3d_adjoint(None, torch.from_numpy(k).to(cuda), torch.from_numpy(g).to(cuda), kshape,
                               need_kernel_grad=False)
    ref = refseq.inplace(g, np.ascontiguousarray(k[::-1, ::-1, ::-1]), centered=True)
    assert rel(gi.cpu().numpy(), ref.astype(np.float64)) <= 1e-5
