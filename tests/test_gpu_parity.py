"""Parity of the CUDA path with the oracle, through the C ABI.

Tolerances (float32 path against references):
  * against the FP64 oracle and the cuFFT restatement of the reference:
    rel-L2 <= 1e-5 and max-abs <= 1e-5 * max|out|   (REL_TOL, MAXABS_TOL)
  * padded kernel buffers: bit-exact
  * the reference's own KAT thresholds on its sqrt(sum d^2)/N metric, as
    written in its tests
"""
import numpy as np
import pytest

import fourierconvolutioncudalib_gb300 as fc

REL_TOL = 1e-5
MAXABS_TOL = 1e-5

pytestmark = pytest.mark.gpu


@pytest.fixture(params=["copy", "direct"])
def host_io(request, fclib):
    """convolution3DfftCUDAInPlace with staged copies, and with the passes
    reading and writing the caller's host buffer directly (GB300 accesses
    pageable host memory through the host page tables)."""
    fclib.fc_set_host_io(0 if request.param == "copy" else 1)
    yield request.param
    fclib.fc_set_host_io(2)


@pytest.fixture(params=["fast", "generic"])
def kernels(request, fclib):
    """Run a test on the register-resident kernels (power-of-two axes) and on
    the generic shared-memory kernels (forced on every axis)."""
    fclib.fc_set_generic_kernels(1 if request.param == "generic" else 0)
    yield request.param
    fclib.fc_set_generic_kernels(0)


def _check(out, ref, rel=REL_TOL, mx=MAXABS_TOL):
    from oracle import oracle as orc

    r = orc.rel_l2(out, ref)
    m = orc.max_abs(out, ref)
    scale = float(np.max(np.abs(ref))) or 1.0
    assert r <= rel, f"rel-L2 {r:.3e} > {rel}"
    assert m <= mx * scale, f"max-abs {m:.3e} > {mx} * {scale:.3e}"
    return r, m / scale


def _gauss(k, s):
    r = np.arange(k) - k // 2
    g = np.exp(-(r[:, None, None] ** 2 + r[None, :, None] ** 2 + r[None, None, :] ** 2) / (2 * s * s))
    return (g / g.sum()).astype(np.float32)


def test_c1_plain_small_vs_fp64(cuda, orc, kernels, host_io):
    # 64^3 uniform[0,1) (seed 1), 7^3 isotropic Gaussian sigma 1.5 normalised
    rng = np.random.Generator(np.random.PCG64(1))
    im = rng.random((64, 64, 64)).astype(np.float32)
    k = _gauss(7, 1.5)
    ref = orc.conv_fp64(im, k, "centered")
    out = im.copy()
    fc.convolution3DfftCUDAInPlace(out, (64, 64, 64), k, (7, 7, 7), 0)
    _check(out, ref)
    # cubic image and kernel: the reference's own placement coincides
    _check(out, orc.conv_fp64(im, k, "reference_inplace"))


def test_c1_vs_cufft_sequence(cuda, orc, kernels):
    from baseline import refseq

    rng = np.random.Generator(np.random.PCG64(1))
    im = rng.random((64, 64, 64)).astype(np.float32)
    k = _gauss(7, 1.5)
    out = im.copy()
    fc.convolution3DfftCUDAInPlace(out, (64, 64, 64), k, (7, 7, 7), 0)
    ref = refseq.inplace(im, k, centered=False)
    _check(out, ref)


@pytest.mark.parametrize("shape,kshape", [
    ((24, 20, 30), (5, 3, 7)),        # non-cubic, odd kernel
    ((21, 19, 15), (3, 3, 3)),        # the prime-shape KAT extents (x,y,z)=(15,19,21)
    ((13, 17, 19), (3, 5, 7)),        # odd nx (19): two-rows-per-FFT R2C path
    ((7, 49, 343), (3, 3, 3)),        # radix 7 everywhere
    ((5, 25, 125), (3, 5, 5)),        # radix 5
    ((9, 27, 3), (3, 3, 3)),          # radix 3
    ((32, 16, 8), (4, 2, 6)),         # even kernel dims
    ((1, 64, 64), (1, 5, 5)),         # a 2D image as a 1-plane volume
    ((22, 26, 34), (11, 13, 17)),     # radix 11 and 13 and a generic prime (17)
    ((37, 79, 109), (5, 5, 5)),       # large primes from the padded reference KAT extents
    ((128, 512, 512), (63, 31, 31)),  # the microscope configuration's shapes
    ((64, 256, 1024), (9, 9, 9)),     # 1024 rows
    ((16, 2048, 128), (3, 5, 3)),     # a 2048 column axis (wide y tiles; generic kernel y pass)
    ((256, 64, 32), (5, 3, 3)),       # short rows, long z
    ((96, 448, 384), (63, 31, 31)),   # the non-power-of-two microscope configuration (radices 16, 14, 12, 6, 2)
    ((160, 288, 320), (21, 25, 23)),  # batch-view lengths: radices 10 and 9
    ((64, 352, 400), (9, 11, 13)),    # radices 11 and 5
    ((200, 96, 224), (7, 5, 9)),      # radix 10 chain along z, 14 along x
    ((100, 500, 500), (21, 15, 15)),  # common stack extents: 10x10, 10x10x5
    ((60, 120, 1000), (9, 7, 5)),     # 1000 rows (10x10x10), 12x10 columns, 15x4 along z
    ((150, 360, 72), (11, 9, 7)),     # 15x10 along z, 15x12x2 columns, 12x6 rows
    ((24, 900, 20), (5, 7, 3)),       # 15x15x4 columns, short rows of 20
    ((250, 48, 64), (9, 5, 7)),       # z lengths whose fused-z tiles are 8 and 4 columns wide
    ((500, 20, 30), (7, 3, 5)),
    ((900, 24, 20), (11, 5, 3)),
    ((16, 64, 48), (3, 7, 5)),        # kernel rows exactly fill the kernel y pass's first-stage stride (4)
    ((20, 64, 40), (3, 15, 5)),       # kernel rows beyond that stride: full first stage
])
def test_shapes_vs_fp64(cuda, orc, kernels, host_io, shape, kshape):
    rng = np.random.default_rng(sum(shape) + sum(kshape))
    im = rng.random(shape, dtype=np.float32)
    k = rng.random(kshape, dtype=np.float32)
    k /= k.sum()
    ref = orc.conv_fp64(im, k, "centered")
    out = im.copy()
    nz, ny, nx = shape
    kz, ky, kx = kshape
    fc.convolution3DfftCUDAInPlace(out, (nx, ny, nz), k, (kx, ky, kz), 0)
    _check(out, ref)


def test_reference_kats(cuda, orc, kernels, host_io):
    """Every convolution known-answer case of the reference test suite, through
    convolution3DfftCUDAInPlace with the reference's padding protocol."""
    for case in orc.kat_cases(include_large=True):
        im = case["image"].copy()
        k = case["kernel"]
        nz, ny, nx = im.shape
        kz, ky, kx = k.shape
        fc.convolution3DfftCUDAInPlace(im, (nx, ny, nz), k, (kx, ky, kz), 0)
        got = orc.crop(im, case["off"], case["shape"])
        exp = case["expected"]
        if case["metric"] == "sum":
            s, e = float(np.sum(got, dtype=np.float64)), float(np.sum(exp, dtype=np.float64))
            # the reference checks the crop's sum (BOOST_CHECK_CLOSE); compared here in float64
            assert abs(s - e) <= 1e-6 * max(1.0, abs(e)), (case["name"], s, e)
        if np.any(exp):
            r = orc.rel_l2(got, exp)
            assert r <= 1e-5, (case["name"], r)
        else:
            assert np.max(np.abs(got)) <= 1e-6, case["name"]
        # the reference's own assertion, as written in its test
        if case["metric"] == "l2norm":
            re = case.get("reference_expected", exp)
            assert orc.l2norm(re, got) < case["threshold"], case["name"]


def test_shift_compat_matches_reference_arithmetic(cuda, orc, kernels):
    """With the reference's placement arithmetic the result equals the FP64
    oracle of that (scrambled) placement on non-cubic shapes."""
    rng = np.random.default_rng(7)
    for shape, kshape in [((21, 19, 15), (3, 3, 3)), ((6, 10, 12), (5, 3, 3)), ((16, 16, 8), (7, 5, 5))]:
        im = rng.random(shape, dtype=np.float32)
        k = rng.random(kshape, dtype=np.float32)
        nz, ny, nx = shape
        kz, ky, kx = kshape
        out = im.copy()
        fc.lib().fc_set_shift_compat(1)
        try:
            fc.convolution3DfftCUDAInPlace(out, (nx, ny, nz), k, (kx, ky, kz), 0)
        finally:
            fc.lib().fc_set_shift_compat(0)
        _check(out, orc.conv_fp64(im, k, "reference_inplace"))


def test_padded_kernel_bit_exact(cuda, orc):
    """The padded + shifted kernel buffer is bit-identical to the reference's
    (compat) and to the centred placement (default)."""
    import torch
    from fourierconvolutioncudalib_gb300 import device as fcd

    rng = np.random.default_rng(3)
    for shape, kshape in [((128, 512, 512), (63, 31, 31)), ((21, 19, 15), (3, 3, 3)), ((6, 10, 12), (5, 3, 3)),
                          ((64, 64, 64), (7, 7, 7)), ((96, 448, 384), (63, 31, 31))]:
        k = rng.standard_normal(kshape).astype(np.float32)
        kt = torch.from_numpy(k).to(cuda)
        got_c = fcd.pad_shift_kernel(kt, shape, flags=fc.FC_FLAG_SHIFT_COMPAT).cpu().numpy()
        got_d = fcd.pad_shift_kernel(kt, shape, flags=0).cpu().numpy()
        assert np.array_equal(got_c.view(np.uint32), orc.ref_inplace_padded_kernel(k, shape).view(np.uint32))
        assert np.array_equal(got_d.view(np.uint32), orc.centered_padded_kernel(k, shape).view(np.uint32))


def test_non_inplace_entries(cuda, orc, kernels):
    rng = np.random.default_rng(11)
    im = rng.random((20, 24, 18), dtype=np.float32)   # dims slowest-first (d0,d1,d2)
    k = rng.random((5, 3, 7), dtype=np.float32)
    out = fc.convolution3DfftCUDA(im, im.shape, k, k.shape, 0)
    _check(out, orc.conv_fp64(im, k, "centered"))
    # the non-in-place entry's own placement (consistent dims) is the centred one
    assert np.array_equal(orc.ref_packed_padded_kernel(k, im.shape), orc.centered_padded_kernel(k, im.shape))
    pk = orc.centered_padded_kernel(k, im.shape)
    out2 = fc.convolution3DfftCUDA_test(im, im.shape, pk, 0)
    _check(out2, orc.fft_conv_fp64(im, pk))


def test_errors_leave_image_untouched(cuda):
    im = np.ones((8, 8, 8), np.float32)
    k = np.ones((3, 3, 3), np.float32)
    fc.lib().convolution3DfftCUDAInPlace(im.ctypes.data_as(fc._FP), fc._iarr([8, 8, 8]), k.ctypes.data_as(fc._FP),
                                         fc._iarr([3, 3, 3]), 99)
    assert fc.lib().fc_last_status() == fc.FC_ERR_ARG
    assert np.all(im == 1)
    with pytest.raises(fc.FcError):
        fc.convolution3DfftCUDAInPlace(im, (8, 8, 8), np.ones((9, 3, 3), np.float32), (3, 3, 9), 0)
    assert np.all(im == 1)
    res = fc.lib().convolution3DfftCUDA(im.ctypes.data_as(fc._FP), fc._iarr([8, 8, 8]), None, fc._iarr([3, 3, 3]), 0)
    assert not res
    assert fc.lib().fc_last_status() == fc.FC_ERR_ARG


def test_device_queries(cuda):
    n = fc.getNumDevicesCUDA()
    assert n >= 1
    d = fc.selectDeviceWithHighestComputeCapability()
    assert 0 <= d < n
    assert fc.getCUDAcomputeCapabilityMajorVersion(d) >= 10
    assert fc.getCUDAcomputeCapabilityMinorVersion(d) >= 0
    assert len(fc.getNameDeviceCUDA(d)) > 0
    assert fc.getMemDeviceCUDA(d) > (1 << 30)
    assert fc.cuda_version() >= 13000
    assert fc.gpu_mem_needed_mb([128, 512, 512]) > 0


@pytest.mark.parametrize("chunk_bytes", [0, 3 << 20, 17 << 20, -1])
def test_l2_column_chunks_equivalent(cuda, orc, kernels, chunk_bytes):
    """The y / fused-z / y-inverse passes run over kx column chunks sized for
    L2; every chunking gives the same result as none (and the oracle's)."""
    rng = np.random.default_rng(21)
    im = rng.random((32, 96, 200), dtype=np.float32)
    k = rng.random((7, 5, 9), dtype=np.float32)
    k /= k.sum()
    ref = orc.conv_fp64(im, k, "centered")
    out = im.copy()
    fc.lib().fc_set_l2_chunk_bytes(chunk_bytes)
    try:
        fc.convolution3DfftCUDAInPlace(out, (200, 96, 32), k, (9, 5, 7), 0)
    finally:
        fc.lib().fc_set_l2_chunk_bytes(0)
    _check(out, ref)
