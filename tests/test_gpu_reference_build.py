"""Parity against the reference library's own GPU build (cuFFT), same GPU.

The reference is compiled from its unmodified sources (oracle/build_ref.sh) and
run in a child process (oracle/reference_gpu.py).  Cases:

  * shapes on which the reference InPlace entry places the kernel where it
    intends (nx == nz and kx == kz; src/convolution3Dfft.cu:128-166 decomposes
    the tap index with the kernel's z extent fastest and stores it with the
    image's z extent fastest): our default entry against the reference's
    output;
  * non-cubic shapes, where that placement scrambles the kernel: our
    reference-arithmetic placement (FC_FLAG_SHIFT_COMPAT) against the
    reference's output;
  * the reference's convolution3DfftCUDA (src/convolution3Dfft.cu:299-391),
    whose packed input is transformed as if it had the padded in-place layout,
    against the FP64 oracle;
  * the subsampled-kernel variant against the reference's own device product
    (src/convolution3Dfft.cu:65-125, driven by oracle/ref_subsampled.cu), on
    every x frequency but DC and Nyquist, where that product is not Hermitian;
  * the device-query exports.

Tolerance: rel-L2 <= 1e-5 and max-abs <= 1e-5 * max|reference output|; the
FP64-oracle error of both outputs is checked and printed.  Every shape passed
to the reference is first checked by the oracle's restatement of its
placement, which refuses shapes whose taps would land outside the buffer.
"""
import numpy as np
import pytest

import fourierconvolutioncudalib_gb300 as fc

REL_TOL = 1e-5
MAXABS_TOL = 1e-5

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def refgpu(cuda):
    from oracle import reference_gpu

    if not reference_gpu.available():
        pytest.skip("the reference library could not be built here (its sources travel in oracle/_ref/src)")
    return reference_gpu


def _cmp(out, ref):
    from oracle import oracle as orc

    r = orc.rel_l2(out, ref)
    m = orc.max_abs(out, ref) / (float(np.max(np.abs(ref))) or 1.0)
    return r, m


def _check(out, ref, what):
    r, m = _cmp(out, ref)
    print(f"{what}: rel-L2 {r:.3e}, max-abs/max {m:.3e}")
    assert r <= REL_TOL, f"{what}: rel-L2 {r:.3e} > {REL_TOL}"
    assert m <= MAXABS_TOL, f"{what}: max-abs {m:.3e} > {MAXABS_TOL} * max"


def _gauss(shape_zyx, sig_zyx):
    zz, yy, xx = [np.arange(n) - n // 2 for n in shape_zyx]
    g = np.exp(-(zz[:, None, None] / sig_zyx[0]) ** 2 / 2 - (yy[None, :, None] / sig_zyx[1]) ** 2 / 2
               - (xx[None, None, :] / sig_zyx[2]) ** 2 / 2)
    return (g / g.sum()).astype(np.float32)


def _ours(im, k, compat=False):
    lib = fc.load_library()
    out = np.ascontiguousarray(im, np.float32).copy()
    nz, ny, nx = im.shape
    kz, ky, kx = k.shape
    lib.fc_set_shift_compat(1 if compat else 0)
    try:
        fc.convolution3DfftCUDAInPlace(out, (nx, ny, nz), np.ascontiguousarray(k, np.float32), (kx, ky, kz), 0)
    finally:
        lib.fc_set_shift_compat(0)
    return out


def _consistent_cases():
    from fourierconvolutioncudalib_gb300 import workloads as W

    rng = np.random.Generator(np.random.PCG64(11))
    c1 = W.c1()
    c3 = W.c3()
    return [
        ("c1_64^3_k7^3", c1["image"], c1["kernel"]),
        ("c3_256^3_k21^3", c3["x_true"], c3["k_true"]),
        ("96x80x96_k9x5x9", rng.random((96, 80, 96)).astype(np.float32), _gauss((9, 5, 9), (2.0, 1.0, 1.5))),
        ("45x33x45_k7x4x7", rng.random((45, 33, 45)).astype(np.float32), _gauss((7, 4, 7), (1.5, 1.0, 1.2))),
        ("128x256x128_k31x15x31", rng.random((128, 256, 128)).astype(np.float32),
         _gauss((31, 15, 31), (4.0, 2.0, 3.0))),
    ]


def test_inplace_matches_reference_build_on_consistent_shapes(refgpu, orc):
    cases = _consistent_cases()
    for name, im, k in cases:
        # the reference's placement equals the centred one on these shapes (bit-exact buffers)
        np.testing.assert_array_equal(orc.ref_inplace_padded_kernel(k, im.shape),
                                      orc.centered_padded_kernel(k, im.shape))
    refs = refgpu.inplace_many([(im, k) for _, im, k in cases])
    for (name, im, k), ref in zip(cases, refs):
        ours = _ours(im, k)
        exact = orc.conv_fp64(im, k, "centered")
        rr, rm = _cmp(ref, exact)
        print(f"{name}: reference build vs FP64 rel-L2 {rr:.3e} max {rm:.3e}")
        _check(ours, ref, f"{name} ours vs reference build")
        _check(ours, exact, f"{name} ours vs FP64")


def _compat_cases():
    from fourierconvolutioncudalib_gb300 import workloads as W

    rng = np.random.Generator(np.random.PCG64(12))
    c2 = W.c2()
    return [
        ("c2a_512x512x128_k31x31x63", c2["image"], c2["kernel"]),
        ("24x20x30_k5x3x7", rng.random((24, 20, 30)).astype(np.float32),
         rng.random((5, 3, 7)).astype(np.float32)),
        ("96x448x384_k63x31x31", rng.random((96, 448, 384)).astype(np.float32), _gauss((63, 31, 31), (4, 1.5, 1.5))),
        ("21x19x15_k3x3x3_prime_extents", rng.random((21, 19, 15)).astype(np.float32),
         rng.random((3, 3, 3)).astype(np.float32)),
    ]


def test_shift_compat_matches_reference_build_on_noncubic_shapes(refgpu, orc):
    cases = _compat_cases()
    for name, im, k in cases:
        orc.ref_inplace_padded_kernel(k, im.shape)  # raises if the reference would write outside its buffer
    refs = refgpu.inplace_many([(im, k) for _, im, k in cases])
    for (name, im, k), ref in zip(cases, refs):
        ours = _ours(im, k, compat=True)
        exact = orc.conv_fp64(im, k, "reference_inplace")
        rr, rm = _cmp(ref, exact)
        print(f"{name}: reference build vs FP64 (reference placement) rel-L2 {rr:.3e} max {rm:.3e}")
        _check(ours, ref, f"{name} ours (compat) vs reference build")
        _check(ours, exact, f"{name} ours (compat) vs FP64")


def test_reference_kats_through_reference_build(refgpu, orc):
    """The reference test suite's small known-answer cases through the
    reference build and through ours (compat placement), outputs compared."""
    cases = [c for c in orc.kat_cases(include_large=False)]
    refs = refgpu.inplace_many([(c["image"], c["kernel"]) for c in cases])
    for c, ref in zip(cases, refs):
        ours = _ours(c["image"], c["kernel"], compat=True)
        scale = float(np.max(np.abs(ref))) or 1.0
        d = float(np.max(np.abs(ours.astype(np.float64) - ref))) / scale
        print(f"{c['name']}: ours vs reference build max-abs/max {d:.3e}")
        assert d <= 1e-5, c["name"]


def test_reference_noninplace_entry_layout(refgpu, orc):
    """convolution3DfftCUDA of the reference hands its packed image to an
    in-place cuFFT R2C plan, which reads rows at the padded pitch
    2*(nx/2+1) (src/convolution3Dfft.cu:330-368): its output is not the
    convolution.  Ours computes the convolution."""
    from fourierconvolutioncudalib_gb300 import workloads as W

    c1 = W.c1()
    im, k = c1["image"], c1["kernel"]
    exact = orc.conv_fp64(im, k, "centered")
    ref = refgpu.noninplace(im, k)
    rr, rm = _cmp(ref, exact)
    print(f"reference convolution3DfftCUDA vs FP64 on 64^3/7^3: rel-L2 {rr:.3e}, max-abs/max {rm:.3e}")
    assert rr > 1e-2, "the reference's non-in-place entry matched the convolution"
    dims = (64, 64, 64)
    ours = fc.convolution3DfftCUDA(np.ascontiguousarray(im), dims, k, (7, 7, 7), 0)
    _check(ours, exact, "ours convolution3DfftCUDA vs FP64")


@pytest.mark.parametrize("shape,kshape", [((64, 128, 128), (16, 10, 12)), ((128, 512, 512), (62, 31, 30)),
                                          ((96, 64, 256), (15, 9, 24))])
def test_subsampled_matches_reference_product(refgpu, orc, shape, kshape):
    """convolution3DfftCUDAInPlaceSaveMemory against the reference's own
    subsampled-kernel product (modulateAndNormalizeSubsampled_kernel,
    src/convolution3Dfft.cu:65-125) driven on cuFFT by oracle/ref_subsampled.cu,
    and against the FP64 restatement.  Image extents are powers of two, so the
    ratio k/n is exact in float32 under the reference's fast-math division and
    the nearest-coefficient indices agree; kernel x extents are even, where the
    reference reads inside its half-spectrum rows (for odd ones it reads one
    coefficient past a row at the x Nyquist, where this library takes the
    Hermitian mirror).

    The nearest-coefficient product is not Hermitian on the x DC and Nyquist
    planes (index ties round up on both sides of zero), and what an inverse
    real transform does with the imaginary parts there is left to the
    implementation: this library drops them after the z and y inverses, as
    numpy's irfftn does; cuFFT's C2R agrees at x = 512 and differs at x = 128
    and 256.  Any treatment of those two bins changes the output only by a
    term of period 2 along x, so the reference's output is compared on every
    other x frequency (its spectrum at 0 < fx < nx/2), and the whole output
    against the FP64 restatement."""
    rng = np.random.Generator(np.random.PCG64(sum(shape)))
    im = rng.random(shape).astype(np.float32)
    k = _gauss(kshape, (kshape[0] / 6, kshape[1] / 6, kshape[2] / 6))
    ref = refgpu.subsampled(im, k)
    ours = np.ascontiguousarray(im).copy()
    nz, ny, nx = shape
    kz, ky, kx = kshape
    fc.convolution3DfftCUDAInPlaceSaveMemory(ours, (nx, ny, nz), k, (kx, ky, kz), 0)
    exact = orc.subsampled_fp64(im, k)
    rr, rm = _cmp(ref, exact)
    print(f"{shape} {kshape}: reference product vs FP64 restatement, whole output: rel-L2 {rr:.3e} max {rm:.3e}")
    band = (slice(None), slice(None), slice(1, nx // 2))
    fr = np.fft.rfftn(ref.astype(np.float64))[band]
    fo = np.fft.rfftn(ours.astype(np.float64))[band]
    fe = np.fft.rfftn(exact)[band]
    rb = float(np.linalg.norm(fo - fr) / np.linalg.norm(fr))
    re_ = float(np.linalg.norm(fr - fe) / np.linalg.norm(fe))
    print(f"{shape} {kshape}: x frequencies 0 < fx < nx/2: ours vs reference rel-L2 {rb:.3e}, "
          f"reference vs FP64 {re_:.3e}")
    assert rb <= REL_TOL, f"ours vs reference product off the x DC/Nyquist planes: rel-L2 {rb:.3e}"
    _check(ours, exact, f"{shape} {kshape} ours vs FP64 restatement")


def test_device_queries_match_reference_build(refgpu, fclib):
    import ctypes

    q = refgpu.device_queries(0)
    assert fclib.getNumDevicesCUDA() == q["num_devices"]
    assert fclib.getCUDAcomputeCapabilityMajorVersion(0) == q["cc_major"]
    assert fclib.getCUDAcomputeCapabilityMinorVersion(0) == q["cc_minor"]
    assert fclib.selectDeviceWithHighestComputeCapability() == q["highest_cc_device"]
    assert fclib.getMemDeviceCUDA(0) == q["mem"]
    name = ctypes.create_string_buffer(256)
    fclib.getNameDeviceCUDA(0, name)
    assert name.value.decode() == q["name"]
    assert fclib.cuda_version() == q["cuda_version"]
    print(q)
