"""The oracle pinned against the reference's own test data (CPU only).

Nothing here needs a GPU: the FP64 FFT oracle, the direct-sum restatement and
the placement restatement are checked against the reference test suite's
known answers (committed as tests/golden/ fixtures) and against each other.
"""
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden"


def _kat(name, z):
    g = lambda f: z[f"{name}/{f}"]
    return dict(image=g("image"), kernel=g("kernel"), off=list(g("off")), shape=tuple(g("shape")),
                expected=g("expected"), reference_expected=g("reference_expected"), threshold=float(g("threshold")))


def test_golden_kats_fp64_oracle(orc):
    """The FP64 oracle with the centred placement reproduces every small
    known-answer case exactly (to float64 round-off)."""
    z = np.load(GOLD / "kat_small.npz")
    for name in z["names"]:
        c = _kat(str(name), z)
        out = orc.crop(orc.conv_fp64(c["image"], c["kernel"], "centered"), c["off"], c["shape"])
        exp = c["expected"].astype(np.float64)
        assert np.max(np.abs(out - exp)) <= 1e-9 * max(1.0, np.max(np.abs(exp))), name
        # and the reference's own metric/threshold on its own expectation
        assert orc.l2norm(c["reference_expected"], out.astype(np.float32)) < max(c["threshold"], 1e-5), name


def test_golden_kats_regenerate(orc):
    """kat_cases() still produces the committed fixtures (the generator and
    the restated direct sum have not drifted)."""
    z = np.load(GOLD / "kat_small.npz")
    for c in orc.kat_cases(include_large=False):
        n = c["name"]
        assert np.array_equal(z[f"{n}/image"], c["image"]), n
        assert np.array_equal(z[f"{n}/expected"], c["expected"]), n


def test_reference_placement_hand_case(orc):
    z = np.load(GOLD / "placement.npz")
    k = z["hand/kernel"]
    assert np.array_equal(orc.ref_inplace_padded_kernel(k, (2, 3, 4)), z["hand/reference"])
    assert np.array_equal(orc.centered_padded_kernel(k, (2, 3, 4)), z["hand/centered"])


def test_reference_placement_fixtures(orc):
    z = np.load(GOLD / "placement.npz")
    for i in range(3):
        k = z[f"p{i}/kernel"]
        shape = tuple(z[f"p{i}/shape"])
        assert np.array_equal(orc.ref_inplace_padded_kernel(k, shape), z[f"p{i}/reference"])
        assert np.array_equal(orc.centered_padded_kernel(k, shape), z[f"p{i}/centered"])


@pytest.mark.parametrize("shape,kshape,same", [
    ((8, 8, 8), (3, 3, 3), True),        # nx == nz and kx == kz: the reference places correctly
    ((64, 64, 64), (7, 7, 7), True),
    ((6, 10, 12), (5, 3, 3), False),     # non-cubic: scrambled
    ((21, 19, 15), (3, 3, 3), False),
    ((16, 16, 16), (5, 5, 3), False),
])
def test_reference_placement_quirk(orc, shape, kshape, same):
    rng = np.random.default_rng(0)
    k = rng.random(kshape, dtype=np.float32)
    a = orc.ref_inplace_padded_kernel(k, shape)
    b = orc.centered_padded_kernel(k, shape)
    assert np.isclose(a.sum(), k.sum())
    assert np.array_equal(a, b) == same
    # a centred delta lands at the origin under either placement
    d = np.zeros(kshape, np.float32)
    d[kshape[0] // 2, kshape[1] // 2, kshape[2] // 2] = 1
    assert np.array_equal(orc.ref_inplace_padded_kernel(d, shape), orc.centered_padded_kernel(d, shape))


def test_closest_multiplier(orc):
    # src/convolution3Dfft.cu:26-38 returns the exact multiple or 32
    assert [orc.closest_multiplier(a) for a in (1, 27, 32, 33, 64, 343, 1000, 1024)] == [32, 32, 32, 32, 64, 32, 32,
                                                                                      1024]


def test_direct_sum_matches_fft_oracle(orc):
    """The restated reference CPU convolution (periodic variant) equals the FP64
    FFT oracle for odd kernels; interior-only variant on a padded image."""
    rng = np.random.default_rng(5)
    im = rng.random((10, 12, 14), dtype=np.float32)
    k = rng.random((3, 5, 3), dtype=np.float32)
    d = orc.convolve_direct(im, k, periodic=True)
    f = orc.conv_fp64(im, k, "centered")
    assert np.max(np.abs(d - f)) < 1e-5
    crop = orc.convolve_direct_crop(im, k, (2, 3, 4), (4, 5, 6))
    assert np.allclose(crop, d[2:6, 3:8, 4:10], atol=1e-6)
    padded, off = orc.zero_padd(im, k.shape)
    d2 = orc.convolve_direct(padded, k, offset=off)
    f2 = orc.conv_fp64(padded, k, "centered")
    assert np.max(np.abs(orc.crop(d2, off, im.shape) - orc.crop(f2, off, im.shape))) < 1e-5


def test_even_kernel_offset_convention(orc):
    """For an even kernel edge the reference's GPU path centres at k/2 while its
    CPU direct sum uses k-1-k/2: they differ by one voxel along that axis.  The
    library follows the GPU path (k/2)."""
    rng = np.random.default_rng(9)
    im = rng.random((6, 7, 8), dtype=np.float32)
    k = rng.random((1, 1, 4), dtype=np.float32)
    d = orc.convolve_direct(im, k, periodic=True)
    f = orc.conv_fp64(im, k, "centered")
    assert np.max(np.abs(np.roll(d, -1, axis=2) - f)) < 1e-5


def test_modulate_op_order(orc):
    rng = np.random.default_rng(2)
    a = (rng.standard_normal(64) + 1j * rng.standard_normal(64)).astype(np.complex64)
    b = (rng.standard_normal(64) + 1j * rng.standard_normal(64)).astype(np.complex64)
    d = b.copy()
    orc.modulate_and_normalize(d, a, 0.25)
    c = np.float32(0.25)
    ex = (c * (a.real * b.real - a.imag * b.imag)).astype(np.float32)
    ey = (c * (a.imag * b.real + a.real * b.imag)).astype(np.float32)
    assert np.allclose(d.real, ex, rtol=0, atol=1e-6) and np.allclose(d.imag, ey, rtol=0, atol=1e-6)


def test_reference_path_fp32_port(orc):
    """The float32 CPU port of the reference algorithm (scipy transforms)
    agrees with the FP64 oracle to float32 accuracy."""
    pytest.importorskip("scipy")
    rng = np.random.default_rng(4)
    im = rng.random((16, 20, 24), dtype=np.float32)
    k = rng.random((5, 3, 7), dtype=np.float32)
    k /= k.sum()
    out = orc.reference_path_fp32(im, k, "centered", workers=2)
    assert orc.rel_l2(out, orc.conv_fp64(im, k, "centered")) < 1e-6


def test_metrics(orc):
    a = np.ones(100, np.float32)
    b = a + np.float32(0.1)
    assert abs(orc.l2norm(a, b) - np.sqrt(100 * 0.1 ** 2) / 100) < 1e-7
    assert abs(orc.l2norm_by_nvidia(a, b) - np.sqrt(100 * 0.01) / np.sqrt(100 * 1.1 ** 2)) < 1e-6


def test_rl_oracle_conserves_flux_and_sharpens(orc):
    """The FP64 Richardson-Lucy restatement: with a unit-sum kernel and a
    positive estimate the update keeps sum(x) = sum(y), and it moves a
    blurred pair of spots back towards the spots."""
    rng = np.random.default_rng(1)
    truth = np.ones((16, 20, 24))
    truth[8, 10, 12] = 500.0
    truth[3, 4, 5] = 200.0
    k = rng.random((5, 3, 7))
    k = (k / k.sum()).astype(np.float32)
    y = orc.conv_fp64(truth, k, "centered")
    x = orc.rl_fp64(y, k, 20)
    assert abs(x.sum() / y.sum() - 1) < 1e-12
    err = lambda a: np.linalg.norm(a - truth) / np.linalg.norm(truth)
    assert err(x) < 0.5 * err(y)
    assert np.allclose(orc.correlate_fp64(y, k), orc.conv_fp64(y, np.ascontiguousarray(k[::-1, ::-1, ::-1]), "centered"))


def test_subsampled_oracle_index_map_and_known_answers(orc):
    """The subsampled-kernel restatement (src/convolution3Dfft.cu:65-125):
    the nearest-neighbour index map, r = 1 reading every kernel frequency once
    (the odd-index negation is then a half-period shift on even axes), and a
    1x1x1 kernel scaling the image."""
    assert list(orc.subsampled_index(64, 64, 64)) == list(range(64))
    assert orc.subsampled_index(512, 31, 257)[-1] == 16  # (kx+1)/2: one past the 16 stored columns
    assert orc.subsampled_index(128, 63, 128)[-1] == 0  # 63 mod 63: the index wraps at the top
    idx = orc.subsampled_index(100, 13, 100)
    assert idx.min() >= 0 and idx.max() < 13 and np.all(np.diff(idx[:95]) >= 0)
    rng = np.random.default_rng(2)
    im = rng.random((8, 12, 16))
    k = rng.random((8, 12, 16))
    unshifted = np.fft.irfftn(np.fft.rfftn(im) * np.fft.rfftn(k), s=im.shape, axes=(0, 1, 2))
    expect = np.roll(unshifted, (4, 6, 8), axis=(0, 1, 2))
    assert np.max(np.abs(orc.subsampled_fp64(im, k) - expect)) <= 1e-12 * np.abs(expect).max()
    assert np.max(np.abs(orc.subsampled_fp64(im, np.full((1, 1, 1), 2.0)) - 2 * im)) <= 1e-12
    # odd kx: the x Nyquist reads the Hermitian mirror of the stored half spectrum
    kk = rng.random((3, 5, 7))
    A = orc.subsampled_coefficients(kk, (6, 10, 28))
    full = np.fft.fftn(kk)
    assert orc.subsampled_index(28, 7, 15)[-1] == 4  # past the 4 stored columns of kx = 7
    iz, iy = orc.subsampled_index(6, 3, 6), orc.subsampled_index(10, 5, 10)
    sign = np.where((iz[:, None] + iy[None, :] + 4) % 2 == 1, -1, 1)
    mirror = np.conj(full[(-iz) % 3][:, (-iy) % 5, 3])
    assert np.allclose(A[:, :, -1], sign * mirror, rtol=1e-12, atol=1e-12)


def test_subsampled_coefficients_match_the_reference_loop(orc):
    """The vectorised coefficient map equals a literal restatement of the
    reference's per-element loop (src/convolution3Dfft.cu:68-117): flat index
    i over the half spectrum, dimension 2 fastest, the nearest-neighbour
    indices in float32 with the multiply-add rounded once, the packed
    half-spectrum read k2 + aux*(k1 + kd1*k0), and the parity negation.  Even
    kx keeps every read inside its row (odd kx is covered by the mirror test)."""
    rng = np.random.default_rng(5)
    for shape, kshape in (((6, 10, 12), (3, 5, 4)), ((7, 9, 16), (5, 3, 6)), ((4, 4, 8), (4, 4, 8))):
        kernel = rng.random(kshape)
        imd = shape        # (imDim_0, imDim_1, imDim_2): dimension 2 fastest
        kd = kshape
        packed = np.fft.rfftn(kernel).ravel()  # [kd0][kd1][kd2/2+1]
        r = [np.float32(np.float32(kd[a]) / np.float32(imd[a])) for a in range(3)]

        def near(ra, f, k):
            return int(np.float32(np.float64(ra) * f + 0.5)) % k

        aux = 1 + imd[2] // 2
        n = imd[0] * imd[1] * aux
        loop = np.empty(n, np.complex128)
        for i in range(n):
            k2 = i % aux
            q = (i - k2) // aux
            k1 = q % imd[1]
            k0 = (q - k1) // imd[1]
            k2, k1, k0 = near(r[2], k2, kd[2]), near(r[1], k1, kd[1]), near(r[0], k0, kd[0])
            a = packed[k2 + (1 + kd[2] // 2) * (k1 + kd[1] * k0)]
            loop[i] = -a if (k0 + k1 + k2) % 2 == 1 else a
        got = orc.subsampled_coefficients(kernel, shape).ravel()
        assert np.allclose(got, loop, rtol=0, atol=1e-12 * np.abs(loop).max()), (shape, kshape)


def test_subsampled_index_emulation_matches_fmaf(orc):
    """The numpy index map (float64 multiply-add, one cast to float32) equals a C
    restatement with fmaf (one rounding by definition) over every frequency of
    a grid of axis and kernel lengths, including the ratios near ties."""
    rng = np.random.default_rng(11)
    ns = sorted(set([1, 2, 3, 7, 16, 31, 63, 64, 96, 100, 127, 128, 200, 250, 255, 256, 333, 384, 448, 500, 512,
                     600, 720, 1000, 1024, 2048, 4096] + list(rng.integers(1, 4097, 40))))
    checked = 0
    for n in ns:
        ks = sorted(set([1, 2, 3, n] + [k for k in (5, 7, 9, 15, 21, 31, 41, 63, 64, 127) if k <= n] +
                        list(rng.integers(1, n + 1, 6))))
        for k in ks:
            a = orc.subsampled_index(int(n), int(k), int(n))
            b = orc.subsampled_index_c(int(n), int(k), int(n))
            assert np.array_equal(a, b), (n, k, np.nonzero(a != b)[0][:5])
            checked += int(n)
    assert checked > 100000
