"""CPU oracle for the 3D FFT convolution -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference
legs may import this module; the product (libFourierConvolutionCUDALib.so and
the fourierconvolutioncudalib_gb300 package) never does.

Contents
  * ctypes bindings of fc_oracle.c, the C restatement of the reference's index
    arithmetic (fftShiftKernel + row copy), its direct-sum CPU convolution
    (tests/test_algorithms.hpp:10-58), its spectrum multiply
    (src/convolution3Dfft.cu:41-62) and its error metrics
    (tests/test_utils.hpp:76-108);
  * an FP64 FFT oracle (numpy.fft, double precision) of the circular
    convolution the reference computes;
  * reference_path_fp32: the reference's own algorithm -- pad+shift, 3D R2C of
    image and kernel, modulate-and-normalise, 3D C2R -- run on the host in
    float32 (scipy.fft for the transforms, which stand in for cuFFT, the
    third-party library the reference calls), used as the timed CPU baseline;
  * zero_padd, restating tests/padd_utils.h:99-171;
  * the reference test suite's known-answer cases as data (kat_cases()).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path
from typing import Dict, Iterable, List, Optional, Sequence, Tuple

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libfc_oracle.so"

_lib: Optional[ctypes.CDLL] = None
_I = ctypes.c_int
_IP = ctypes.POINTER(ctypes.c_int)
_FP = ctypes.POINTER(ctypes.c_float)


def build_oracle(force: bool = False) -> Path:
    """Compile fc_oracle.c with gcc (OpenMP), portable flags only."""
    src = HERE / "fc_oracle.c"
    if not force and LIB.exists() and LIB.stat().st_mtime >= src.stat().st_mtime:
        return LIB
    BUILD.mkdir(exist_ok=True)
    tmp = BUILD / "libfc_oracle.so.tmp"
    cmd = ["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c11", str(src), "-o", str(tmp), "-lm"]
    subprocess.run(cmd, check=True, capture_output=True)
    os.replace(tmp, LIB)
    return LIB


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build_oracle()
        L = ctypes.CDLL(str(LIB))
        L.fco_closest_multiplier.restype = _I
        L.fco_closest_multiplier.argtypes = [_I, _I]
        for nm in ("fco_ref_inplace_padded_kernel", "fco_ref_packed_padded_kernel", "fco_centered_padded_kernel"):
            getattr(L, nm).restype = _I
            getattr(L, nm).argtypes = [_FP, _IP, _IP, _FP]
        L.fco_convolve_direct.restype = None
        L.fco_convolve_direct.argtypes = [_FP, _IP, _FP, _IP, _FP, _IP, _I, _I]
        L.fco_convolve_direct_crop.restype = None
        L.fco_convolve_direct_crop.argtypes = [_FP, _IP, _FP, _IP, _IP, _IP, _FP, _I]
        L.fco_modulate_and_normalize.restype = None
        L.fco_modulate_and_normalize.argtypes = [_FP, _FP, ctypes.c_longlong, ctypes.c_float, _I]
        L.fco_l2norm.restype = ctypes.c_double
        L.fco_l2norm.argtypes = [_FP, _FP, ctypes.c_longlong]
        L.fco_l2norm_by_nvidia.restype = ctypes.c_double
        L.fco_l2norm_by_nvidia.argtypes = [_FP, _FP, ctypes.c_longlong]
        L.fco_max_threads.restype = _I
        L.fco_subsampled_index.restype = None
        L.fco_subsampled_index.argtypes = [_I, _I, _I, _IP]
        _lib = L
    return _lib


def _f(a: np.ndarray):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(_FP)


def _i(v: Sequence[int]):
    return (ctypes.c_int * len(v))(*[int(x) for x in v])


# ------------------------------------------------------------------ placement
def closest_multiplier(a: int, m: int = 32) -> int:
    """src/convolution3Dfft.cu:26-38"""
    return lib().fco_closest_multiplier(int(a), int(m))


def ref_inplace_padded_kernel(kernel: np.ndarray, image_shape_zyx: Sequence[int]) -> np.ndarray:
    """Padded kernel exactly as convolution3DfftCUDAInPlace builds it
    (src/convolution3Dfft.cu:442-486): kernel [kz][ky][kx] -> [nz][ny][nx]."""
    kz, ky, kx = kernel.shape
    nz, ny, nx = image_shape_zyx
    out = np.empty((nz, ny, nx), np.float32)
    k = np.ascontiguousarray(kernel, np.float32)
    if lib().fco_ref_inplace_padded_kernel(_f(k), _i([kx, ky, kz]), _i([nx, ny, nz]), _f(out)) != 0:
        raise ValueError("reference placement writes outside the image buffer for these shapes")
    return out


def ref_packed_padded_kernel(kernel: np.ndarray, image_shape: Sequence[int]) -> np.ndarray:
    """Padded kernel as convolution3DfftCUDA builds it (src/convolution3Dfft.cu:344-348);
    dims slowest-first for both arrays."""
    out = np.empty(tuple(image_shape), np.float32)
    k = np.ascontiguousarray(kernel, np.float32)
    if lib().fco_ref_packed_padded_kernel(_f(k), _i(kernel.shape), _i(image_shape), _f(out)) != 0:
        raise ValueError("reference placement writes outside the image buffer for these shapes")
    return out


def centered_padded_kernel(kernel: np.ndarray, image_shape_zyx: Sequence[int]) -> np.ndarray:
    """Centred circular placement: tap (iz,iy,ix) -> ((iz-kz/2)%nz, (iy-ky/2)%ny, (ix-kx/2)%nx)."""
    kz, ky, kx = kernel.shape
    nz, ny, nx = image_shape_zyx
    out = np.empty((nz, ny, nx), np.float32)
    k = np.ascontiguousarray(kernel, np.float32)
    if lib().fco_centered_padded_kernel(_f(k), _i([kx, ky, kz]), _i([nx, ny, nz]), _f(out)) != 0:
        raise ValueError("kernel larger than image")
    return out


# ------------------------------------------------------------------ direct sum
def convolve_direct(image: np.ndarray, kernel: np.ndarray, offset: Optional[Sequence[int]] = None,
                    periodic: bool = False, threads: int = 1, result: Optional[np.ndarray] = None) -> np.ndarray:
    """tests/test_algorithms.hpp:10-58 (float accumulator, flipped kernel).
    Non-periodic: only [offset, shape-offset) is written; the rest of `result`
    (default: a copy of the image, as the reference fixture does) is kept."""
    im = np.ascontiguousarray(image, np.float32)
    k = np.ascontiguousarray(kernel, np.float32)
    if result is None:
        result = im.copy()
    off = list(offset) if offset is not None else [s // 2 for s in k.shape]
    lib().fco_convolve_direct(_f(im), _i(im.shape), _f(k), _i(k.shape), _f(result), _i(off), int(periodic),
                              int(threads))
    return result


def convolve_direct_crop(image: np.ndarray, kernel: np.ndarray, crop0: Sequence[int], cropn: Sequence[int],
                         threads: int = 1) -> np.ndarray:
    """Periodic direct sum restricted to an output crop (bounded CPU-baseline sample)."""
    im = np.ascontiguousarray(image, np.float32)
    k = np.ascontiguousarray(kernel, np.float32)
    out = np.empty(tuple(cropn), np.float32)
    lib().fco_convolve_direct_crop(_f(im), _i(im.shape), _f(k), _i(k.shape), _i(crop0), _i(cropn), _f(out),
                                   int(threads))
    return out


# ------------------------------------------------------------------ multiply and metrics
def modulate_and_normalize(dst: np.ndarray, src: np.ndarray, c: float, threads: int = 1) -> np.ndarray:
    """In place: dst <- c * src * dst with the operation order of
    src/convolution3Dfft.cu:41-45 (src = kernel spectrum, dst = image spectrum)."""
    assert dst.dtype == np.complex64 and src.dtype == np.complex64 and dst.flags.c_contiguous
    d = dst.view(np.float32).reshape(-1)
    s = np.ascontiguousarray(src).view(np.float32).reshape(-1)
    lib().fco_modulate_and_normalize(_f(d), _f(s), dst.size, ctypes.c_float(c), int(threads))
    return dst


def l2norm(reference: np.ndarray, data: np.ndarray) -> float:
    """tests/test_utils.hpp:76-88: sqrt(sum d^2) / n"""
    r = np.ascontiguousarray(reference, np.float32)
    d = np.ascontiguousarray(data, np.float32)
    return lib().fco_l2norm(_f(r), _f(d), d.size)


def l2norm_by_nvidia(reference: np.ndarray, data: np.ndarray) -> float:
    """tests/test_utils.hpp:90-108: sqrt(sum d^2) / sqrt(sum data^2)"""
    r = np.ascontiguousarray(reference, np.float32)
    d = np.ascontiguousarray(data, np.float32)
    return lib().fco_l2norm_by_nvidia(_f(r), _f(d), d.size)


def rel_l2(x: np.ndarray, ref: np.ndarray) -> float:
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    den = np.linalg.norm(ref.ravel())
    return float(np.linalg.norm((x - ref).ravel()) / (den if den > 0 else 1.0))


def max_abs(x: np.ndarray, ref: np.ndarray) -> float:
    return float(np.max(np.abs(np.asarray(x, np.float64) - np.asarray(ref, np.float64))))


# ------------------------------------------------------------------ FFT oracles
def fft_conv_fp64(image: np.ndarray, padded_kernel: np.ndarray) -> np.ndarray:
    """Circular convolution in double precision: irfftn(rfftn(im) * rfftn(k))."""
    a = np.fft.rfftn(np.asarray(image, np.float64))
    b = np.fft.rfftn(np.asarray(padded_kernel, np.float64))
    return np.fft.irfftn(a * b, s=image.shape, axes=(0, 1, 2))


def conv_fp64(image: np.ndarray, kernel: np.ndarray, placement: str = "centered") -> np.ndarray:
    """FP64 oracle of the convolution with the given kernel placement:
    'centered' (the intended centre shift), 'reference_inplace' (the
    reference InPlace index arithmetic) or 'dense' (kernel already padded)."""
    if placement == "centered":
        pk = centered_padded_kernel(kernel, image.shape)
    elif placement == "reference_inplace":
        pk = ref_inplace_padded_kernel(kernel, image.shape)
    elif placement == "dense":
        pk = np.asarray(kernel, np.float32)
    else:
        raise ValueError(placement)
    return fft_conv_fp64(image, pk)


def correlate_fp64(image: np.ndarray, kernel: np.ndarray) -> np.ndarray:
    """FP64 circular correlation with the centred kernel: the conjugate kernel
    spectrum, i.e. convolution with the kernel flipped about its centre."""
    pk = centered_padded_kernel(kernel, image.shape).astype(np.float64)
    a = np.fft.rfftn(np.asarray(image, np.float64))
    return np.fft.irfftn(a * np.conj(np.fft.rfftn(pk)), s=image.shape, axes=(0, 1, 2))


def subsampled_index(n: int, k: int, m: int) -> np.ndarray:
    """Kernel frequency read by image frequencies 0..m-1 of an axis of length n
    (src/convolution3Dfft.cu:68-70, :106-108): (int)(r*f + 0.5f) % k with
    r = (float)k / (float)n in float32 and the multiply-add rounded once (the
    contracted expression).  r*f + 0.5 is exact in float64 (24-bit r times an
    integer below 2**13), so one cast to float32 is the fused rounding."""
    r = np.float32(np.float32(k) / np.float32(n))
    f = np.arange(m, dtype=np.float64)
    v = (np.float64(r) * f + 0.5).astype(np.float32)
    return np.trunc(v).astype(np.int64) % k


def subsampled_index_c(n: int, k: int, m: int) -> np.ndarray:
    """subsampled_index restated in C with fmaf (fc_oracle.c), for cross-checking
    the float64 emulation of the fused float32 multiply-add."""
    out = np.empty(m, np.int32)
    lib().fco_subsampled_index(int(n), int(k), int(m), out.ctypes.data_as(_IP))
    return out


def subsampled_coefficients(kernel: np.ndarray, image_shape_zyx: Sequence[int]) -> np.ndarray:
    """The kernel coefficient of every image frequency of the subsampled-kernel
    product (src/convolution3Dfft.cu:65-125) in double precision: the
    spectrum of the unpadded, unshifted kernel at its own size, read at the
    nearest-neighbour indices, negated where the three indices sum to an odd
    number (:113-117).  The full spectrum is indexed, so an x index past the
    stored half (odd kx, at the image's x Nyquist) takes the Hermitian mirror;
    the reference reads past its half-spectrum row there."""
    nz, ny, nx = image_shape_zyx
    kz, ky, kx = kernel.shape
    K = np.fft.fftn(np.asarray(kernel, np.float64))
    iz = subsampled_index(nz, kz, nz)
    iy = subsampled_index(ny, ky, ny)
    ix = subsampled_index(nx, kx, nx // 2 + 1)
    A = K[np.ix_(iz, iy, ix)]
    odd = (iz[:, None, None] + iy[None, :, None] + ix[None, None, :]) % 2 == 1
    return np.where(odd, -A, A)


def subsampled_fp64(image: np.ndarray, kernel: np.ndarray) -> np.ndarray:
    """FP64 oracle of the subsampled-kernel convolution: the image's half
    spectrum times subsampled_coefficients, inverse real transform.  Where the
    product is not Hermitian on the x DC and Nyquist planes, the imaginary
    parts of those bins are dropped after the z and y inverses (numpy's irfftn,
    and the library's C2R passes)."""
    x = np.asarray(image, np.float64)
    A = subsampled_coefficients(kernel, x.shape)
    return np.fft.irfftn(np.fft.rfftn(x) * A, s=x.shape, axes=(0, 1, 2))


def rl_fp64(observed: np.ndarray, kernel: np.ndarray, iterations: int,
            estimate: Optional[np.ndarray] = None) -> np.ndarray:
    """Richardson-Lucy deconvolution in double precision (the published
    multiplicative update of Richardson 1972 / Lucy 1974; no reference
    counterpart): x <- x * correlate(y / conv(x, k), k) with the centred
    circular placement, ratio 0 where conv(x, k) <= 0."""
    y = np.asarray(observed, np.float64)
    K = np.fft.rfftn(centered_padded_kernel(kernel, y.shape).astype(np.float64))
    x = (y if estimate is None else np.asarray(estimate, np.float64)).copy()
    for _ in range(iterations):
        est = np.fft.irfftn(np.fft.rfftn(x) * K, s=y.shape, axes=(0, 1, 2))
        ratio = np.divide(y, est, out=np.zeros_like(y), where=est > 0)
        x = x * np.fft.irfftn(np.fft.rfftn(ratio) * np.conj(K), s=y.shape, axes=(0, 1, 2))
    return x


def reference_path_fp32(image: np.ndarray, kernel: np.ndarray, placement: str = "centered",
                        workers: int = -1) -> np.ndarray:
    """The reference's InPlace algorithm on the host in float32:
    pad+shift (src/convolution3Dfft.cu:442-486), R2C of image and kernel
    (:523-525), modulate-and-normalise with 1/N (:527-536), C2R (:547).
    The transforms are scipy.fft's single-precision R2C/C2R (standing in for
    cuFFT) on `workers` threads."""
    import scipy.fft as sfft

    if placement == "centered":
        pk = centered_padded_kernel(kernel, image.shape)
    elif placement == "reference_inplace":
        pk = ref_inplace_padded_kernel(kernel, image.shape)
    else:
        pk = np.ascontiguousarray(kernel, np.float32)
    im = np.ascontiguousarray(image, np.float32)
    spec = sfft.rfftn(im, workers=workers)
    kspec = sfft.rfftn(pk, workers=workers)
    spec = np.ascontiguousarray(spec, np.complex64)
    kspec = np.ascontiguousarray(kspec, np.complex64)
    nthreads = os.cpu_count() if workers in (-1, None) else workers
    modulate_and_normalize(spec, kspec, np.float32(1.0) / np.float32(im.size), threads=nthreads)
    # norm='forward' leaves the inverse unscaled, as cuFFT's C2R is (the 1/N is in the multiply)
    return np.asarray(sfft.irfftn(spec, s=im.shape, workers=workers, norm="forward"), np.float32)


# ------------------------------------------------------------------ padding utilities
def zero_padd(image: np.ndarray, kernel_shape: Sequence[int], factor: int = 1) -> Tuple[np.ndarray, List[int]]:
    """tests/padd_utils.h:99-171: extents n + 2*factor*(k/2) per axis (:20-23),
    offsets factor*(k/2) (:34-36); image inserted at the offsets."""
    ext = [n + 2 * factor * (k // 2) for n, k in zip(image.shape, kernel_shape)]
    off = [factor * (k // 2) for k in kernel_shape]
    out = np.zeros(ext, np.float32)
    out[off[0]:off[0] + image.shape[0], off[1]:off[1] + image.shape[1], off[2]:off[2] + image.shape[2]] = image
    return out, off


def crop(padded: np.ndarray, off: Sequence[int], shape: Sequence[int]) -> np.ndarray:
    return padded[off[0]:off[0] + shape[0], off[1]:off[1] + shape[1], off[2]:off[2] + shape[2]]


# ------------------------------------------------------------------ known-answer cases
def _ramp(shape) -> np.ndarray:
    return np.arange(int(np.prod(shape)), dtype=np.float64).astype(np.float32).reshape(shape)


def fixture_3d(kernel_dim: int = 3, image_dim: int = 8) -> Dict[str, np.ndarray]:
    """tests/test_fixtures.hpp:22-292 (convolutionFixture3D<3,8>): the 8^3 ramp
    image and the 3^3 kernels of the legacy suite, plus the asymmetric kernels."""
    h = kernel_dim // 2
    K = kernel_dim
    d = {}
    d["image"] = _ramp((image_dim,) * 3)
    z = np.zeros((K, K, K), np.float32)
    d["trivial"] = z.copy()
    ident = z.copy()
    ident.reshape(-1)[K ** 3 // 2] = 1.0
    d["identity"] = ident
    hor, ver, dep = z.copy(), z.copy(), z.copy()
    for i in range(K):
        hor[h, h, i] = i + 1
        ver[h, i, h] = i + 1
        dep[i, h, h] = i + 1
    d["horizontal"], d["vertical"], d["depth"] = hor, ver, dep
    d["all1"] = np.ones((K, K, K), np.float32)
    ac = np.zeros((K + 1, K, K - 1), np.float32)
    ao = ac.copy()
    ai = ac.copy()
    ai[ac.shape[0] // 2, ac.shape[1] // 2, ac.shape[2] // 2] = 1.0
    for zz in range(ac.shape[0]):
        for yy in range(ac.shape[1]):
            for xx in range(ac.shape[2]):
                if zz == ac.shape[0] // 2 and yy == ac.shape[1] // 2:
                    ac[zz, yy, xx] = xx + 1
                    ao[zz, yy, xx] = 1
                if xx == ac.shape[2] // 2 and yy == ac.shape[1] // 2:
                    ac[zz, yy, xx] = zz + 101
                    ao[zz, yy, xx] = 1
                if xx == ac.shape[2] // 2 and zz == ac.shape[0] // 2:
                    ac[zz, yy, xx] = yy + 11
                    ao[zz, yy, xx] = 1
    d["asymm_cross"], d["asymm_one"], d["asymm_identity"] = ac, ao, ai
    return d


def kat_cases(include_large: bool = True) -> List[dict]:
    """Known-answer cases of the reference test suite, restated as data.

    Each case: name, image (padded, as passed to the InPlace entry), kernel,
    offsets/shape of the crop, expected crop (closed form or CPU direct sum),
    the reference's metric and threshold, and the citation."""
    cases = []
    fx = fixture_3d()
    img = fx["image"]
    # trivial: 8^3 ramp, zero kernel, no padding -> all zeros (test_gpu_convolve.cpp:18-30)
    cases.append(dict(name="trivial_convolve", image=img.copy(), kernel=fx["trivial"], off=[0, 0, 0],
                      shape=img.shape, expected=np.zeros_like(img), metric="sum", threshold=1e-5,
                      cite="tests/test_gpu_convolve.cpp:18-30"))
    # legacy suite: pad 8^3 by the 3^3 kernel, crop, compare with the CPU direct sum
    for nm, cite in (("identity", "33-55"), ("horizontal", "57-89"), ("vertical", "91-126"), ("depth", "128-162"),
                     ("all1", "164-197")):
        k = fx[nm]
        padded, off = zero_padd(img, k.shape)
        exp_full = convolve_direct(padded, k, offset=[s // 2 for s in k.shape])
        expected = crop(exp_full, off, img.shape).copy() if nm != "identity" else img.copy()
        cases.append(dict(name=f"{nm}_convolve", image=padded, kernel=k, off=off, shape=img.shape, expected=expected,
                          metric="sum", threshold=1e-5, cite=f"tests/test_gpu_convolve.cpp:{cite}"))
    # asymmetric volumes: 13x17x19 (x,y,z), 3^3 kernels (test_gpu_convolve.cpp:204-467)
    s_shape = (19, 17, 13)
    for nm, thr, cite in (("identity", 1e-4, "204-268"), ("horizontal", 1e-2, "270-335"),
                          ("vertical", 2e-2, "337-403"), ("diagonal", 2e-2, "405-467")):
        k = np.zeros((3, 3, 3), np.float32)
        if nm == "identity":
            k[1, 1, 1] = 1
            stack = _ramp(s_shape)
            expected = stack.copy()
        else:
            stack = np.ones(s_shape, np.float32)
            if nm == "horizontal":
                k[1, 1, 0:3] = 1
            elif nm == "vertical":
                k[1, 0:3, 1] = 1
            else:
                for i in range(3):
                    k[i, i, i] = 1
            expected = None
        padded, off = zero_padd(stack, k.shape)
        ref_expected = stack.copy() if nm == "identity" else np.full(s_shape, 3.0, np.float32)
        if expected is None:
            # the reference expects 3 everywhere (:325-330), which ignores the
            # zero border of the padded stack; the exact answer is the direct sum
            expected = crop(convolve_direct(padded, k, offset=off), off, s_shape).copy()
        cases.append(dict(name=f"{nm}_convolve_of_prime_shape", image=padded, kernel=k, off=off, shape=s_shape,
                          expected=expected, reference_expected=ref_expected, metric="l2norm", threshold=thr,
                          cite=f"tests/test_gpu_convolve.cpp:{cite}"))
    if include_large:
        # 128^3 constant 42, 31x31x91 (x,y,z) delta*2 -> 84 (test_gpu_numerical_stability.cpp:40-96)
        k = np.zeros((91, 31, 31), np.float32)
        k[45, 15, 15] = 2
        stack = np.full((128, 128, 128), 42, np.float32)
        padded, off = zero_padd(stack, k.shape)
        cases.append(dict(name="times_two_128", image=padded, kernel=k, off=off, shape=stack.shape,
                          expected=np.full(stack.shape, 84, np.float32), metric="l2norm", threshold=1e-3,
                          cite="tests/test_gpu_numerical_stability.cpp:40-96"))
        # 128^3 ramp i, 3x3x5 (x,y,z) delta*2 -> 2i, padding factor 1 and 10 (:98-215)
        k = np.zeros((5, 3, 3), np.float32)
        k[2, 1, 1] = 2
        stack = _ramp((128, 128, 128))
        for fac, cite in ((1, "98-155"), (10, "159-215")):
            padded, off = zero_padd(stack, k.shape, fac)
            cases.append(dict(name=f"ramp_with_tiny_kernel_times_two_padd_{fac}", image=padded, kernel=k, off=off,
                              shape=stack.shape, expected=(2 * stack.astype(np.float64)).astype(np.float32),
                              metric="l2norm", threshold=1e-3, cite=f"tests/test_gpu_numerical_stability.cpp:{cite}"))
    # normalised ramps i/N with a 31x31x91 unit delta (:222-382).  The
    # reference compares against 2x the image (its expected is doubled while
    # the delta is 1); the true answer is the image itself, which is what is
    # stored as `expected`; `reference_expected` keeps the doubled version.
    sizes = (16, 128, 256) if include_large else (16,)
    for n in sizes:
        k = np.zeros((91, 31, 31), np.float32)
        k[45, 15, 15] = 1
        N = n ** 3
        scale = np.float32(1.0) / np.float32(N)
        stack = (np.arange(N, dtype=np.float32) * scale).reshape(n, n, n)
        padded, off = zero_padd(stack, k.shape)
        thr = 1e-2 if n == 16 else 1e-3
        cases.append(dict(name=f"ramp_normalized_{n}", image=padded, kernel=k, off=off, shape=stack.shape,
                          expected=stack.copy(), reference_expected=2 * stack, metric="l2norm", threshold=thr,
                          cite="tests/test_gpu_numerical_stability.cpp:222-382"))
    return cases
