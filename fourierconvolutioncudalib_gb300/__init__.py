"""GB300-native 3D FFT convolution with the FourierConvolutionCUDALib C ABI.

The product is the shared library libFourierConvolutionCUDALib.so built from
``csrc/`` (hand-written sm_103a kernels, no cuFFT).  This module loads it with
ctypes and mirrors the reference's entry points with the same names and
argument meaning (reference header src/convolution3Dfft.h:29-84), taking
numpy arrays instead of raw pointers, plus thin wrappers of the device-pointer
API for torch tensors.  Where the reference would exit() or throw across the C
ABI, these functions raise :class:`FcError` with the library's status.

There is no CPU fallback: if the library is missing, importing the functions
that compute raises.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

__all__ = [
    "FcError", "lib", "load_library", "library_path",
    "convolution3DfftCUDAInPlace", "convolution3DfftCUDA", "convolution3DfftCUDA_test",
    "convolution3DfftCUDAInPlaceSaveMemory",
    "selectDeviceWithHighestComputeCapability", "getCUDAcomputeCapabilityMajorVersion",
    "getCUDAcomputeCapabilityMinorVersion", "getNumDevicesCUDA", "getNameDeviceCUDA", "getMemDeviceCUDA",
    "cuda_version", "gpu_mem_needed_mb", "plan_radices",
    "FC_FLAG_SHIFT_COMPAT", "FC_FLAG_DENSE_KERNEL", "FC_FLAG_TC_FP16", "FC_FLAG_TC_BF16", "FC_FLAG_CORRELATE",
]

FC_OK, FC_ERR_ARG, FC_ERR_CUDA, FC_ERR_NOMEM, FC_ERR_UNSUPPORTED, FC_ERR_TIMEOUT = range(6)
FC_FLAG_SHIFT_COMPAT = 1
FC_FLAG_DENSE_KERNEL = 2
FC_FLAG_TC_FP16 = 4
FC_FLAG_TC_BF16 = 8
FC_FLAG_CORRELATE = 16

_PKG = Path(__file__).resolve().parent
LIB_NAME = "libFourierConvolutionCUDALib.so"


def library_path() -> Path:
    return Path(os.environ.get("FC_LIBRARY", _PKG / LIB_NAME))


class FcError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[fc status {status}] {message}")
        self.status = status
        self.message = message


_lib: Optional[ctypes.CDLL] = None

_P = ctypes.c_void_p
_I = ctypes.c_int
_IP = ctypes.POINTER(ctypes.c_int)
_FP = ctypes.POINTER(ctypes.c_float)
_SZ = ctypes.c_size_t

_SIGNATURES = {
    "convolution3DfftCUDA_test": (_FP, [_FP, _IP, _FP, _I]),
    "convolution3DfftCUDA": (_FP, [_FP, _IP, _FP, _IP, _I]),
    "convolution3DfftCUDAInPlace": (None, [_FP, _IP, _FP, _IP, _I]),
    "convolution3DfftCUDAInPlaceSaveMemory": (None, [_FP, _IP, _FP, _IP, _I]),
    "selectDeviceWithHighestComputeCapability": (_I, []),
    "getCUDAcomputeCapabilityMinorVersion": (_I, [_I]),
    "getCUDAcomputeCapabilityMajorVersion": (_I, [_I]),
    "getNumDevicesCUDA": (_I, []),
    "getNameDeviceCUDA": (None, [_I, ctypes.c_char_p]),
    "getMemDeviceCUDA": (ctypes.c_longlong, [_I]),
    "cuda_version": (_I, []),
    "gpu_mem_needed_mb": (_I, [_IP, _I]),
    "fc_last_status": (_I, []),
    "fc_last_error": (ctypes.c_char_p, []),
    "fc_free_result": (None, [_FP]),
    "fc_set_shift_compat": (None, [_I]),
    "fc_set_generic_kernels": (None, [_I]),
    "fc_set_host_io": (None, [_I]),
    "fc_set_l2_chunk_bytes": (None, [ctypes.c_longlong]),
    "fc_release_device": (_I, [_I]),
    "fc_version": (ctypes.c_char_p, []),
    "fc_conv3d_workspace_bytes": (_SZ, [_IP, _IP, _I]),
    "fc_conv3d_device": (_I, [_P, _P, _IP, _P, _IP, _I, _P, _SZ, _P]),
    "fc_kernel_spectrum_bytes": (_SZ, [_IP, _IP, _I]),
    "fc_kernel_spectrum_device": (_I, [_P, _IP, _IP, _I, _P, _SZ, _P]),
    "fc_conv3d_kspec_workspace_bytes": (_SZ, [_IP]),
    "fc_conv3d_kspec_device": (_I, [_P, _P, _IP, _P, _IP, _I, _P, _SZ, _P]),
    "fc_rl_workspace_bytes": (_SZ, [_IP, _IP, _I]),
    "fc_conv3d_subsampled_workspace_bytes": (_SZ, [_IP, _IP]),
    "fc_conv3d_subsampled_device": (_I, [_P, _P, _IP, _P, _IP, _P, _SZ, _P]),
    "fc_rl_deconvolve_device": (_I, [_P, _P, _IP, _P, _IP, _I, _I, _P, _SZ, _P]),
    "fc_conv3d_adjoint_workspace_bytes": (_SZ, [_IP, _IP, _I]),
    "fc_conv3d_adjoint_device": (_I, [_P, _P, _P, _P, _P, _IP, _IP, _I, _P, _SZ, _P]),
    "fc_conv3d_batched_workspace_bytes": (_SZ, [_I, _IP, _I]),
    "fc_conv3d_batched_device": (_I, [_I, ctypes.POINTER(_P), ctypes.POINTER(_P), ctypes.POINTER(_P), _IP, _I, _P,
                                      _SZ, _P]),
    "fc_fft3d_workspace_bytes": (_SZ, [_IP]),
    "fc_rfft3d_device": (_I, [_P, _P, _IP, _P, _SZ, _P]),
    "fc_irfft3d_device": (_I, [_P, _P, _IP, _P, _SZ, _P]),
    "fc_pad_shift_kernel_device": (_I, [_P, _IP, _IP, _I, _P, _P]),
    "fc_plan_radices": (_I, [_I, _IP, _I]),
    "fc_profile_enable": (None, [_I]),
    "fc_batched_last_plan": (_I, [_IP]),
    "fc_profile_only": (None, [ctypes.c_char_p]),
    "fc_profile_read": (_I, [ctypes.c_char_p, _I, _FP, ctypes.POINTER(ctypes.c_double), _I]),
    "fc_launch_count": (_I, []),
    "fc_conv3d_device_noalloc": (_I, [_P, _P, _IP, _P, _IP, _I, _P]),
    "fc_device_wait_status": (_I, [_P]),
    "fc_test_set_wait_fault": (_I, [ctypes.c_longlong, _I]),
    "fc_fault_inject": (_I, [ctypes.c_char_p]),
}


def load_library(path: Optional[os.PathLike] = None) -> ctypes.CDLL:
    """Load (once) and return the CDLL with argument types set."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else library_path()
    if not p.exists():
        raise FcError(FC_ERR_UNSUPPORTED, f"{p} not built; run fourierconvolutioncudalib_gb300.build.build()")
    cdll = ctypes.CDLL(str(p))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(cdll, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = cdll
    return cdll


def lib() -> ctypes.CDLL:
    return load_library()


def _check(rc: Optional[int] = None) -> None:
    L = lib()
    st = L.fc_last_status() if rc is None else rc
    if st != FC_OK:
        raise FcError(st, L.fc_last_error().decode(errors="replace"))


def _iarr(v: Sequence[int]):
    return (ctypes.c_int * len(v))(*[int(x) for x in v])


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(_FP)


def _as_f32c(a: np.ndarray, name: str) -> np.ndarray:
    if not isinstance(a, np.ndarray) or a.dtype != np.float32 or not a.flags.c_contiguous:
        raise FcError(FC_ERR_ARG, f"{name} must be a C-contiguous float32 numpy array")
    return a


# ---------------------------------------------------------------- reference entry points
def convolution3DfftCUDAInPlace(im: np.ndarray, imDim: Sequence[int], kernel: np.ndarray,
                                kernelDim: Sequence[int], devCUDA: int) -> None:
    """Overwrite ``im`` with its circular convolution by ``kernel``.

    imDim = (nx, ny, nz), kernelDim = (kx, ky, kz), x fastest; arrays are C-order
    [z][y][x] float32 (reference src/convolution3Dfft.cu:394-421)."""
    _as_f32c(im, "im")
    _as_f32c(kernel, "kernel")
    if im.size != int(np.prod(imDim)) or kernel.size != int(np.prod(kernelDim)):
        raise FcError(FC_ERR_ARG, "array sizes do not match the given dimensions")
    lib().convolution3DfftCUDAInPlace(_fptr(im), _iarr(imDim), _fptr(kernel), _iarr(kernelDim), int(devCUDA))
    _check()


def convolution3DfftCUDAInPlaceSaveMemory(im: np.ndarray, imDim: Sequence[int], kernel: np.ndarray,
                                          kernelDim: Sequence[int], devCUDA: int) -> None:
    """Overwrite ``im`` with the subsampled-kernel approximation of its
    convolution by ``kernel``: the kernel's spectrum at its own size, read at
    the nearest kernel frequency of each image frequency (reference
    src/convolution3Dfft.h:58-64, src/convolution3Dfft.cu:65-125).  Same
    dimension order and errors as convolution3DfftCUDAInPlace."""
    _as_f32c(im, "im")
    _as_f32c(kernel, "kernel")
    if im.size != int(np.prod(imDim)) or kernel.size != int(np.prod(kernelDim)):
        raise FcError(FC_ERR_ARG, "array sizes do not match the given dimensions")
    lib().convolution3DfftCUDAInPlaceSaveMemory(_fptr(im), _iarr(imDim), _fptr(kernel), _iarr(kernelDim),
                                                int(devCUDA))
    _check()


def _take_result(ptr, n: int) -> np.ndarray:
    if not ptr:
        _check()
        raise FcError(FC_ERR_CUDA, "NULL result")
    out = np.ctypeslib.as_array(ptr, shape=(n,)).copy()
    lib().fc_free_result(ptr)
    return out


def convolution3DfftCUDA(im: np.ndarray, imDim: Sequence[int], kernel: np.ndarray, kernelDim: Sequence[int],
                         devCUDA: int) -> np.ndarray:
    """Return the convolution as a new array; imDim/kernelDim slowest-first
    (index 2 fastest), reference src/convolution3Dfft.h:34-45."""
    _as_f32c(im, "im")
    _as_f32c(kernel, "kernel")
    n = int(np.prod(imDim))
    if im.size != n or kernel.size != int(np.prod(kernelDim)):
        raise FcError(FC_ERR_ARG, "array sizes do not match the given dimensions")
    ptr = lib().convolution3DfftCUDA(_fptr(im), _iarr(imDim), _fptr(kernel), _iarr(kernelDim), int(devCUDA))
    return _take_result(ptr, n).reshape(im.shape)


def convolution3DfftCUDA_test(im: np.ndarray, imDim: Sequence[int], kernel: np.ndarray, devCUDA: int) -> np.ndarray:
    """Convolution with an image-sized, already shifted kernel (reference src/convolution3Dfft.h:29-32)."""
    _as_f32c(im, "im")
    _as_f32c(kernel, "kernel")
    n = int(np.prod(imDim))
    if im.size != n or kernel.size != n:
        raise FcError(FC_ERR_ARG, "array sizes do not match the given dimensions")
    ptr = lib().convolution3DfftCUDA_test(_fptr(im), _iarr(imDim), _fptr(kernel), int(devCUDA))
    return _take_result(ptr, n).reshape(im.shape)


def selectDeviceWithHighestComputeCapability() -> int:
    return lib().selectDeviceWithHighestComputeCapability()


def getCUDAcomputeCapabilityMajorVersion(devCUDA: int) -> int:
    return lib().getCUDAcomputeCapabilityMajorVersion(int(devCUDA))


def getCUDAcomputeCapabilityMinorVersion(devCUDA: int) -> int:
    return lib().getCUDAcomputeCapabilityMinorVersion(int(devCUDA))


def getNumDevicesCUDA() -> int:
    return lib().getNumDevicesCUDA()


def getNameDeviceCUDA(devCUDA: int) -> str:
    buf = ctypes.create_string_buffer(256)
    lib().getNameDeviceCUDA(int(devCUDA), buf)
    return buf.value.decode(errors="replace")


def getMemDeviceCUDA(devCUDA: int) -> int:
    return lib().getMemDeviceCUDA(int(devCUDA))


def cuda_version() -> int:
    return lib().cuda_version()


def gpu_mem_needed_mb(shape: Sequence[int]) -> int:
    return lib().gpu_mem_needed_mb(_iarr(shape), len(shape))


def plan_radices(n: int) -> list:
    buf = (ctypes.c_int * 32)()
    k = lib().fc_plan_radices(int(n), buf, 32)
    if k < 0:
        raise FcError(FC_ERR_UNSUPPORTED, f"no plan for {n}")
    return list(buf[:k])
