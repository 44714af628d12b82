"""Device-pointer entry points for torch CUDA tensors.

These wrap the library's fc_* C ABI (include/convolution3Dfft.h) for tensors
that are already resident on the GPU.  Every call is enqueued on the current
torch stream (or the one given) and returns without synchronising.  Torch is
used only for memory and streams; all compute runs in the library's kernels.
"""
from __future__ import annotations

import ctypes
from typing import List, Optional, Sequence, Tuple

import torch

from . import FC_FLAG_CORRELATE, FC_FLAG_DENSE_KERNEL, FcError, FC_ERR_ARG, _check, _iarr, lib

__all__ = ["conv3d", "conv3d_adjoint", "conv3d_batched", "rfft3d", "irfft3d", "pad_shift_kernel",
           "kernel_spectrum", "conv3d_kspec", "rl_deconvolve", "conv3d_subsampled", "subsampled_workspace_bytes",
           "workspace_bytes", "profile", "launch_count"]


def _dims(t: torch.Tensor) -> Tuple[int, int, int]:
    if t.dim() != 3:
        raise FcError(FC_ERR_ARG, "expected a 3-D tensor [z][y][x]")
    nz, ny, nx = t.shape
    return int(nx), int(ny), int(nz)


def _f32(t: torch.Tensor, name: str) -> torch.Tensor:
    if not t.is_cuda or t.dtype != torch.float32 or not t.is_contiguous():
        raise FcError(FC_ERR_ARG, f"{name} must be a contiguous float32 CUDA tensor")
    return t


def _stream(stream: Optional[torch.cuda.Stream]) -> int:
    return (stream or torch.cuda.current_stream()).cuda_stream


def _ws(ws: Optional[torch.Tensor], need: int, device) -> Tuple[int, int]:
    if ws is None:
        ws = torch.empty(need, dtype=torch.uint8, device=device)
    if ws.numel() * ws.element_size() < need:
        raise FcError(FC_ERR_ARG, "workspace too small")
    _ws.keep = ws  # keep the allocation alive until the next call on this thread
    return ws.data_ptr(), ws.numel() * ws.element_size()


def workspace_bytes(image_shape: Sequence[int], kernel_shape: Optional[Sequence[int]], flags: int = 0) -> int:
    """Bytes of scratch for a plain convolution; shapes are torch order (z, y, x)."""
    nz, ny, nx = image_shape
    kd = _iarr([kernel_shape[2], kernel_shape[1], kernel_shape[0]]) if kernel_shape is not None else None
    n = lib().fc_conv3d_workspace_bytes(_iarr([nx, ny, nz]), kd, int(flags))
    if n == 0:
        _check()
    return int(n)


def conv3d(image: torch.Tensor, kernel: torch.Tensor, out: Optional[torch.Tensor] = None, flags: int = 0,
           workspace: Optional[torch.Tensor] = None, stream: Optional[torch.cuda.Stream] = None) -> torch.Tensor:
    """Circular convolution of image [nz,ny,nx] by kernel [kz,ky,kx] (or an
    image-sized shifted kernel with FC_FLAG_DENSE_KERNEL)."""
    _f32(image, "image")
    _f32(kernel, "kernel")
    nx, ny, nz = _dims(image)
    if flags & FC_FLAG_DENSE_KERNEL:
        kd = None
    else:
        kx, ky, kz = _dims(kernel)
        kd = _iarr([kx, ky, kz])
    if out is None:
        out = torch.empty_like(image)
    _f32(out, "out")
    need = lib().fc_conv3d_workspace_bytes(_iarr([nx, ny, nz]), kd, int(flags))
    if need == 0:
        _check()
    wp, wb = _ws(workspace, need, image.device)
    rc = lib().fc_conv3d_device(image.data_ptr(), out.data_ptr(), _iarr([nx, ny, nz]), kernel.data_ptr(), kd,
                                int(flags), wp, wb, _stream(stream))
    _check(rc)
    return out


def _kdims(kernel_shape: Optional[Sequence[int]], flags: int):
    if flags & FC_FLAG_DENSE_KERNEL:
        return None
    kz, ky, kx = kernel_shape
    return _iarr([kx, ky, kz])


def kernel_spectrum(kernel: torch.Tensor, image_shape: Sequence[int], flags: int = 0,
                    stream: Optional[torch.cuda.Stream] = None) -> torch.Tensor:
    """The kernel's spectrum for images of image_shape (z, y, x), as an opaque
    device buffer for conv3d_kspec / reuse across calls."""
    _f32(kernel, "kernel")
    nz, ny, nx = image_shape
    kd = _kdims(tuple(kernel.shape), flags)
    need = lib().fc_kernel_spectrum_bytes(_iarr([nx, ny, nz]), kd, int(flags))
    if need == 0:
        _check()
    buf = torch.empty(need, dtype=torch.uint8, device=kernel.device)
    _check(lib().fc_kernel_spectrum_device(kernel.data_ptr(), kd, _iarr([nx, ny, nz]), int(flags), buf.data_ptr(),
                                           need, _stream(stream)))
    return buf


def conv3d_kspec(image: torch.Tensor, kspec: torch.Tensor, kernel_shape: Optional[Sequence[int]],
                 out: Optional[torch.Tensor] = None, correlate: bool = False, flags: int = 0,
                 workspace: Optional[torch.Tensor] = None, stream: Optional[torch.cuda.Stream] = None) -> torch.Tensor:
    """Convolution (or correlation) of image with a kernel spectrum from kernel_spectrum()."""
    _f32(image, "image")
    nx, ny, nz = _dims(image)
    if out is None:
        out = torch.empty_like(image)
    _f32(out, "out")
    if correlate:
        flags |= FC_FLAG_CORRELATE
    need = lib().fc_conv3d_kspec_workspace_bytes(_iarr([nx, ny, nz]))
    if need == 0:
        _check()
    wp, wb = _ws(workspace, need, image.device)
    _check(lib().fc_conv3d_kspec_device(image.data_ptr(), out.data_ptr(), _iarr([nx, ny, nz]), kspec.data_ptr(),
                                        _kdims(kernel_shape, flags), int(flags), wp, wb, _stream(stream)))
    return out


def rl_deconvolve(observed: torch.Tensor, kernel: torch.Tensor, iterations: int,
                  estimate: Optional[torch.Tensor] = None, flags: int = 0, workspace: Optional[torch.Tensor] = None,
                  stream: Optional[torch.cuda.Stream] = None) -> torch.Tensor:
    """Richardson-Lucy deconvolution of observed [nz,ny,nx] by kernel [kz,ky,kx];
    estimate (updated in place) starts as a copy of observed when not given."""
    _f32(observed, "observed")
    _f32(kernel, "kernel")
    nx, ny, nz = _dims(observed)
    if estimate is None:
        estimate = observed.clone()
    _f32(estimate, "estimate")
    kd = _kdims(tuple(kernel.shape), flags)
    need = lib().fc_rl_workspace_bytes(_iarr([nx, ny, nz]), kd, int(flags))
    if need == 0:
        _check()
    wp, wb = _ws(workspace, need, observed.device)
    _check(lib().fc_rl_deconvolve_device(observed.data_ptr(), estimate.data_ptr(), _iarr([nx, ny, nz]),
                                         kernel.data_ptr(), kd, int(iterations), int(flags), wp, wb, _stream(stream)))
    return estimate


def subsampled_workspace_bytes(image_shape: Sequence[int], kernel_shape: Sequence[int]) -> int:
    """Bytes of scratch for conv3d_subsampled; shapes are torch order (z, y, x)."""
    nz, ny, nx = image_shape
    kz, ky, kx = kernel_shape
    n = lib().fc_conv3d_subsampled_workspace_bytes(_iarr([nx, ny, nz]), _iarr([kx, ky, kz]))
    if n == 0:
        _check()
    return int(n)


def conv3d_subsampled(image: torch.Tensor, kernel: torch.Tensor, out: Optional[torch.Tensor] = None,
                      workspace: Optional[torch.Tensor] = None,
                      stream: Optional[torch.cuda.Stream] = None) -> torch.Tensor:
    """Subsampled-kernel approximation of the convolution of image [nz,ny,nx]
    by kernel [kz,ky,kx] (fc_conv3d_subsampled_device): the kernel's spectrum
    at its own size, read at the nearest kernel frequency of each image
    frequency."""
    _f32(image, "image")
    _f32(kernel, "kernel")
    nx, ny, nz = _dims(image)
    kx, ky, kz = _dims(kernel)
    if out is None:
        out = torch.empty_like(image)
    _f32(out, "out")
    need = subsampled_workspace_bytes((nz, ny, nx), (kz, ky, kx))
    wp, wb = _ws(workspace, need, image.device)
    _check(lib().fc_conv3d_subsampled_device(image.data_ptr(), out.data_ptr(), _iarr([nx, ny, nz]),
                                             kernel.data_ptr(), _iarr([kx, ky, kz]), wp, wb, _stream(stream)))
    return out


def conv3d_adjoint(image: Optional[torch.Tensor], kernel: Optional[torch.Tensor], grad_out: torch.Tensor,
                   kernel_shape: Sequence[int], need_image_grad: bool = True, need_kernel_grad: bool = True,
                   flags: int = 0, workspace: Optional[torch.Tensor] = None,
                   stream: Optional[torch.cuda.Stream] = None):
    """Gradients of y = conv3d(image, kernel): (grad_image, grad_kernel)."""
    _f32(grad_out, "grad_out")
    nx, ny, nz = _dims(grad_out)
    kz, ky, kx = kernel_shape
    gi = torch.empty_like(grad_out) if need_image_grad else None
    gk = torch.empty((kz, ky, kx), dtype=torch.float32, device=grad_out.device) if need_kernel_grad else None
    need = lib().fc_conv3d_adjoint_workspace_bytes(_iarr([nx, ny, nz]), _iarr([kx, ky, kz]), int(flags))
    if need == 0:
        _check()
    wp, wb = _ws(workspace, need, grad_out.device)
    rc = lib().fc_conv3d_adjoint_device(
        image.data_ptr() if image is not None else None, kernel.data_ptr() if kernel is not None else None,
        grad_out.data_ptr(), gi.data_ptr() if gi is not None else None, gk.data_ptr() if gk is not None else None,
        _iarr([nx, ny, nz]), _iarr([kx, ky, kz]), int(flags), wp, wb, _stream(stream))
    _check(rc)
    return gi, gk


def conv3d_batched(images: List[torch.Tensor], kernels: List[torch.Tensor],
                   outs: Optional[List[torch.Tensor]] = None, flags: int = 0,
                   workspace: Optional[torch.Tensor] = None, stream: Optional[torch.cuda.Stream] = None):
    n = len(images)
    if n == 0 or len(kernels) != n:
        raise FcError(FC_ERR_ARG, "need one kernel per view")
    dims = []
    for im, k in zip(images, kernels):
        _f32(im, "image")
        _f32(k, "kernel")
        dims += [*_dims(im), *_dims(k)]
    if outs is None:
        outs = [torch.empty_like(im) for im in images]
    arr = lambda ts: (ctypes.c_void_p * n)(*[t.data_ptr() for t in ts])
    need = lib().fc_conv3d_batched_workspace_bytes(n, _iarr(dims), int(flags))
    if need == 0:
        _check()
    wp, wb = _ws(workspace, need, images[0].device)
    rc = lib().fc_conv3d_batched_device(n, arr(images), arr(outs), arr(kernels), _iarr(dims), int(flags), wp, wb,
                                        _stream(stream))
    _check(rc)
    return outs


def rfft3d(x: torch.Tensor, workspace: Optional[torch.Tensor] = None, stream=None) -> torch.Tensor:
    """Unnormalised 3D R2C of x [nz,ny,nx] -> complex64 [nz,ny,nx//2+1]."""
    _f32(x, "x")
    nx, ny, nz = _dims(x)
    spec = torch.empty((nz, ny, nx // 2 + 1), dtype=torch.complex64, device=x.device)
    need = lib().fc_fft3d_workspace_bytes(_iarr([nx, ny, nz]))
    wp, wb = _ws(workspace, need, x.device)
    _check(lib().fc_rfft3d_device(x.data_ptr(), spec.data_ptr(), _iarr([nx, ny, nz]), wp, wb, _stream(stream)))
    return spec


def irfft3d(spec: torch.Tensor, nx: int, workspace: Optional[torch.Tensor] = None, stream=None) -> torch.Tensor:
    """Unnormalised 3D C2R of spec [nz,ny,nx//2+1] -> float32 [nz,ny,nx]."""
    if not spec.is_cuda or spec.dtype != torch.complex64 or not spec.is_contiguous():
        raise FcError(FC_ERR_ARG, "spec must be a contiguous complex64 CUDA tensor")
    nz, ny, _ = spec.shape
    out = torch.empty((nz, ny, nx), dtype=torch.float32, device=spec.device)
    need = lib().fc_fft3d_workspace_bytes(_iarr([nx, ny, nz]))
    wp, wb = _ws(workspace, need, spec.device)
    _check(lib().fc_irfft3d_device(spec.data_ptr(), out.data_ptr(), _iarr([nx, ny, nz]), wp, wb, _stream(stream)))
    return out


def pad_shift_kernel(kernel: torch.Tensor, image_shape: Sequence[int], flags: int = 0, stream=None) -> torch.Tensor:
    """The zero-padded, shifted kernel as the convolution's first pass sees it."""
    _f32(kernel, "kernel")
    kx, ky, kz = _dims(kernel)
    nz, ny, nx = image_shape
    out = torch.empty((nz, ny, nx), dtype=torch.float32, device=kernel.device)
    _check(lib().fc_pad_shift_kernel_device(kernel.data_ptr(), _iarr([kx, ky, kz]), _iarr([nx, ny, nz]), int(flags),
                                            out.data_ptr(), _stream(stream)))
    return out


def profile(enable: Optional[bool] = None, only: Optional[str] = None) -> List[Tuple[str, float, float]]:
    """Enable/disable per-pass event timing (``only``: record just the pass of
    that name); with no argument, read and clear the records: list of
    (pass name, milliseconds, algorithmic bytes)."""
    L = lib()
    if enable is not None:
        L.fc_profile_only((only or "").encode())
        L.fc_profile_enable(1 if enable else 0)
        return []
    cap = 1 << 16
    names = ctypes.create_string_buffer(64 * cap)
    ms = (ctypes.c_float * cap)()
    by = (ctypes.c_double * cap)()
    n = L.fc_profile_read(names, 64, ms, by, cap)
    raw = names.raw
    return [(raw[64 * i: 64 * (i + 1)].split(b"\0", 1)[0].decode(), float(ms[i]), float(by[i])) for i in range(n)]


def launch_count() -> int:
    return lib().fc_launch_count()
