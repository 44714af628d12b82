"""Loader for the cuFFT restatement of the reference's InPlace sequence
(refseq_cufft.cu) -- baseline timing and GPU parity only, not the product."""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess
from pathlib import Path
from typing import Optional

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "librefseq_cufft.so"
_lib: Optional[ctypes.CDLL] = None


def build(force: bool = False) -> Path:
    src = HERE / "refseq_cufft.cu"
    if not force and LIB.exists() and LIB.stat().st_mtime >= src.stat().st_mtime:
        return LIB
    BUILD.mkdir(exist_ok=True)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    tmp = BUILD / "librefseq_cufft.so.tmp"
    libdir = Path(nvcc).resolve().parent.parent / "lib64"
    cmd = [nvcc, "-std=c++17", "-O2", "-Xcompiler", "-fPIC,-fvisibility=hidden", "-gencode",
           "arch=compute_103a,code=sm_103a", "-shared", "-cudart", "static", str(src), "-o", str(tmp),
           "-L", str(libdir), "-lcufft", "-Xlinker", f"-rpath,{libdir}"]
    subprocess.run(cmd, check=True, capture_output=True)
    os.replace(tmp, LIB)
    return LIB


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB))
        IP = ctypes.POINTER(ctypes.c_int)
        FP = ctypes.POINTER(ctypes.c_float)
        L.refseq_inplace.restype = ctypes.c_int
        L.refseq_inplace.argtypes = [FP, IP, FP, IP, ctypes.c_int]
        L.refseq_device_only.restype = ctypes.c_int
        L.refseq_device_only.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_void_p]
        L.refseq_last_error.restype = ctypes.c_char_p
        L.refseq_release.restype = None
        _lib = L
    return _lib


def inplace(im: np.ndarray, kernel: np.ndarray, centered: bool = False) -> np.ndarray:
    """Run the restated reference InPlace sequence on a copy of im [nz,ny,nx]."""
    out = np.ascontiguousarray(im, np.float32).copy()
    k = np.ascontiguousarray(kernel, np.float32)
    nz, ny, nx = out.shape
    kz, ky, kx = k.shape
    IA = ctypes.c_int * 3
    FP = ctypes.POINTER(ctypes.c_float)
    rc = lib().refseq_inplace(out.ctypes.data_as(FP), IA(nx, ny, nz), k.ctypes.data_as(FP), IA(kx, ky, kz),
                              1 if centered else 0)
    if rc != 0:
        raise RuntimeError(lib().refseq_last_error().decode())
    return out
