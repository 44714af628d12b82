"""The reference library's own GPU build -- TEST INFRASTRUCTURE ONLY.

oracle/build_ref.sh compiles FourierConvolutionCUDALib from its unmodified
sources (src/convolution3Dfft.cu, src/standardCUDAfunctions.cu) with cuFFT
into oracle/_ref/libfc_reference.so.  This module runs that library, for the
parity tests (our output against the reference's on the same inputs) and for
the timing of the reference's GPU build beside ours.  Only tests/ and bench.py
use it; the product never does.

Every call runs in a child process (a fresh interpreter, not a fork): the
reference ends its process with exit() on a CUDA error (src/book.h:22-30) and
throws C++ exceptions through its C ABI on cuFFT errors (src/book.h:112-121),
and neither should take down the calling test or benchmark.  The child loads
only numpy, ctypes and the reference library.

Callers pass only shapes that the reference handles within its buffers: the
InPlace entry's kernel placement (src/convolution3Dfft.cu:128-166, :442-461)
stays inside the padded kernel when the kernel is no larger than the image on
every axis, which `oracle.ref_inplace_padded_kernel` checks (it raises for
shapes that would write outside).
"""
from __future__ import annotations

import ctypes
import json
import os
import platform
import subprocess
import sys
import tempfile
import time
from pathlib import Path
from typing import Dict, List, Optional, Sequence

import numpy as np

HERE = Path(__file__).resolve().parent
REF_DIR = HERE / "_ref"
LIB = REF_DIR / "libfc_reference.so"
SUBLIB = REF_DIR / "libfc_reference_sub.so"


def build() -> Optional[Path]:
    """Run build_ref.sh; the library's path, or None where no sources exist."""
    r = subprocess.run(["bash", str(HERE / "build_ref.sh")], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed: " + (r.stderr or r.stdout)[-2000:])
    return library_path()


def library_path() -> Optional[Path]:
    """The built library when it was built for this host's architecture."""
    tag = REF_DIR / ".built_for"
    if LIB.exists() and SUBLIB.exists() and tag.exists() and tag.read_text().strip() == platform.machine():
        return LIB
    return None


def available() -> bool:
    try:
        return build() is not None
    except RuntimeError:
        return False


# ------------------------------------------------------------------ parent side
def _run_child(spec: dict, arrays: Dict[str, np.ndarray], timeout: float = 600.0) -> Dict[str, np.ndarray]:
    lib = library_path()
    if lib is None:
        raise RuntimeError("the reference library is not built for this host (oracle/build_ref.sh)")
    with tempfile.TemporaryDirectory(prefix="fc_ref_") as td:
        fin = Path(td) / "in.npz"
        fout = Path(td) / "out.npz"
        np.savez(fin, **arrays)
        spec = dict(spec, lib=str(lib), fin=str(fin), fout=str(fout))
        env = dict(os.environ)
        env["PYTHONPATH"] = str(HERE.parent) + os.pathsep + env.get("PYTHONPATH", "")
        r = subprocess.run([sys.executable, "-m", "oracle.reference_gpu", json.dumps(spec)], capture_output=True,
                           text=True, timeout=timeout, env=env, cwd=str(HERE.parent))
        if r.returncode != 0 or not fout.exists():
            raise RuntimeError(f"reference child failed (rc {r.returncode}): {(r.stdout + r.stderr)[-1500:]}")
        with np.load(fout) as z:
            return {k: z[k] for k in z.files}


def inplace(image: np.ndarray, kernel: np.ndarray, device: int = 0) -> np.ndarray:
    """convolution3DfftCUDAInPlace of the reference on a copy of image [nz][ny][nx]
    with kernel [kz][ky][kx] (imDim = {nx,ny,nz}, kernelDim = {kx,ky,kz})."""
    return inplace_many([(image, kernel)], device)[0]


def inplace_many(cases: Sequence, device: int = 0) -> List[np.ndarray]:
    """Several InPlace calls in one child process (one CUDA context)."""
    arrays = {}
    for i, (im, k) in enumerate(cases):
        arrays[f"im{i}"] = np.ascontiguousarray(im, np.float32)
        arrays[f"k{i}"] = np.ascontiguousarray(k, np.float32)
    out = _run_child({"op": "inplace", "n": len(cases), "device": device}, arrays)
    return [out[f"out{i}"] for i in range(len(cases))]


def noninplace(image: np.ndarray, kernel: np.ndarray, device: int = 0) -> np.ndarray:
    """convolution3DfftCUDA of the reference: dims slowest-first for both arrays
    (imDim = {nz,ny,nx}, kernelDim = {kz,ky,kx}); returns its new[] result."""
    out = _run_child({"op": "noninplace", "device": device},
                     {"im0": np.ascontiguousarray(image, np.float32), "k0": np.ascontiguousarray(kernel, np.float32)})
    return out["out0"]


def time_inplace(image: np.ndarray, kernel: np.ndarray, reps: int, warmup: int = 2, device: int = 0) -> dict:
    """Wall time of convolution3DfftCUDAInPlace calls on pageable host buffers
    (the image restored before each call, outside the timed call); returns
    the per-call seconds and the output of the last call."""
    out = _run_child({"op": "time_inplace", "reps": int(reps), "warmup": int(warmup), "device": device},
                     {"im0": np.ascontiguousarray(image, np.float32), "k0": np.ascontiguousarray(kernel, np.float32)},
                     timeout=1800.0)
    return {"seconds": [float(s) for s in out["seconds"]], "output": out["out0"]}


def subsampled(image: np.ndarray, kernel: np.ndarray, device: int = 0) -> np.ndarray:
    """The reference's subsampled-kernel product (modulateAndNormalizeSubsampled_kernel,
    src/convolution3Dfft.cu:65-125) driven by oracle/ref_subsampled.cu: cuFFT R2C of
    the image and of the kernel at their own sizes, the reference's kernel,
    cuFFT C2R.  image [nz][ny][nx], kernel [kz][ky][kx]."""
    out = _run_child({"op": "subsampled", "device": device},
                     {"im0": np.ascontiguousarray(image, np.float32), "k0": np.ascontiguousarray(kernel, np.float32)})
    return out["out0"]


def device_queries(device: int = 0) -> dict:
    """The reference's device-query exports (src/standardCUDAfunctions.cu:13-71,
    src/convolution3Dfft.cu:581-584) for one device."""
    out = _run_child({"op": "queries", "device": device}, {"dummy": np.zeros(1, np.float32)})
    return json.loads(bytes(out["json"]).decode())


# ------------------------------------------------------------------ child side
def _bind(path: str) -> ctypes.CDLL:
    L = ctypes.CDLL(path, mode=ctypes.RTLD_LOCAL)
    FP = ctypes.POINTER(ctypes.c_float)
    IP = ctypes.POINTER(ctypes.c_int)
    L.convolution3DfftCUDAInPlace.restype = None
    L.convolution3DfftCUDAInPlace.argtypes = [FP, IP, FP, IP, ctypes.c_int]
    L.convolution3DfftCUDA.restype = FP
    L.convolution3DfftCUDA.argtypes = [FP, IP, FP, IP, ctypes.c_int]
    L.getNumDevicesCUDA.restype = ctypes.c_int
    L.getCUDAcomputeCapabilityMajorVersion.restype = ctypes.c_int
    L.getCUDAcomputeCapabilityMajorVersion.argtypes = [ctypes.c_int]
    L.getCUDAcomputeCapabilityMinorVersion.restype = ctypes.c_int
    L.getCUDAcomputeCapabilityMinorVersion.argtypes = [ctypes.c_int]
    L.selectDeviceWithHighestComputeCapability.restype = ctypes.c_int
    L.getNameDeviceCUDA.restype = None
    L.getNameDeviceCUDA.argtypes = [ctypes.c_int, ctypes.c_char_p]
    L.getMemDeviceCUDA.restype = ctypes.c_longlong
    L.getMemDeviceCUDA.argtypes = [ctypes.c_int]
    L.cuda_version.restype = ctypes.c_int
    return L


def _child(spec: dict) -> None:
    L = _bind(spec["lib"])
    FP = ctypes.POINTER(ctypes.c_float)
    IA = ctypes.c_int * 3
    dev = int(spec["device"])
    with np.load(spec["fin"]) as z:
        arrays = {k: z[k] for k in z.files}
    out: Dict[str, np.ndarray] = {}
    op = spec["op"]
    if op in ("inplace", "time_inplace"):
        n = int(spec.get("n", 1))
        for i in range(n):
            im = arrays[f"im{i}"]
            k = arrays[f"k{i}"]
            nz, ny, nx = im.shape
            kz, ky, kx = k.shape
            kc = np.ascontiguousarray(k, np.float32)
            if op == "inplace":
                buf = np.ascontiguousarray(im, np.float32).copy()
                L.convolution3DfftCUDAInPlace(buf.ctypes.data_as(FP), IA(nx, ny, nz), kc.ctypes.data_as(FP),
                                              IA(kx, ky, kz), dev)
                out[f"out{i}"] = buf
            else:
                buf = np.empty_like(im)
                secs = []
                for r in range(int(spec["warmup"]) + int(spec["reps"])):
                    np.copyto(buf, im)
                    t = time.perf_counter()
                    L.convolution3DfftCUDAInPlace(buf.ctypes.data_as(FP), IA(nx, ny, nz), kc.ctypes.data_as(FP),
                                                  IA(kx, ky, kz), dev)
                    dt = time.perf_counter() - t
                    if r >= int(spec["warmup"]):
                        secs.append(dt)
                out["seconds"] = np.asarray(secs, np.float64)
                out[f"out{i}"] = buf
    elif op == "noninplace":
        im = np.ascontiguousarray(arrays["im0"], np.float32)
        k = np.ascontiguousarray(arrays["k0"], np.float32)
        p = L.convolution3DfftCUDA(im.ctypes.data_as(FP), IA(*im.shape), k.ctypes.data_as(FP), IA(*k.shape), dev)
        res = np.ctypeslib.as_array(p, shape=(im.size,)).reshape(im.shape).copy()
        out["out0"] = res  # the new[] buffer is left to the process exit
    elif op == "subsampled":
        S = ctypes.CDLL(str(Path(spec["lib"]).parent / "libfc_reference_sub.so"), mode=ctypes.RTLD_LOCAL)
        S.fcref_subsampled.restype = ctypes.c_int
        S.fcref_subsampled.argtypes = [FP, ctypes.c_int, ctypes.c_int, ctypes.c_int, FP, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int, FP, ctypes.c_int]
        im = np.ascontiguousarray(arrays["im0"], np.float32)
        k = np.ascontiguousarray(arrays["k0"], np.float32)
        res = np.empty_like(im)
        rc = S.fcref_subsampled(im.ctypes.data_as(FP), *im.shape, k.ctypes.data_as(FP), *k.shape,
                                res.ctypes.data_as(FP), dev)
        if rc != 0:
            raise RuntimeError(f"fcref_subsampled failed with code {rc}")
        out["out0"] = res
    elif op == "queries":
        n = L.getNumDevicesCUDA()  # initialises the runtime (and the driver) first
        name = ctypes.create_string_buffer(256)
        L.getNameDeviceCUDA(dev, name)
        d = {"num_devices": n, "cc_major": L.getCUDAcomputeCapabilityMajorVersion(dev),
             "cc_minor": L.getCUDAcomputeCapabilityMinorVersion(dev),
             "highest_cc_device": L.selectDeviceWithHighestComputeCapability(),
             "name": name.value.decode(errors="replace"), "mem": int(L.getMemDeviceCUDA(dev)),
             "cuda_version": L.cuda_version()}
        out["json"] = np.frombuffer(json.dumps(d).encode(), np.uint8)
    else:
        raise ValueError(op)
    np.savez(spec["fout"], **out)


if __name__ == "__main__":
    _child(json.loads(sys.argv[1]))
