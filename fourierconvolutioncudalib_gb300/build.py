"""In-tree build of libFourierConvolutionCUDALib.so for sm_103a.

Two translation units (host orchestration + kernels) are compiled in parallel
with nvcc and linked into one shared library next to this file.  The CUDA
runtime is linked statically, so the library needs only the driver at run
time; symbols are hidden except the C ABI declared in include/convolution3Dfft.h.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB_NAME = "libFourierConvolutionCUDALib.so"
LIB_PATH = PKG / LIB_NAME

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden", "-I", str(ROOT / "include")]
# (source, object name, extra flags); fc_tc.cu is built once per 16-bit operand type
SOURCES = [(f, Path(f).stem, []) for f in [
    "fc_host.cpp", "fc_kernels.cu", "fc_fast_rows.cu", "fc_fast_cols.cu", "fc_fast_zconv.cu", "fc_fast_zadj.cu",
    "fc_batched_rows_fwd.cu", "fc_batched_rows_inv.cu", "fc_batched_cols_fwd.cu", "fc_batched_cols_inv.cu",
    "fc_batched_zconv.cu", "fc_noalloc.cu", "fc_fast_pipe.cu", "fc_fast_zsub.cu"]] + [
    ("fc_tc.cu", "fc_tc_fp16", ["-DFC_TC_MODE=1"]), ("fc_tc.cu", "fc_tc_bf16", ["-DFC_TC_MODE=2"])]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _sources_mtime() -> float:
    files = list(CSRC.glob("*")) + [ROOT / "include" / "convolution3Dfft.h", Path(__file__)]
    return max(f.stat().st_mtime for f in files if f.is_file())


def _compile(entry, verbose: bool) -> Path:
    src, stem, flags = entry
    obj = BUILD / (stem + ".o")
    extra = os.environ.get("FC_NVCC_EXTRA", "").split()  # e.g. -DFC_ZCONV_MIN_BLOCKS=3 for tuning builds
    cmd = [nvcc(), *COMMON, *ARCH, *flags, *extra, "-c", str(CSRC / src), "-o", str(obj)]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile the library if any source is newer than it; return its path."""
    if not force and LIB_PATH.exists() and LIB_PATH.stat().st_mtime >= _sources_mtime():
        return LIB_PATH
    BUILD.mkdir(exist_ok=True)
    workers = min(len(SOURCES), os.cpu_count() or 4)
    # longest translation units first
    order = sorted(SOURCES, key=lambda e: 0 if e[0].startswith(("fc_batched", "fc_fast_z", "fc_tc")) else 1)
    with ThreadPoolExecutor(max_workers=workers) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), order))
    tmp = BUILD / (LIB_NAME + ".tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs), "-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
