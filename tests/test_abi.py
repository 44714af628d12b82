"""The C ABI library without a GPU: it loads, exports exactly what
include/convolution3Dfft.h declares, and its host-only logic (radix plans,
scratch estimates, argument validation) behaves.  No compute call is made."""
import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "convolution3Dfft.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = "\n".join(ln for ln in text.splitlines() if not ln.lstrip().startswith("#"))
    names = re.findall(r"FUNCTION_PREFIX\s+[\w\s\*]+?\b(\w+)\s*\(", text)
    return sorted(set(names))


REFERENCE_EXPORTS = [  # reference src/convolution3Dfft.h:29-84
    "convolution3DfftCUDA_test", "convolution3DfftCUDA", "convolution3DfftCUDAInPlace",
    "selectDeviceWithHighestComputeCapability", "getCUDAcomputeCapabilityMinorVersion",
    "getCUDAcomputeCapabilityMajorVersion", "getNumDevicesCUDA", "getNameDeviceCUDA", "getMemDeviceCUDA",
    "cuda_version", "gpu_mem_needed_mb",
]


def test_header_declares_reference_exports():
    decl = declared_functions()
    for name in REFERENCE_EXPORTS:
        assert name in decl, name


def test_library_exports_every_declared_symbol(fclib):
    import fourierconvolutioncudalib_gb300 as fc

    path = fc.library_path()
    out = subprocess.run(["nm", "-D", "--defined-only", str(path)], capture_output=True, text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    decl = set(declared_functions())
    assert decl <= exported, decl - exported
    # nothing else leaks out of the library (hidden visibility)
    assert exported <= decl, exported - decl
    for name in decl:
        assert hasattr(fclib, name)


def test_library_named_for_jna(fclib):
    import fourierconvolutioncudalib_gb300 as fc

    assert fc.library_path().name == "libFourierConvolutionCUDALib.so"


def test_plan_radices(fclib):
    import fourierconvolutioncudalib_gb300 as fc

    assert fc.plan_radices(512) == [8, 8, 8]
    assert fc.plan_radices(128) == [16, 8]
    assert fc.plan_radices(256) == [16, 16]
    assert fc.plan_radices(384) == [16, 8, 3]
    assert fc.plan_radices(448) == [8, 8, 7]
    assert fc.plan_radices(96) == [8, 4, 3]
    assert fc.plan_radices(352) == [8, 4, 11]
    assert fc.plan_radices(218) == [2, 109]
    assert fc.plan_radices(13 * 17) == [13, 17]
    assert fc.plan_radices(1) == [1]
    for n in (2, 3, 60, 343, 1000, 1024, 4096, 158, 148, 168, 4093):
        r = fc.plan_radices(n)
        assert int(np.prod(r)) == n


def test_gpu_mem_needed_is_host_only(fclib):
    import fourierconvolutioncudalib_gb300 as fc

    mb = fc.gpu_mem_needed_mb([128, 512, 512])
    # spectrum + kernel spectrum (same size here) + image + kernel: ~ 4 x 140 MB
    assert 400 < mb < 700
    assert fc.gpu_mem_needed_mb([64]) >= 0
    assert fc.lib().gpu_mem_needed_mb(fc._iarr([0, 4, 4]), 3) == -1
    assert fc.lib().fc_last_status() == fc.FC_ERR_ARG


def test_workspace_bytes_monotone(fclib):
    import fourierconvolutioncudalib_gb300 as fc

    L = fc.lib()
    a = L.fc_conv3d_workspace_bytes(fc._iarr([512, 512, 128]), fc._iarr([31, 31, 63]), 0)
    b = L.fc_conv3d_workspace_bytes(fc._iarr([512, 512, 128]), fc._iarr([63, 63, 127]), 0)
    c = L.fc_conv3d_workspace_bytes(fc._iarr([512, 512, 128]), fc._iarr([31, 31, 63]), fc.FC_FLAG_SHIFT_COMPAT)
    assert 0 < a < b <= c
    assert L.fc_conv3d_workspace_bytes(fc._iarr([512, 512, 128]), fc._iarr([513, 1, 1]), 0) == 0
    assert L.fc_last_status() == fc.FC_ERR_ARG


def test_argument_validation_without_gpu(fclib):
    """Invalid calls fail with a status before any device work, and never exit."""
    import fourierconvolutioncudalib_gb300 as fc

    L = fc.lib()
    im = np.ones((4, 4, 4), np.float32)
    k = np.ones((3, 3, 3), np.float32)
    FP = ctypes.POINTER(ctypes.c_float)
    L.convolution3DfftCUDAInPlace(None, fc._iarr([4, 4, 4]), k.ctypes.data_as(FP), fc._iarr([3, 3, 3]), 0)
    assert L.fc_last_status() == fc.FC_ERR_ARG
    L.convolution3DfftCUDAInPlace(im.ctypes.data_as(FP), fc._iarr([4, 0, 4]), k.ctypes.data_as(FP),
                                  fc._iarr([3, 3, 3]), 0)
    assert L.fc_last_status() == fc.FC_ERR_ARG
    L.convolution3DfftCUDAInPlace(im.ctypes.data_as(FP), fc._iarr([4, 4, 4]), k.ctypes.data_as(FP),
                                  fc._iarr([5, 3, 3]), 0)
    assert L.fc_last_status() == fc.FC_ERR_ARG
    assert np.all(im == 1)
    assert not L.convolution3DfftCUDA(im.ctypes.data_as(FP), None, k.ctypes.data_as(FP), fc._iarr([3, 3, 3]), 0)
    assert L.fc_last_status() == fc.FC_ERR_ARG
    assert L.fc_conv3d_device(None, None, fc._iarr([4, 4, 4]), None, fc._iarr([3, 3, 3]), 0, None, 0, None) == \
        fc.FC_ERR_ARG
    msg = L.fc_last_error().decode()
    assert "NULL" in msg
    with pytest.raises(fc.FcError):
        fc.convolution3DfftCUDAInPlace(im, (4, 4, 4), np.ones((3, 3), np.float32), (3, 3, 1), 0)


def test_fault_controls_validate_without_gpu(fclib):
    """The failure-path test controls check their arguments on the host:
    allocation fault specifications are "alloc:n" (n >= 1) or "off", and a
    negative wait limit is refused before any device is touched."""
    import fourierconvolutioncudalib_gb300 as fc

    L = fc.lib()
    try:
        for good in (b"alloc:1", b"alloc:25", b"off", b""):
            assert L.fc_fault_inject(good) == fc.FC_OK, good
        for bad in (b"alloc:0", b"alloc:-2", b"alloc:", b"alloc:3x", b"free:1", b"oom"):
            assert L.fc_fault_inject(bad) == fc.FC_ERR_ARG, bad
            assert "alloc:n" in L.fc_last_error().decode()
    finally:
        assert L.fc_fault_inject(b"off") == fc.FC_OK
    assert L.fc_test_set_wait_fault(-1, 0) == fc.FC_ERR_ARG


def test_version_and_cuda_version(fclib):
    import fourierconvolutioncudalib_gb300 as fc

    assert b"sm_103a" in fc.lib().fc_version()
    assert fc.cuda_version() >= 13000


def test_reuse_rl_and_batched_plan_entries_without_gpu(fclib):
    """The kernel-spectrum, Richardson-Lucy and batched-plan entries validate
    their arguments on the host: sizes grow with the shapes, bad shapes and
    the compat placement are refused with a status, NULL pointers never reach
    the device, and no batched call has a plan yet."""
    import fourierconvolutioncudalib_gb300 as fc

    L = fc.lib()
    small = L.fc_kernel_spectrum_bytes(fc._iarr([64, 64, 32]), fc._iarr([5, 5, 5]), 0)
    big = L.fc_kernel_spectrum_bytes(fc._iarr([64, 64, 32]), fc._iarr([5, 5, 9]), 0)
    assert 0 < small < big  # kernel planes are kept pruned to the kernel's depth
    assert L.fc_conv3d_kspec_workspace_bytes(fc._iarr([64, 64, 32])) > 0
    assert L.fc_rl_workspace_bytes(fc._iarr([64, 64, 32]), fc._iarr([5, 5, 5]), 0) > \
        L.fc_conv3d_kspec_workspace_bytes(fc._iarr([64, 64, 32]))
    assert L.fc_kernel_spectrum_bytes(fc._iarr([64, 64, 32]), fc._iarr([65, 5, 5]), 0) == 0
    assert L.fc_last_status() == fc.FC_ERR_ARG
    assert L.fc_kernel_spectrum_bytes(fc._iarr([64, 64, 32]), fc._iarr([5, 5, 5]), fc.FC_FLAG_SHIFT_COMPAT) == 0
    assert L.fc_last_status() == fc.FC_ERR_UNSUPPORTED
    assert L.fc_kernel_spectrum_device(None, fc._iarr([5, 5, 5]), fc._iarr([64, 64, 32]), 0, None, 0, None) == \
        fc.FC_ERR_ARG
    assert L.fc_conv3d_kspec_device(None, None, fc._iarr([64, 64, 32]), None, fc._iarr([5, 5, 5]), 0, None, 0,
                                    None) == fc.FC_ERR_ARG
    assert L.fc_rl_deconvolve_device(None, None, fc._iarr([64, 64, 32]), None, fc._iarr([5, 5, 5]), 3, 0, None, 0,
                                     None) == fc.FC_ERR_ARG
    assert L.fc_batched_last_plan(None) == -1
    # subsampled kernel: only the image spectrum and the kernel's own-size
    # spectrum, less than the plain path's padded kernel planes
    sub = L.fc_conv3d_subsampled_workspace_bytes(fc._iarr([64, 64, 32]), fc._iarr([5, 5, 9]))
    assert 0 < sub < L.fc_conv3d_workspace_bytes(fc._iarr([64, 64, 32]), fc._iarr([5, 5, 9]), 0)
    assert L.fc_conv3d_subsampled_workspace_bytes(fc._iarr([64, 64, 32]), fc._iarr([5, 5, 33])) == 0
    assert L.fc_last_status() == fc.FC_ERR_ARG
    assert L.fc_conv3d_subsampled_device(None, None, fc._iarr([64, 64, 32]), None, fc._iarr([5, 5, 5]), None, 0,
                                         None) == fc.FC_ERR_ARG
    FP = ctypes.POINTER(ctypes.c_float)
    k = np.ones((3, 3, 3), np.float32)
    L.convolution3DfftCUDAInPlaceSaveMemory(None, fc._iarr([4, 4, 4]), k.ctypes.data_as(FP), fc._iarr([3, 3, 3]), 0)
    assert L.fc_last_status() == fc.FC_ERR_ARG


def test_other_entries_refuse_bad_arguments_without_gpu(fclib):
    """The adjoint, batched, transform and placement entries check their
    arguments on the host: bad shapes give a zero workspace size with
    FC_ERR_ARG, and NULL pointers (including one view's pointer in a batch)
    are refused before any device work."""
    import fourierconvolutioncudalib_gb300 as fc

    L = fc.lib()
    I = fc._iarr
    assert L.fc_conv3d_adjoint_workspace_bytes(I([64, 64, 32]), I([5, 5, 5]), 0) > 0
    assert L.fc_conv3d_adjoint_workspace_bytes(I([64, 64, 32]), I([65, 5, 5]), 0) == 0
    assert L.fc_last_status() == fc.FC_ERR_ARG
    assert L.fc_fft3d_workspace_bytes(I([64, 64, 32])) > 0
    assert L.fc_fft3d_workspace_bytes(I([0, 64, 32])) == 0
    assert L.fc_last_status() == fc.FC_ERR_ARG
    two = I([64, 64, 32, 5, 5, 5, 32, 32, 16, 3, 3, 3])
    assert L.fc_conv3d_batched_workspace_bytes(2, two, 0) > L.fc_conv3d_batched_workspace_bytes(1, two, 0) > 0
    assert L.fc_conv3d_batched_workspace_bytes(0, None, 0) == 0
    assert L.fc_last_status() == fc.FC_ERR_ARG
    assert L.fc_rfft3d_device(None, None, I([8, 8, 8]), None, 0, None) == fc.FC_ERR_ARG
    assert L.fc_irfft3d_device(None, None, I([8, 8, 8]), None, 0, None) == fc.FC_ERR_ARG
    assert L.fc_pad_shift_kernel_device(None, I([3, 3, 3]), I([8, 8, 8]), 0, None, None) == fc.FC_ERR_ARG
    assert L.fc_conv3d_adjoint_device(None, None, None, None, None, I([8, 8, 8]), I([3, 3, 3]), 0, None, 0,
                                      None) == fc.FC_ERR_ARG
    P = ctypes.c_void_p
    views = (P * 2)(P(4096), None)  # the second view's pointer is NULL
    rc = L.fc_conv3d_batched_device(2, views, views, views, I([8, 8, 8, 3, 3, 3, 8, 8, 8, 3, 3, 3]), 0, None, 0,
                                    None)
    assert rc == fc.FC_ERR_ARG
    assert "view 1" in L.fc_last_error().decode()


def test_device_wrappers_refuse_host_tensors(fclib):
    """The torch wrappers accept only contiguous float32 CUDA tensors and say
    so before calling the library."""
    torch = pytest.importorskip("torch")
    import fourierconvolutioncudalib_gb300 as fc
    from fourierconvolutioncudalib_gb300 import device as fcd

    img = torch.zeros((8, 8, 8))
    ker = torch.ones((3, 3, 3)) / 27
    for call in (lambda: fcd.conv3d(img, ker), lambda: fcd.conv3d_subsampled(img, ker),
                 lambda: fcd.rl_deconvolve(img, ker, 1), lambda: fcd.kernel_spectrum(ker, (8, 8, 8))):
        with pytest.raises(fc.FcError, match="CUDA tensor"):
            call()


def test_header_compiles_as_c_and_links_from_cpp(fclib, tmp_path):
    """include/convolution3Dfft.h is usable from C (C99) and from C++, with
    the reference header's constants (MAX_THREADS_CUDA, MAX_BLOCKS_CUDA,
    dimsImage; src/convolution3Dfft.h:18-21), and a C++ program that calls
    the reference entry points links against the library by its JNA name
    (built, not run: running needs a GPU)."""
    import shutil

    import fourierconvolutioncudalib_gb300 as fc

    gcc, gxx = shutil.which("gcc"), shutil.which("g++")
    if not gcc or not gxx:
        pytest.skip("no host C/C++ compiler")
    inc = str(ROOT / "include")
    c_src = tmp_path / "use.c"
    c_src.write_text('#include "convolution3Dfft.h"\n'
                     'int main(void) { int d[3] = {8, 8, 8}; float im[512], k[27];\n'
                     '  convolution3DfftCUDAInPlace(im, d, k, d, 0);\n'
                     '  return fc_last_status() + (MAX_THREADS_CUDA != 1024) + (MAX_BLOCKS_CUDA != 65535)\n'
                     '         + (dimsImage != 3); }\n')
    subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", inc, "-c", str(c_src), "-o",
                    str(tmp_path / "use.o")], check=True)
    cpp_src = tmp_path / "use.cpp"
    cpp_src.write_text('#include "convolution3Dfft.h"\n'
                       'static_assert(MAX_THREADS_CUDA == 1024 && MAX_BLOCKS_CUDA == 65535 && dimsImage == 3, "");\n'
                       'int main() { int d[dimsImage] = {8, 8, 8};\n'
                       '  float* out = convolution3DfftCUDA(nullptr, d, nullptr, d, 0);\n'
                       '  fc_free_result(out); return getNumDevicesCUDA() < 0; }\n')
    lib = fc.library_path()
    subprocess.run([gxx, "-std=c++11", "-Wall", "-Wextra", "-Werror", "-I", inc, str(cpp_src), "-L", str(lib.parent),
                    "-lFourierConvolutionCUDALib", "-Wl,-rpath," + str(lib.parent), "-o", str(tmp_path / "use")],
                   check=True)
