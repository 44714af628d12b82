"""Concurrent calls from several host threads (JNA callers such as Fiji
plugins call the library from many Java threads).

ctypes releases the GIL for the duration of a foreign call, so the threads
below run inside the library at the same time: the reference-facing InPlace
entry on host buffers (pageable and page-locked), and the device entry on one
CUDA stream per thread.  Every result is checked against the FP64 oracle with
the plain path's tolerance (rel-L2 <= 1e-5).
"""
import threading

import numpy as np
import pytest

import fourierconvolutioncudalib_gb300 as fc

pytestmark = pytest.mark.gpu

CASES = [((24, 40, 64), (5, 3, 7)), ((32, 64, 48), (7, 5, 3)), ((16, 96, 80), (3, 9, 5)), ((40, 32, 128), (9, 7, 5))]


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def _data(i):
    shape, kshape = CASES[i % len(CASES)]
    rng = np.random.default_rng(100 + i)
    im = rng.random(shape).astype(np.float32)
    k = rng.random(kshape).astype(np.float32)
    return im, k / k.sum()


def _run_threads(fn, n):
    errors = []

    def body(i):
        try:
            fn(i)
        except Exception as e:  # collected and re-raised in the main thread
            errors.append((i, repr(e)))

    ts = [threading.Thread(target=body, args=(i,)) for i in range(n)]
    for t in ts:
        t.start()
    for t in ts:
        t.join(300)
    assert not errors, errors


def test_inplace_entry_from_many_threads(cuda, orc):
    import torch

    results = {}

    def work(i):
        im, k = _data(i)
        nz, ny, nx = im.shape
        kz, ky, kx = k.shape
        if i % 2:  # page-locked buffer (direct host I/O)
            buf = torch.from_numpy(im.copy()).pin_memory().numpy()
        else:
            buf = im.copy()
        for _ in range(3):
            work_buf = buf.copy() if i % 2 == 0 else buf
            if i % 2:
                np.copyto(buf, im)
            fc.convolution3DfftCUDAInPlace(work_buf, (nx, ny, nz), k, (kx, ky, kz), 0)
            results.setdefault(i, []).append(work_buf.copy())

    _run_threads(work, 8)
    for i, outs in results.items():
        im, k = _data(i)
        ref = orc.conv_fp64(im, k, "centered")
        for o in outs:
            assert _rel(o, ref) <= 1e-5, i


def test_device_entry_from_many_threads_and_streams(cuda, orc):
    import torch
    from fourierconvolutioncudalib_gb300 import device as fcd

    outs = {}

    def work(i):
        im, k = _data(i)
        s = torch.cuda.Stream(device=cuda)
        with torch.cuda.stream(s):
            img = torch.from_numpy(im).to(cuda, non_blocking=False)
            ker = torch.from_numpy(k).to(cuda)
            res = []
            for _ in range(3):
                res.append(fcd.conv3d(img, ker, stream=s))
            s.synchronize()
            outs[i] = [r.cpu().numpy() for r in res]

    _run_threads(work, 8)
    for i, rs in outs.items():
        im, k = _data(i)
        ref = orc.conv_fp64(im, k, "centered")
        for r in rs:
            assert _rel(r, ref) <= 1e-5, i
