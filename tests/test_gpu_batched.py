"""The batched form: several volumes of uneven sizes, each with its own PSF,
through fc_conv3d_batched_device (one persistent launch per pass over a
device work-list, the sequence captured in a CUDA graph and replayed).

Tolerances: each view against the FP64 oracle, rel-L2 <= 1e-5 and max-abs <=
1e-5 * max|ref|; against the same view through the single-volume entry,
rel-L2 <= 1e-6 (same arithmetic, possibly different launch split).
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm((a - b).ravel()) / np.linalg.norm(b.ravel()))


def _views(rng, shapes):
    out = []
    for (nz, ny, nx), (kz, ky, kx) in shapes:
        im = rng.random((nz, ny, nx), dtype=np.float32)
        k = rng.random((kz, ky, kx), dtype=np.float32)
        out.append((im, k / k.sum()))
    return out


def _run_batched(cuda, views, workspace=None):
    import torch
    from fourierconvolutioncudalib_gb300 import device as fcd

    imgs = [torch.from_numpy(v[0]).to(cuda) for v in views]
    kers = [torch.from_numpy(v[1]).to(cuda) for v in views]
    outs = fcd.conv3d_batched(imgs, kers, workspace=workspace)
    torch.cuda.synchronize()
    return imgs, kers, outs


def test_batched_c4_views(cuda, orc):
    """The six multi-view shapes of the batched configuration, each with its
    own rotated anisotropic PSF."""
    import torch
    from fourierconvolutioncudalib_gb300 import device as fcd
    from fourierconvolutioncudalib_gb300 import workloads as W

    views = [(v["image"], v["kernel"]) for v in W.c4()]
    imgs, kers, outs = _run_batched(cuda, views)
    for (im, k), out in zip(views, outs):
        ref = orc.conv_fp64(im, k, "centered")
        got = out.cpu().numpy()
        assert _rel(got, ref) <= 1e-5
        assert np.max(np.abs(got - ref)) <= 1e-5 * np.max(np.abs(ref))
    for img, ker, out in zip(imgs, kers, outs):
        single = fcd.conv3d(img, ker)
        torch.cuda.synchronize()
        assert _rel(out.cpu().numpy(), single.cpu().numpy()) <= 1e-6


def test_batched_graph_replay_and_mixed_paths(cuda, orc):
    """Second call with the same buffers replays the captured graph; a view with
    a length outside the register-resident set (13*17) runs on the generic
    path inside the same call."""
    import torch
    from fourierconvolutioncudalib_gb300 import device as fcd

    rng = np.random.default_rng(31)
    views = _views(rng, [((24, 40, 64), (5, 7, 9)), ((13, 34, 221), (3, 5, 7)), ((32, 96, 160), (9, 9, 9))])
    imgs = [torch.from_numpy(v[0]).to(cuda) for v in views]
    kers = [torch.from_numpy(v[1]).to(cuda) for v in views]
    outs = [torch.empty_like(i) for i in imgs]
    dims = [(i.shape, k.shape) for i, k in zip(imgs, kers)]
    need = fcd.lib().fc_conv3d_batched_workspace_bytes(len(views), fcd._iarr([d for (s, ks) in dims for d in
                                                                               (s[2], s[1], s[0], ks[2], ks[1], ks[0])]),
                                                         0)
    ws = torch.empty(need, dtype=torch.uint8, device=cuda)
    fcd.conv3d_batched(imgs, kers, outs=outs, workspace=ws)
    torch.cuda.synchronize()
    first = [o.cpu().numpy().copy() for o in outs]
    for o in outs:
        o.zero_()
    # new input values in the same buffers: the replayed graph must pick them up
    for (im, _), t in zip(views, imgs):
        t.copy_(torch.from_numpy(im[::-1].copy()).to(cuda))
    fcd.conv3d_batched(imgs, kers, outs=outs, workspace=ws)
    torch.cuda.synchronize()
    for (im, k), f, o in zip(views, first, outs):
        assert _rel(f, orc.conv_fp64(im, k, "centered")) <= 1e-5
        assert _rel(o.cpu().numpy(), orc.conv_fp64(np.ascontiguousarray(im[::-1]), k, "centered")) <= 1e-5


def test_batched_autotune_cache(cuda, orc, tmp_path):
    """FC_AUTOTUNE=1 times the launch options of every pass once per shape
    signature and appends the choice to the cache file; results unchanged."""
    rng = np.random.default_rng(5)
    views = _views(rng, [((16, 48, 96), (3, 5, 7)), ((20, 64, 128), (5, 5, 5))])
    cache = tmp_path / "tune.txt"
    old = {k: os.environ.get(k) for k in ("FC_AUTOTUNE", "FC_TUNE_CACHE")}
    os.environ["FC_AUTOTUNE"] = "1"
    os.environ["FC_TUNE_CACHE"] = str(cache)
    try:
        _, _, outs = _run_batched(cuda, views)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    text = cache.read_text().strip().splitlines()
    assert len(text) == 1 and len(text[0].split()) == 7
    assert all(c in "012" for c in text[0].split()[1:6]) and text[0].split()[6] in "01234"
    for (im, k), out in zip(views, outs):
        assert _rel(out.cpu().numpy(), orc.conv_fp64(im, k, "centered")) <= 1e-5


def test_batched_every_schedule_and_choice(cuda, orc, tmp_path):
    """Each schedule (pass-major, view-major, view-concurrent, plain per view, plain concurrent) with the
    persistent work-list launches and with one launch per view, forced through
    the tuning cache; every view against the FP64 oracle."""
    rng = np.random.default_rng(9)
    views = _views(rng, [((16, 48, 96), (3, 5, 7)), ((20, 64, 128), (5, 5, 5)), ((24, 40, 64), (5, 7, 9))])
    cache = tmp_path / "tune.txt"
    old = {k: os.environ.get(k) for k in ("FC_AUTOTUNE", "FC_TUNE_CACHE")}
    keep = []  # earlier buffers stay allocated, so every run gets new pointers and a new graph entry
    try:
        os.environ["FC_TUNE_CACHE"] = str(cache)
        os.environ["FC_AUTOTUNE"] = "1"
        keep.append(_run_batched(cuda, views))
        sig = cache.read_text().split()[0]
        os.environ["FC_AUTOTUNE"] = "0"
        for sched in (0, 1, 2, 3, 4):
            for choice in (0, 2):
                cache.write_text(" ".join([sig] + [str(choice)] * 5 + [str(sched)]) + "\n")
                imgs, kers, outs = _run_batched(cuda, views)
                keep.append((imgs, kers, outs))
                import ctypes
                from fourierconvolutioncudalib_gb300 import device as fcd
                ch = (ctypes.c_int * 5)()
                assert fcd.lib().fc_batched_last_plan(ch) == sched and list(ch) == [choice] * 5
                for (im, k), out in zip(views, outs):
                    assert _rel(out.cpu().numpy(), orc.conv_fp64(im, k, "centered")) <= 1e-5, (sched, choice)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
