"""The tensor-core precision mode (FC_FLAG_TC_FP16 / FC_FLAG_TC_BF16): the
radix-16 stages of the 128..1024-point axes run as 32x32 real DFT products on
the tensor cores with per-column power-of-two scaling and hi+lo 16-bit
operands (fp32 accumulation).

Tolerances against the FP64 oracle (rel-L2 / max-abs relative to max|ref|):
  fp16 hi+lo (22 significant bits per operand):  <= 2e-6 / 1e-5
  bf16 hi+lo (16 significant bits per operand):  <= 1e-5 / 5e-5
The fp32 path is held to 1e-5 elsewhere; the TC mode is opt-in.
"""
import numpy as np
import pytest

import fourierconvolutioncudalib_gb300 as fc

pytestmark = pytest.mark.gpu

TOL = {"fp16": (2e-6, 1e-5), "bf16": (1e-5, 5e-5)}


@pytest.mark.parametrize("mode", ["fp16", "bf16"])
@pytest.mark.parametrize("shape,kshape", [((128, 256, 512), (15, 13, 11)), ((64, 128, 1024), (9, 9, 9)),
                                          ((96, 200, 256), (5, 7, 9))])
def test_tc_vs_fp64(cuda, orc, mode, shape, kshape):
    import torch
    from fourierconvolutioncudalib_gb300 import device as fcd

    rng = np.random.default_rng(sum(shape))
    im = (100 + 1000 * rng.random(shape)).astype(np.float32)  # positive, wide dynamic range like the spot data
    k = rng.random(kshape).astype(np.float32)
    k /= k.sum()
    flag = fc.FC_FLAG_TC_FP16 if mode == "fp16" else fc.FC_FLAG_TC_BF16
    out = fcd.conv3d(torch.from_numpy(im).to(cuda), torch.from_numpy(k).to(cuda), flags=flag)
    torch.cuda.synchronize()
    got = out.cpu().numpy().astype(np.float64)
    ref = orc.conv_fp64(im, k, "centered")
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    mx = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    print(f"tc {mode} {shape}: rel-L2 {rel:.3e} max-abs {mx:.3e}")
    assert rel <= TOL[mode][0]
    assert mx <= TOL[mode][1]


def test_tc_flags_exclusive(cuda):
    import torch
    from fourierconvolutioncudalib_gb300 import device as fcd

    x = torch.zeros((8, 8, 8), device=cuda)
    with pytest.raises(fc.FcError):
        fcd.conv3d(x, torch.ones((3, 3, 3), device=cuda), flags=fc.FC_FLAG_TC_FP16 | fc.FC_FLAG_TC_BF16)


@pytest.mark.parametrize("mode", ["fp16", "bf16"])
def test_tc_subnormal_psf_taps(cuda, orc, mode):
    """A narrow Gaussian PSF whose edge taps are subnormal floats: every column
    scale stays finite and the result meets the same FP64 tolerance."""
    import torch
    from fourierconvolutioncudalib_gb300 import device as fcd
    from fourierconvolutioncudalib_gb300 import workloads as W

    k = W.gaussian_psf((31, 31, 31), (1.2, 1.0, 1.0))
    tiny = k[(k > 0) & (k < np.finfo(np.float32).tiny)]
    assert tiny.size > 0  # the case needs subnormal taps
    im = W.spot_volume((64, 128, 256), 300, 3)
    flag = fc.FC_FLAG_TC_FP16 if mode == "fp16" else fc.FC_FLAG_TC_BF16
    out = fcd.conv3d(torch.from_numpy(im).to(cuda), torch.from_numpy(k).to(cuda), flags=flag)
    torch.cuda.synchronize()
    got = out.cpu().numpy().astype(np.float64)
    assert np.all(np.isfinite(got))
    ref = orc.conv_fp64(im, k, "centered")
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    mx = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    print(f"tc {mode} subnormal PSF: rel-L2 {rel:.3e} max-abs {mx:.3e}")
    assert rel <= TOL[mode][0]
    assert mx <= TOL[mode][1]
