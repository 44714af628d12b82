"""Parity of the convolution under each pass-kernel selection.

The library picks, per pass, a persistent kernel whose tiles arrive by
asynchronous copies (x passes: bulk copies; fused z pass: tensor-map copies of
the image tile and of the kernel planes; y passes, when selected: tensor-map
copies) with programmatic dependent launch, or a one-tile-per-CTA kernel.  The
selection is read from the environment once per process (FC_PIPE, FC_YPIPE,
FC_ZPIPE, and FC_PDL, a mask of the pass kinds launched with programmatic
dependent launch), so each variant runs in a child process.  Tolerance: rel-L2
<= 1e-5 and max-abs <= 1e-5 * max against the FP64 oracle, on shapes that
include columns longer than 256 (z = 300, 512, 1024: the tensor-map stage in
two or four boxes) and spectra whose last one or two columns go in 8-row tiles
with a partial last tile (x = 34 and 96 with y = 36 and 44).
"""
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent

CHILD = r"""
import numpy as np, torch, sys
sys.path.insert(0, sys.argv[1])
import fourierconvolutioncudalib_gb300 as fc
from fourierconvolutioncudalib_gb300 import device as fcd
from oracle import oracle as orc
fc.load_library()
rng = np.random.default_rng(5)
for shape, kshape in (((128, 512, 512), (63, 31, 31)), ((96, 448, 384), (31, 15, 21)), ((200, 96, 224), (7, 5, 9)),
                      ((300, 64, 64), (9, 9, 9)), ((512, 32, 48), (15, 5, 7)), ((1024, 16, 32), (21, 3, 3)),
                      ((64, 36, 34), (9, 5, 5)), ((128, 44, 96), (15, 7, 9))):
    im = rng.random(shape, dtype=np.float32)
    k = rng.random(kshape, dtype=np.float32)
    k /= k.sum()
    out = fcd.conv3d(torch.from_numpy(im).cuda(), torch.from_numpy(k).cuda()).cpu().numpy()
    ref = orc.conv_fp64(im, k, "centered")
    rel = orc.rel_l2(out, ref)
    mx = orc.max_abs(out, ref) / float(np.max(np.abs(ref)))
    print(shape, kshape, "rel-L2 %.3e max-abs %.3e" % (rel, mx))
    assert rel <= 1e-5 and mx <= 1e-5, (shape, rel, mx)
print("ok")
"""


@pytest.mark.parametrize("env", [{}, {"FC_YPIPE": "1"}, {"FC_YPIPE": "0"}, {"FC_ZPIPE": "0"}, {"FC_PDL": "0"},
                                 {"FC_PDL": "5"}, {"FC_PIPE": "0", "FC_PDL": "0", "FC_YPIPE": "1"}],
                         ids=["default", "y-tensor-map-all", "y-one-tile-per-cta", "z-one-tile-per-cta", "no-pdl",
                              "pdl-x-and-z-only", "x-one-tile-per-cta"])
def test_pass_kernel_variants(cuda, fclib, env):
    e = dict(os.environ)
    e.update(env)
    r = subprocess.run([sys.executable, "-c", CHILD, str(ROOT)], env=e, capture_output=True, text=True, timeout=600)
    print(r.stdout[-2000:])
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout[-1500:] + r.stderr[-1500:]
