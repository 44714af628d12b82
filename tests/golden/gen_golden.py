"""Generate the committed golden fixtures of tests/golden/.

Sources (no FFT involved, so they pin the oracle rather than come from it):
  * the reference test suite's known-answer convolutions (test_gpu_convolve.cpp,
    test_gpu_numerical_stability.cpp) with their closed-form expectations or
    the reference's own CPU direct sum (tests/test_algorithms.hpp:10-58,
    restated in oracle/fc_oracle.c);
  * the reference's kernel placement (fftShiftKernel + row copy of
    src/convolution3Dfft.cu:128-166, :442-486) for a few small shapes, where
    the expected buffer is also written out by hand below (hand_cases).

Run from the repository root:  python tests/golden/gen_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle as orc  # noqa: E402

OUT = Path(__file__).resolve().parent


def hand_cases():
    """Placements worked out by hand from the reference's index formula.

    Image (nx,ny,nz) = (4,3,2), kernel (kx,ky,kz) = (1,1,2) with taps [a, b]
    stored [kz][ky][kx] = [[[a]],[[b]]].  The reference decomposes tap tid with
    kernelDim_2 = kz = 2 fastest: tid 0 -> (x,y,z) = (0,0,0), tid 1 -> (0,0,1);
    centring subtracts (kx/2, ky/2, kz/2) = (0,0,1): tid 0 -> z = -1 -> +nz = 1,
    tid 1 -> z = 0.  Destination z + nz*(y + ny*x): tid 0 -> 1, tid 1 -> 0.
    Read back as [nz][ny][nx]: flat 0 = (z0,y0,x0) holds b, flat 1 = (z0,y0,x1)
    holds a -- the z-tap a lands on the x axis.  The centred placement puts b
    at (0,0,0) and a at (z=1,y=0,x=0) = flat 12."""
    a, b = 3.0, 5.0
    k = np.array([[[a]], [[b]]], np.float32)
    ref = np.zeros((2, 3, 4), np.float32)
    ref.reshape(-1)[0] = b
    ref.reshape(-1)[1] = a
    cen = np.zeros((2, 3, 4), np.float32)
    cen.reshape(-1)[0] = b
    cen.reshape(-1)[12] = a
    return k, ref, cen


def main() -> None:
    cases = orc.kat_cases(include_large=False)
    arrays = {}
    names = []
    for c in cases:
        n = c["name"]
        names.append(n)
        arrays[f"{n}/image"] = c["image"]
        arrays[f"{n}/kernel"] = c["kernel"]
        arrays[f"{n}/off"] = np.array(c["off"], np.int32)
        arrays[f"{n}/shape"] = np.array(c["shape"], np.int32)
        arrays[f"{n}/expected"] = c["expected"]
        arrays[f"{n}/reference_expected"] = c.get("reference_expected", c["expected"])
        arrays[f"{n}/threshold"] = np.array(c["threshold"], np.float64)
    arrays["names"] = np.array(names)
    np.savez_compressed(OUT / "kat_small.npz", **arrays)

    k, ref, cen = hand_cases()
    rng = np.random.default_rng(20240601)
    place = {"hand/kernel": k, "hand/reference": ref, "hand/centered": cen}
    for i, (shape, kshape) in enumerate([((6, 10, 12), (5, 3, 3)), ((21, 19, 15), (3, 3, 3)), ((8, 9, 10), (3, 5, 7))]):
        kk = rng.standard_normal(kshape).astype(np.float32)
        place[f"p{i}/kernel"] = kk
        place[f"p{i}/shape"] = np.array(shape, np.int32)
        place[f"p{i}/reference"] = orc.ref_inplace_padded_kernel(kk, shape)
        place[f"p{i}/centered"] = orc.centered_padded_kernel(kk, shape)
    np.savez_compressed(OUT / "placement.npz", **place)
    print("wrote", OUT / "kat_small.npz", OUT / "placement.npz")


if __name__ == "__main__":
    main()
