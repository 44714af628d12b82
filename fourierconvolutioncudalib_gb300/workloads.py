"""Seeded synthetic workloads of the benchmark configurations.

Microscope-like volumes (background + Gaussian spots + Poisson noise) and
anisotropic Gaussian PSFs, generated in float64 from numpy's PCG64 and cast
to float32.  Shapes are given in array order (z, y, x).
"""
from __future__ import annotations

from typing import Dict, Iterable, List, Optional, Sequence, Tuple

import numpy as np

def spot_volume(shape_zyx: Sequence[int], n_spots: int, seed: int, background: float = 100.0,
                sigma: float = 2.0, amp: Tuple[float, float] = (200.0, 2000.0), poisson: bool = True) -> np.ndarray:
    """Background + Gaussian spots (uniform centres, uniform amplitudes), then
    Poisson noise; generated in float64 from numpy's PCG64 and cast to float32."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nz, ny, nx = shape_zyx
    vol = np.full((nz, ny, nx), background, np.float64)
    cz = rng.uniform(0, nz, n_spots)
    cy = rng.uniform(0, ny, n_spots)
    cx = rng.uniform(0, nx, n_spots)
    a = rng.uniform(amp[0], amp[1], n_spots)
    r = int(np.ceil(4 * sigma))
    off = np.arange(-r, r + 1)
    for z0, y0, x0, aa in zip(cz, cy, cx, a):
        iz = (np.floor(z0).astype(int) + off) % nz
        iy = (np.floor(y0).astype(int) + off) % ny
        ix = (np.floor(x0).astype(int) + off) % nx
        gz = np.exp(-0.5 * ((np.floor(z0) + off - z0) / sigma) ** 2)
        gy = np.exp(-0.5 * ((np.floor(y0) + off - y0) / sigma) ** 2)
        gx = np.exp(-0.5 * ((np.floor(x0) + off - x0) / sigma) ** 2)
        vol[np.ix_(iz, iy, ix)] += aa * gz[:, None, None] * gy[None, :, None] * gx[None, None, :]
    if poisson:
        vol = rng.poisson(vol).astype(np.float64)
    return vol.astype(np.float32)


def gaussian_psf(shape_zyx: Sequence[int], sigma_zyx: Sequence[float], rotation: Optional[np.ndarray] = None,
                 mix: Optional[Iterable[Tuple[float, Sequence[float]]]] = None) -> np.ndarray:
    """Anisotropic Gaussian PSF (optionally rotated, or a weighted mixture of
    Gaussians), normalised to sum 1, float32."""
    kz, ky, kx = shape_zyx
    z, y, x = np.meshgrid(np.arange(kz) - kz // 2, np.arange(ky) - ky // 2, np.arange(kx) - kx // 2, indexing="ij")
    pts = np.stack([z, y, x], -1).astype(np.float64)
    if rotation is not None:
        pts = pts @ rotation.T
    comps = list(mix) if mix is not None else [(1.0, sigma_zyx)]
    g = np.zeros((kz, ky, kx))
    for w, s in comps:
        s = np.asarray(s, np.float64)
        g += w * np.exp(-0.5 * np.sum((pts / s) ** 2, -1))
    g /= g.sum()
    return g.astype(np.float32)


def euler_zyz(a: float, b: float, c: float) -> np.ndarray:
    def rz(t):
        return np.array([[1, 0, 0], [0, np.cos(t), -np.sin(t)], [0, np.sin(t), np.cos(t)]])  # about z in (z,y,x)

    def ry(t):
        return np.array([[np.cos(t), 0, np.sin(t)], [0, 1, 0], [-np.sin(t), 0, np.cos(t)]])

    return rz(a) @ ry(b) @ rz(c)


# ------------------------------------------------------------------ benchmark configurations
# image dims are quoted (x, y, z) as in the configuration text; arrays are (z, y, x)
C4_VIEWS_XYZ = [(320, 288, 160), (256, 256, 200), (400, 352, 96), (224, 320, 128), (512, 384, 64), (288, 288, 288)]


def c1() -> Dict[str, np.ndarray]:
    """64^3 uniform[0,1) (seed 1); 7^3 isotropic Gaussian sigma 1.5, sum 1."""
    rng = np.random.Generator(np.random.PCG64(1))
    im = rng.random((64, 64, 64)).astype(np.float32)
    return dict(image=im, kernel=gaussian_psf((7, 7, 7), (1.5, 1.5, 1.5)))


def c2(nonpow2: bool = False) -> Dict[str, np.ndarray]:
    """512x512x128 (or 384x448x96) microscope stack; PSF 31x31x63 (x,y,z),
    sigma (1.5, 1.5, 4.0), sum 1."""
    shape, seed = ((96, 448, 384), 3) if nonpow2 else ((128, 512, 512), 2)
    im = spot_volume(shape, 2000, seed)
    return dict(image=im, kernel=gaussian_psf((63, 31, 31), (4.0, 1.5, 1.5)))


def c3() -> Dict[str, np.ndarray]:
    """256^3 with 5000 spots (seed 4); 21^3 Gaussian sigma (2,2,3) (x,y,z) plus
    5% uniform perturbation, renormalised; truth, target and perturbed inputs
    of the least-squares deconvolution loss."""
    rng = np.random.Generator(np.random.PCG64(4))
    x_true = spot_volume((256, 256, 256), 5000, 4)
    k = gaussian_psf((21, 21, 21), (3.0, 2.0, 2.0)).astype(np.float64)
    k = k + 0.05 * k.max() * rng.random(k.shape)
    k_true = (k / k.sum()).astype(np.float32)
    x = (x_true * (1 + 0.1 * rng.standard_normal(x_true.shape))).astype(np.float32)
    kp = (k_true * (1 + 0.1 * rng.standard_normal(k_true.shape))).astype(np.float32)
    return dict(x_true=x_true, k_true=k_true, image=x, kernel=kp, noise_seed=np.array(4))


def c4() -> List[Dict[str, np.ndarray]]:
    """6 views of uneven sizes, each with its own rotated anisotropic PSF."""
    views = []
    for (nx, ny, nz), ss in zip(C4_VIEWS_XYZ, np.random.SeedSequence(5).spawn(6)):
        rng = np.random.Generator(np.random.PCG64(ss))
        n_spots = max(100, (nx * ny * nz) // 16384)
        im = spot_volume((nz, ny, nx), n_spots, int(rng.integers(1 << 31)))
        edge = int(rng.choice(np.arange(21, 42, 2)))
        sxy = rng.uniform(1.2, 2.0)
        sz = rng.uniform(3.0, 5.0)
        rot = euler_zyz(*rng.uniform(0, 2 * np.pi, 3))
        views.append(dict(image=im, kernel=gaussian_psf((edge, edge, edge), (sz, sxy, sxy), rotation=rot)))
    return views


def c5(plane: int = 1024) -> Dict[str, np.ndarray]:
    """1024x1024x256 with 20000 spots (seed 6); 63^3 mixture of 3 anisotropic
    Gaussians with weights 0.7 / 0.2 / 0.1, sum 1.  plane=512: the 512x512x256
    case with 5000 spots and the same PSF (the same 256-long z pass on a
    quarter of the columns, for profiler captures)."""
    im = spot_volume((256, plane, plane), 20000 * (plane * plane) // (1024 * 1024), 6)
    mix = [(0.7, (3.0, 1.5, 1.5)), (0.2, (6.0, 3.0, 3.0)), (0.1, (10.0, 6.0, 6.0))]
    return dict(image=im, kernel=gaussian_psf((63, 63, 63), (1, 1, 1), mix=mix))
